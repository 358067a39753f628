"""Generate golden vectors for the per-pair math from the reference itself.

Runs only where the reference sources exist: ``make -C oracle`` compiles the
reference's radial.cpp, cutoffs.cpp and y_grad.cpp (unmodified) into
oracle/_ref/libflare_ref_math.so; this script evaluates them at seeded random
points and writes tests/golden/per_pair.npz.  The test-suite then pins the
oracle's restatement (and, through it, the CUDA kernels) against these values.

Usage:  make -C oracle && python tests/golden/make_golden.py
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "..", "oracle", "_ref", "libflare_ref_math.so")


def main():
    lib = ctypes.CDLL(LIB)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.ref_get_Y.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int] + [dp] * 4
    lib.ref_calculate_radial.argtypes = (
        [ctypes.c_char_p, ctypes.c_char_p] + [ctypes.c_double] * 5 +
        [ctypes.c_int, dp, ctypes.c_int, dp, ctypes.c_int] + [dp] * 4)
    rng = np.random.Generator(np.random.PCG64(777))

    # Spherical harmonics, l = 10 (reference maximum), 64 directions and radii.
    L = 10
    nh = (L + 1) ** 2
    pts = rng.normal(size=(64, 3)) * rng.uniform(0.5, 5.0, size=(64, 1))
    pts[0] = [0.0, 0.0, 2.0]          # on the z axis
    pts[1] = [1.5, 0.0, 0.0]          # on the x axis
    Y = np.zeros((64, 4, nh))
    for i, (x, y, z) in enumerate(pts):
        bufs = [np.zeros(nh) for _ in range(4)]
        lib.ref_get_Y(x, y, z, L, *[b.ctypes.data_as(dp) for b in bufs])
        Y[i] = np.stack(bufs)

    # Radial x cutoff for the Chebyshev basis with every cutoff function.
    N = 10
    rcut = 5.0
    rpts = rng.normal(size=(48, 3))
    rpts /= np.linalg.norm(rpts, axis=1, keepdims=True)
    rr = rng.uniform(0.3, 5.2, size=48)           # some beyond the cutoff
    rpts *= rr[:, None]
    cut_cases = [("quadratic", []), ("hard", []), ("cosine", []),
                 ("polynomial", [6.0]), ("power", [2.0])]
    R = {}
    for name, ch in cut_cases:
        out = np.zeros((48, 4, N))
        cha = np.asarray(ch if ch else [0.0], dtype=np.float64)
        rh = np.asarray([0.0, rcut], dtype=np.float64)
        for i in range(48):
            x, y, z = rpts[i]
            bufs = [np.zeros(N) for _ in range(4)]
            lib.ref_calculate_radial(b"chebyshev", name.encode(), x, y, z,
                                     rr[i], rcut, N, rh.ctypes.data_as(dp), 2,
                                     cha.ctypes.data_as(dp), len(ch),
                                     *[b.ctypes.data_as(dp) for b in bufs])
            out[i] = np.stack(bufs)
        R[name] = out

    # Every radial basis (radial.cpp:6-336) with the quadratic cutoff, the
    # hyperparameters as the B2 descriptor passes them: radial_hyps[1]
    # replaced by the pair cutoff (b2.cpp:352).
    basis_cases = [("chebyshev", [0.5, rcut]),
                   ("weighted_chebyshev", [0.5, rcut, 3.0]),
                   ("equispaced_gaussians", [0.5, rcut, 0.8]),
                   ("weighted_positive_chebyshev", [0.5, rcut, 3.0]),
                   ("positive_chebyshev", [0.5, rcut]),
                   ("bessel", [0.0, rcut]),
                   ("fourier_quarter", [0.5, rcut]),
                   ("fourier_half", [0.5, rcut]),
                   ("fourier", [0.5, rcut, 0.75])]
    B = {}
    zero = np.zeros(1)
    for name, rh in basis_cases:
        out = np.zeros((48, 4, N))
        rha = np.asarray(rh, dtype=np.float64)
        for i in range(48):
            x, y, z = rpts[i]
            bufs = [np.zeros(N) for _ in range(4)]
            lib.ref_calculate_radial(name.encode(), b"quadratic", x, y, z,
                                     rr[i], rcut, N, rha.ctypes.data_as(dp),
                                     len(rh), zero.ctypes.data_as(dp), 0,
                                     *[b.ctypes.data_as(dp) for b in bufs])
            out[i] = np.stack(bufs)
        B[name] = out
    np.savez_compressed(
        os.path.join(HERE, "per_pair.npz"), ylm_points=pts, ylm_lmax=L,
        ylm=Y, radial_points=rpts, radial_r=rr, radial_rcut=rcut,
        radial_nmax=N, **{f"radial_{k}": v for k, v in R.items()},
        **{f"cutoff_hyps_{k}": np.asarray(ch) for k, ch in cut_cases},
        **{f"basis_{k}": v for k, v in B.items()},
        **{f"basis_hyps_{k}": np.asarray(rh) for k, rh in basis_cases})
    print("wrote per_pair.npz")


if __name__ == "__main__":
    main()
