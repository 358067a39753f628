"""Mapped models: the coefficient files a LAMMPS run of the reference loads,
written from a solved sparse GP, and GPU evaluation from those files.

Writers (the reference's SparseGP methods, src/flare_pp/bffs/sparse_gp.cpp):
  * ``write_mapping_coefficients`` — lmp.flare, the pair style's beta
    (:1199-1264; coefficients normalized_dot_product.cpp:653-767);
  * ``write_varmap_coefficients`` — the power-1 variance map (:1266-1335;
    normalized_dot_product.cpp:769-830);
  * ``write_L_inverse`` / ``write_sparse_descriptors`` — the files of
    compute flare/std/atom (:1337-1466).
The text layout (headers, number format, line breaks) follows the writers
line by line, so the files are interchangeable with the reference's.

Evaluators (GPU):
  * ``MappedPotential`` — energies, forces and stresses from an lmp.flare
    file with the pair style's arithmetic (pair_flare.cpp:68-175,
    lammps_descriptor.cpp:250-326), optionally the mapped local std of a
    varmap file (compute_flare_std_atom.cpp:179-193);
  * ``LocalStdFromFiles`` — the local std from the L_inverse and sparse
    descriptor files (compute_flare_std_atom.cpp:194-226).
The mapping coefficients themselves are computed on the GPU in FP64
(``fgb_model_mapping``) and the varmap QR by cuSOLVER (``fgb_qr_thin_q``).
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr, stream_ptr
from .core import B2, _Model, _device, pack_structures

EMPTY_THRESH = 1e-8


# ---------------------------------------------------------------- format
def _num(v):
    """A double as the reference's streams print it (std::scientific,
    precision 16)."""
    return f"{float(v):.16e}"


def _header(contributor):
    return f"DATE: {time.ctime()} CONTRIBUTOR: {contributor}\n"


def _b2_block(calc, coeff_size):
    """B2::write_to_file (b2.cpp:52-74)."""
    S, N, L = calc.descriptor_settings
    cut = "".join(f"{c:.2f} " for c in np.asarray(calc.cutoffs).reshape(-1))
    return (f"{calc.radial_basis}\n{S} {N} {L} {coeff_size}\n"
            f"{calc.cutoff_function}\n{cut}\n")


def _kernel_info(kernel):
    """NormalizedDotProduct::write_info (normalized_dot_product.cpp:832-835)."""
    return f"{float(kernel.power):.0f} NormalizedDotProduct\n"


def _padded_rows(rows, reset_count):
    """Rows of coefficients, 5 per line, two spaces before positive values
    and one otherwise, a line break before each new row; the mapping writer
    keeps its column count across rows (sparse_gp.cpp:1236-1259), the
    varmap writer resets it (:1309-1331)."""
    out = []
    count = 0
    for row in rows:
        if count != 0:
            out.append("\n")
            if reset_count:
                count = 0
        for v in row:
            out.append("  " if v > 0 else " ")
            out.append(_num(v))
            count += 1
            if count == 5:
                count = 0
                out.append("\n")
    return "".join(out)


# ------------------------------------------------------------- writers
def mapping_coefficients(sgp, kernel_index=0):
    """Per-species mapping coefficients in the reference's layout: power 2,
    the upper triangle of sigma^2 sum alpha s^ s^T row by row with the
    off-diagonal entries doubled; power 1, sigma^2 sum alpha s^."""
    if kernel_index != 0 or sgp.n_kernels != 1:
        raise NotImplementedError("mapping of one kernel (index 0)")
    k = sgp.kernels[0]
    power = float(k.power)
    if power not in (1.0, 2.0):
        raise ValueError("Mapping coefficients of the normalized dot product "
                         "kernel are implemented for power 1 and 2 only.")
    m = sgp._device_model()
    calc = m.b2
    S = calc.descriptor_settings[0]
    p = calc.n_descriptors
    per = p * p if power == 2.0 else p
    beta = np.zeros(S * per)
    check(lib().fgb_model_mapping(m.h, ptr(beta), stream_ptr()),
          "write_mapping_coefficients")
    if power == 1.0:
        return beta.reshape(S, p)
    full = beta.reshape(S, p, p)
    iu = np.triu_indices(p)
    factor = np.where(iu[0] == iu[1], 1.0, 2.0)
    return np.stack([full[s][iu] * factor for s in range(S)])


def fold_guard(sgp):
    """The mixed path's force-precision guard: (largest |sigma^2 sum alpha
    s^ s^T| entry, True when the force stage runs at FP64 level).  The
    FP32-level force stage errs by about 2.5e-7 eV/A per unit of that
    entry, so models whose entry exceeds 200 get FP64-level forces."""
    m = sgp._device_model()
    fmax = ctypes.c_double(0.0)
    f64 = ctypes.c_int(0)
    check(lib().fgb_model_fold_guard(m.h, ctypes.byref(fmax),
                                     ctypes.byref(f64), stream_ptr()),
          "fold_guard")
    return fmax.value, bool(f64.value)


def write_mapping_coefficients(sgp, file_name, contributor, kernel_index=0):
    """SparseGP::write_mapping_coefficients (sparse_gp.cpp:1199-1264)."""
    coeffs = mapping_coefficients(sgp, kernel_index)
    calc = sgp._device_model().b2
    text = (_header(contributor) + _kernel_info(sgp.kernels[kernel_index]) +
            _b2_block(calc, coeffs.shape[1]) +
            _padded_rows(coeffs, reset_count=False))
    with open(file_name, "w") as f:
        f.write(text)
    return coeffs


def varmap_coefficients(sgp, kernel_index=0):
    """NormalizedDotProduct::compute_varmap_coefficients
    (normalized_dot_product.cpp:769-830): per species the leading p x p
    block of the thin Q of [S^T; sqrt(jitter)/sigma I], zero past the
    species' sparse count.  Depends only on the sparse set, sigma and the
    jitter (the reference builds a power-1 copy of the model for it)."""
    if kernel_index != 0 or sgp.n_kernels != 1:
        raise NotImplementedError("variance map of one kernel (index 0)")
    sig = float(sgp.kernels[0].sigma)
    cd = sgp.sparse_descriptors[0]
    p = cd.n_descriptors
    jr = np.sqrt(sgp.Kuu_jitter)
    dev = _device()
    out = np.zeros((cd.n_types, p * p))
    for s in range(cd.n_types):
        n = int(cd.n_clusters_by_type[s])
        if n == 0:
            continue
        pi = np.array(cd.descriptors[s], np.float64, copy=True)
        norms = np.asarray(cd.descriptor_norms[s], np.float64)
        ok = norms >= EMPTY_THRESH
        pi[ok] = pi[ok] / norms[ok, None]
        A = np.zeros((p + n, n))
        A[:p] = pi.T
        A[p:] = jr * np.eye(n) / sig
        a = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)   # column-major
        q = torch.empty_like(a)
        check(lib().fgb_qr_thin_q(p + n, n, ptr(a), ptr(q), stream_ptr()),
              "write_varmap_coefficients")
        Q = q.cpu().numpy().T                                       # (p + n) x n
        block = np.zeros((p, p))
        w = min(n, p)
        block[:, :w] = Q[:p, :w]
        out[s] = block.reshape(-1)
    return out


def write_varmap_coefficients(sgp, file_name, contributor, kernel_index=0):
    """SparseGP::write_varmap_coefficients (sparse_gp.cpp:1266-1335)."""
    coeffs = varmap_coefficients(sgp, kernel_index)
    calc = sgp._device_model().b2
    hyps = sgp.hyperparameters
    text = (_header(contributor) + f"{len(hyps)}\n" +
            "".join(_num(h) + " " for h in hyps) +
            "\nNormalizedDotProduct\n" + _b2_block(calc, coeffs.shape[1]) +
            _padded_rows(coeffs, reset_count=True))
    with open(file_name, "w") as f:
        f.write(text)
    sgp.varmap_coeffs = coeffs
    return coeffs


def write_L_inverse(sgp, file_name, contributor):
    """SparseGP::write_L_inverse (sparse_gp.cpp:1337-1391): per kernel the
    lower triangle of its diagonal block of L_inv, 5 values per line."""
    calc = sgp._device_model().b2
    hyps = sgp.hyperparameters
    parts = ["L_inverse_block file " + _header(contributor),
             _kernel_info(sgp.kernels[0]), f"{len(hyps)}\n",
             "".join(_num(h) + " " for h in hyps), "\n"]
    start = 0
    for i in range(sgp.n_kernels):
        parts.append(_b2_block(calc, sgp.n_kernels))
        n = int(sgp.sparse_descriptors[i].n_clusters)
        blk = np.asarray(sgp.L_inv)[start:start + n, start:start + n]
        start += n
        parts.append(f"{n}\n")
        count = 1
        for j in range(n):
            for k in range(j + 1):
                parts.append(_num(blk[j, k]) + " ")
                if count % 5 == 0:
                    parts.append("\n")
                count += 1
        if count % 5 != 0:
            parts.append("\n")
    with open(file_name, "w") as f:
        f.write("".join(parts))


def write_sparse_descriptors(sgp, file_name, contributor):
    """SparseGP::write_sparse_descriptors (sparse_gp.cpp:1393-1466): the
    sparse descriptors per kernel and species, normalised for the
    NormalizedDotProduct kernel, zeros for empty environments."""
    parts = ["sparse_descriptors file " + _header(contributor),
             f"{sgp.n_kernels}\n"]
    for i in range(sgp.n_kernels):
        cd = sgp.sparse_descriptors[i]
        parts.append(f"{i} {int(cd.n_clusters)} {int(cd.n_types)}\n")
        count = 1
        for s in range(cd.n_types):
            n = int(cd.n_clusters_by_type[s])
            parts.append(f"{n}\n")
            d = np.asarray(cd.descriptors[s], np.float64).reshape(n, -1) \
                if n else np.zeros((0, cd.n_descriptors))
            norms = np.asarray(cd.descriptor_norms[s], np.float64)
            for j in range(n):
                for k in range(cd.n_descriptors):
                    if norms[j] < EMPTY_THRESH:
                        v = 0.0
                    else:
                        v = d[j, k] / norms[j]
                    parts.append(_num(v) + " ")
                    if count % 5 == 0:
                        parts.append("\n")
                    count += 1
            if count % 5 != 1:
                parts.append("\n")
    with open(file_name, "w") as f:
        f.write("".join(parts))


# ------------------------------------------------------------- readers
class _Tokens:
    """Whitespace-separated values after a fixed number of header lines
    (the readers' grab(), pair_flare.cpp:432-450)."""

    def __init__(self, lines):
        self.lines = lines
        self.i = 0
        self.buf = []

    def line(self):
        s = self.lines[self.i]
        self.i += 1
        return s

    def take(self, n):
        while len(self.buf) < n:
            self.buf.extend(self.lines[self.i].split())
            self.i += 1
        out, self.buf = self.buf[:n], self.buf[n:]
        return np.array([float(x) for x in out])


def read_mapping_file(file_name):
    """PairFLARE::read_file (pair_flare.cpp:262-425)."""
    with open(file_name) as f:
        t = _Tokens(f.read().splitlines())
    t.line()                                        # date and contributor
    w = t.line().split()
    power, kernel = int(float(w[0])), w[1]
    radial = t.line().split()[0]
    S, N, L, beta_size = (int(x) for x in t.line().split()[:4])
    cutoff_function = t.line().split()[0]
    cutoffs = t.take(S * S).reshape(S, S)
    nr = N * S
    nd = nr * (nr + 1) // 2 * (L + 1)
    expect = nd if power == 1 else nd * (nd + 1) // 2
    if power not in (1, 2):
        raise ValueError("Power should be 1 or 2.")
    if beta_size != expect:
        raise ValueError("Beta size doesn't match the number of descriptors.")
    if kernel not in ("NormalizedDotProduct", "DotProduct"):
        raise ValueError("Kernel string not recognized, expected <power> "
                         "<kernel string>")
    beta = t.take(S * beta_size).reshape(S, beta_size)
    if power == 2:
        mats = np.zeros((S, nd, nd))
        iu = np.triu_indices(nd)
        for s in range(S):
            vals = beta[s] / np.where(iu[0] == iu[1], 1.0, 2.0)
            mats[s][iu] = vals
            mats[s][(iu[1], iu[0])] = vals
        beta = mats
    return {"power": power, "kernel": kernel, "radial_basis": radial,
            "descriptor_settings": [S, N, L], "cutoff_function": cutoff_function,
            "cutoffs": cutoffs, "beta": beta, "n_descriptors": nd}


def read_varmap_file(file_name):
    """The variance-map file of compute flare/std/atom: hyperparameters and
    per-species Q blocks (n_d x n_d)."""
    with open(file_name) as f:
        t = _Tokens(f.read().splitlines())
    t.line()
    n_hyps = int(t.line().split()[0])
    hyps = t.take(n_hyps)
    kernel = t.line().split()[0]
    radial = t.line().split()[0]
    S, N, L, size = (int(x) for x in t.line().split()[:4])
    cutoff_function = t.line().split()[0]
    cutoffs = t.take(S * S).reshape(S, S)
    nd = int(round(np.sqrt(size)))
    Q = t.take(S * size).reshape(S, nd, nd)
    return {"hyperparameters": hyps, "kernel": kernel, "radial_basis": radial,
            "descriptor_settings": [S, N, L], "cutoff_function": cutoff_function,
            "cutoffs": cutoffs, "Q": Q}


def read_L_inverse(file_name):
    """ComputeFlareStdAtom::read_L_inverse (compute_flare_std_atom.cpp:
    484-610): power, kernel, hyperparameters, descriptor settings and the
    lower triangle of L_inv."""
    with open(file_name) as f:
        t = _Tokens(f.read().splitlines())
    t.line()
    w = t.line().split()
    power, kernel = int(float(w[0])), w[1]
    n_hyps = int(t.line().split()[0])
    hyps = t.take(n_hyps)
    radial = t.line().split()[0]
    S, N, L, n_kernels = (int(x) for x in t.line().split()[:4])
    cutoff_function = t.line().split()[0]
    cutoffs = t.take(S * S).reshape(S, S)
    n = int(t.take(1)[0])
    vals = t.take(n * (n + 1) // 2)
    Linv = np.zeros((n, n))
    Linv[np.tril_indices(n)] = vals
    return {"power": power, "kernel": kernel, "hyperparameters": hyps,
            "radial_basis": radial, "descriptor_settings": [S, N, L],
            "cutoff_function": cutoff_function, "cutoffs": cutoffs,
            "L_inv": Linv}


def read_sparse_descriptors(file_name, n_descriptors):
    """ComputeFlareStdAtom::read_sparse_descriptors
    (compute_flare_std_atom.cpp:612-694): per species the (normalised)
    sparse descriptors of kernel 0, n_clusters_by_type x n_descriptors."""
    with open(file_name) as f:
        t = _Tokens(f.read().splitlines())
    t.line()
    int(t.take(1)[0])                               # number of kernels
    _, n_clusters, n_types = (int(x) for x in t.take(3))
    out = []
    for s in range(n_types):
        n = int(t.take(1)[0])
        out.append(t.take(n * n_descriptors).reshape(n, n_descriptors))
    return out


# ----------------------------------------------------------- evaluators
def _b2_from(info):
    S, N, L = info["descriptor_settings"]
    cut = np.asarray(info["cutoffs"], np.float64)
    return B2(info["radial_basis"], info["cutoff_function"],
              [0.0, float(cut.max())], [], [S, N, L], cut)


def _run(handle_fn, structures):
    offsets, cells, pos, sp = pack_structures(structures)
    dev = _device()
    N, S = int(offsets[-1]), len(structures)
    d_pos = torch.from_numpy(pos).to(dev)
    d_sp = torch.from_numpy(sp).to(dev)
    out = {"energy": torch.zeros(S, dtype=torch.float64, device=dev),
           "forces": torch.zeros((max(N, 1), 3), dtype=torch.float64, device=dev),
           "stress": torch.zeros((S, 6), dtype=torch.float64, device=dev),
           "atom_energies": torch.zeros(max(N, 1), dtype=torch.float64, device=dev),
           "local_var": torch.zeros(max(N, 1), dtype=torch.float64, device=dev)}
    handle_fn(S, offsets, cells, d_pos, d_sp, out)
    torch.cuda.current_stream().synchronize()
    return {k: (v.cpu().numpy()[:N] if k in ("forces", "atom_energies",
                                             "local_var") else v.cpu().numpy())
            for k, v in out.items()}, offsets


class MappedPotential:
    """Energies, forces and stresses (and, with a varmap file, the mapped
    local std) from an lmp.flare coefficient file, on the GPU."""

    def __init__(self, coefficient_file, varmap_file=None):
        info = read_mapping_file(coefficient_file)
        self.info = info
        self.power = info["power"]
        self.normalized = info["kernel"] == "NormalizedDotProduct"
        self.b2 = _b2_from(info)
        self.cutoff = float(np.max(info["cutoffs"]))
        beta = np.ascontiguousarray(info["beta"], np.float64)
        Q = None
        if varmap_file is not None:
            vm = read_varmap_file(varmap_file)
            if vm["descriptor_settings"] != info["descriptor_settings"]:
                raise ValueError("variance map and coefficients disagree")
            Q = np.ascontiguousarray(vm["Q"], np.float64)
            self.sigma = float(vm["hyperparameters"][0])
        h = ctypes.c_void_p()
        check(lib().fgb_mapped_create(ctypes.byref(h), self.b2.handle,
                                      self.power, int(self.normalized),
                                      ptr(beta), ptr(Q)), "MappedPotential")
        self.h = h
        self.has_std = Q is not None

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.fgb_mapped_destroy(self.h)
            self.h = None

    def predict(self, structures, std=False, precision="fp64"):
        """dict: energy [S], forces [N, 3], stress [S, 6] (flare order),
        atom_energies [N]; with ``std`` the mapped local std [N].
        ``precision`` "mixed": descriptor in double-float and adjoint in
        FP32 (the prediction pipeline's mixed mode)."""
        prec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}[precision]
        if std and not self.has_std:
            raise ValueError("no variance map loaded")
        want = 0x7 | (0x8 if std else 0)

        def go(S, offsets, cells, d_pos, d_sp, out):
            check(lib().fgb_mapped_predict(
                self.h, S, ptr(offsets), ptr(cells), ptr(d_pos), ptr(d_sp),
                self.cutoff, want, ptr(out["energy"]), ptr(out["forces"]),
                ptr(out["stress"]), ptr(out["atom_energies"]),
                ptr(out["local_var"]), prec, stream_ptr()), "MappedPotential")

        r, _ = _run(go, structures)
        if std:
            v = r["local_var"]
            r["std"] = np.sign(v) * np.sqrt(np.abs(v))
        del r["local_var"]
        return r


class LocalStdFromFiles:
    """The local std of compute flare/std/atom (non-mapped form) from the
    L_inverse and sparse-descriptor files: std_i = sign(v) sqrt|v| with
    v = 1 - sigma^2 |L_inv k_i|^2, k_i = (s^ . d^_i)^power, i.e. this
    library's local variance divided by sigma^2."""

    def __init__(self, L_inverse_file, sparse_descriptors_file):
        li = read_L_inverse(L_inverse_file)
        self.info = li
        self.b2 = _b2_from(li)
        self.cutoff = float(np.max(li["cutoffs"]))
        self.sigma = float(li["hyperparameters"][0])
        nd = self.b2.n_descriptors
        blocks = read_sparse_descriptors(sparse_descriptors_file, nd)
        counts = np.array([b.shape[0] for b in blocks], np.int32)
        desc = np.concatenate(blocks) if blocks else np.zeros((0, nd))
        M = desc.shape[0]
        if li["L_inv"].shape != (M, M):
            raise ValueError("L_inverse and sparse descriptors disagree")
        self._model = _Model(self.b2, self.sigma, li["power"])
        self._model.set(counts, desc, np.zeros(M), li["L_inv"])

    def std(self, structures, precision="fp64"):
        offsets, cells, pos, sp = pack_structures(structures)
        dev = _device()
        N, S = int(offsets[-1]), len(structures)
        d_pos = torch.from_numpy(pos).to(dev)
        d_sp = torch.from_numpy(sp).to(dev)
        v = torch.zeros(max(N, 1), dtype=torch.float64, device=dev)
        prec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}[precision]
        check(lib().fgb_predict(self._model.h, S, ptr(offsets), ptr(cells),
                                ptr(d_pos), ptr(d_sp), self.cutoff,
                                _lib.FGB_WANT_LOCAL_VAR, prec, None, None,
                                None, ptr(v), stream_ptr()), "LocalStdFromFiles")
        torch.cuda.current_stream().synchronize()
        var = v.cpu().numpy()[:N] / self.sigma ** 2
        return np.sign(var) * np.sqrt(np.abs(var))
