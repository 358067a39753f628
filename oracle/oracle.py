"""FP64 CPU oracle for FLARE's sparse-GP prediction path.

TEST INFRASTRUCTURE ONLY: the parity checker for the test-suite and the timed
CPU baseline of bench.py.  Product code never imports this module.

The heavy loops live in ``flare_oracle.cpp`` (built to ``liboracle.so`` next to
this file); GEMMs and dense linear algebra use numpy/scipy LAPACK, standing in
for Eigen 3.3.7 (GEMM, LLT, HouseholderQR, triangular solve), which the
reference fetches at configure time and which is absent here.

Restated reference code (paths inside mir-group/flare):
  Structure ............... src/flare_pp/structure.cpp:7-118
  B2.compute_struc ........ src/flare_pp/descriptors/b2.cpp:76-179 (regroup)
  ClusterDescriptor ....... src/flare_pp/descriptors/descriptor.cpp:60-176
  envs_envs / envs_struc .. src/flare_pp/kernels/normalized_dot_product.cpp:28-214
  SparseGP ................ src/flare_pp/bffs/sparse_gp.cpp:14-757
  SGP_Calculator post ..... flare/bffs/sgp/calculator.py:57-122,188-206
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import scipy.linalg as sla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

RADIAL_IDS = {"chebyshev": 0, "weighted_chebyshev": 1,
              "equispaced_gaussians": 2, "weighted_positive_chebyshev": 3,
              "positive_chebyshev": 4, "bessel": 5, "fourier_quarter": 6,
              "fourier_half": 7, "fourier": 8}
CUTOFF_IDS = {"quadratic": 0, "hard": 1, "cosine": 2, "polynomial": 3, "power": 4}


def build(force=False):
    """Compile liboracle.so from flare_oracle.cpp (g++, OpenMP, no FMA)."""
    src = os.path.join(_HERE, "flare_oracle.cpp")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-std=c++17", src, "-o", _LIB_PATH]
    subprocess.check_call(cmd)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_cell_setup.argtypes = [dp, dp]
        L.orc_wrap_positions.argtypes = [dp, dp, ctypes.c_int, dp]
        L.orc_neighbors.argtypes = [dp, dp, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int, ip, dp, ip, ip]
        L.orc_neighbors.restype = ctypes.c_longlong
        L.orc_radial.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_double, ctypes.c_double, dp,
                                 ctypes.c_int, dp, dp, dp, dp]
        L.orc_ylm.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int, dp, dp, dp,
                                                      dp]
        L.orc_b2.argtypes = [ctypes.c_int, ip, ip, dp, ip, ctypes.c_int,
                             ctypes.c_int, ctypes.c_double, ctypes.c_double,
                             dp, ctypes.c_int,
                             ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip,
                             ip, dp, dp, dp, dp, dp, dp]
        L.orc_b2.restype = ctypes.c_longlong
        L.orc_envs_struc_block.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
            dp, dp, ip, ip, ip, ip, dp, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, dp]
        L.orc_self_kernel_block.argtypes = [
            ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, ip, ip, ip, ip, dp,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        L.orc_self_kernel_block.restype = ctypes.c_int
        L.orc_struc_struc_block.argtypes = (
            [ctypes.c_int] * 4 + [dp] * 8 + [ip, ip, ip, ip, dp] * 2 +
            [ctypes.c_double] * 4 + [dp])
        L.orc_struc_struc_block.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None \
        else ctypes.POINTER(ctypes.c_double)()


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None \
        else ctypes.POINTER(ctypes.c_int)()


# ---------------------------------------------------------------- per pair
def ylm(x, y, z, lmax):
    """Real Y_lm and gradients at one point (y_grad.cpp:667 convention)."""
    nh = (lmax + 1) ** 2
    out = [np.zeros(nh) for _ in range(4)]
    lib().orc_ylm(x, y, z, lmax, *[_dp(o) for o in out])
    return out


def radial(radial_basis, cutoff_function, x, y, z, r, rcut, nmax, r1=0.0,
           cutoff_hyps=(), h2=0.0):
    ch = np.asarray(cutoff_hyps, dtype=np.float64).reshape(-1)
    if ch.size == 0:
        ch = np.zeros(1)
    out = [np.zeros(nmax) for _ in range(4)]
    lib().orc_radial(RADIAL_IDS[radial_basis], CUTOFF_IDS[cutoff_function], x,
                     y, z, r, rcut, nmax, r1, h2, _dp(ch), len(cutoff_hyps),
                     *[_dp(o) for o in out])
    return out


# --------------------------------------------------------------- settings
class B2Settings:
    """Mirror of the B2 constructor arguments (b2.cpp:13-50)."""

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings, cutoffs=None):
        self.radial_basis = radial_basis
        self.cutoff_function = cutoff_function
        self.radial_hyps = list(map(float, radial_hyps))
        self.cutoff_hyps = list(map(float, cutoff_hyps))
        self.descriptor_settings = list(map(int, descriptor_settings))
        S = self.descriptor_settings[0]
        if cutoffs is None:
            cutoffs = np.full((S, S), self.radial_hyps[1])
        self.cutoffs = np.ascontiguousarray(np.asarray(cutoffs, np.float64))

    @property
    def n_descriptors(self):
        S, N, L = self.descriptor_settings
        nr = S * N
        return nr * (nr + 1) // 2 * (L + 1)


class DescriptorValues:
    """Species-regrouped descriptor values (b2.cpp:104-176)."""


class ClusterDescriptor:
    """descriptor.cpp:60-176: per-species descriptor rows + norms."""

    def __init__(self, n_types, n_descriptors):
        self.n_types = n_types
        self.n_descriptors = n_descriptors
        self.descriptors = [np.zeros((0, n_descriptors)) for _ in range(n_types)]
        self.descriptor_norms = [np.zeros(0) for _ in range(n_types)]
        self.n_clusters_by_type = [0] * n_types
        self.cumulative_type_count = [0] * n_types
        self.n_clusters = 0

    @staticmethod
    def from_values(dv, clusters_by_type=None):
        c = ClusterDescriptor(dv.n_types, dv.n_descriptors)
        if clusters_by_type is None:
            clusters_by_type = [list(range(dv.n_clusters_by_type[s]))
                                for s in range(dv.n_types)]
        c.add_clusters_by_type(dv, clusters_by_type)
        return c

    def add_clusters_by_type(self, dv, clusters):
        for s in range(self.n_types):
            idx = np.asarray(clusters[s], dtype=np.int64)
            self.descriptors[s] = np.vstack(
                [self.descriptors[s], dv.descriptors[s][idx]]) if idx.size else \
                self.descriptors[s]
            self.descriptor_norms[s] = np.concatenate(
                [self.descriptor_norms[s], dv.descriptor_norms[s][idx]])
        for s in range(self.n_types):
            self.n_clusters_by_type[s] += len(clusters[s])
            self.n_clusters += len(clusters[s])
            if s > 0:
                self.cumulative_type_count[s] = (
                    self.cumulative_type_count[s - 1] +
                    self.n_clusters_by_type[s - 1])


# -------------------------------------------------------------- structure
class Structure:
    """Restatement of Structure (structure.cpp:7-118) + B2 descriptors."""

    def __init__(self, cell, species, positions, cutoff, descriptor_calculators,
                 compute_dervs=True):
        L = lib()
        self.cell = np.ascontiguousarray(np.asarray(cell, np.float64))
        self.species = [int(s) for s in species]
        self.positions = np.ascontiguousarray(np.asarray(positions, np.float64))
        self.noa = len(self.species)
        self.cutoff = float(cutoff)
        setup = np.zeros(38)
        L.orc_cell_setup(_dp(self.cell), _dp(setup))
        self.volume = setup[36]
        self.single_sweep_cutoff = setup[37]
        self.sweep = int(math.ceil(self.cutoff / self.single_sweep_cutoff))
        n = self.noa
        self.wrapped_positions = np.zeros((n, 3))
        L.orc_wrap_positions(_dp(self.cell), _dp(self.positions), n,
                             _dp(self.wrapped_positions))
        self.neighbor_count = np.zeros(n, dtype=np.int32)
        P = L.orc_neighbors(_dp(self.cell), _dp(self.wrapped_positions), n,
                            self.cutoff, self.sweep, _ip(self.neighbor_count),
                            None, None, None)
        self.relative_positions = np.zeros((P, 4))
        self.structure_indices = np.zeros(P, dtype=np.int32)
        self.shifts = np.zeros((P, 3), dtype=np.int32)
        L.orc_neighbors(_dp(self.cell), _dp(self.wrapped_positions), n,
                        self.cutoff, self.sweep, _ip(self.neighbor_count),
                        _dp(self.relative_positions),
                        _ip(self.structure_indices), _ip(self.shifts))
        self.n_neighbors = int(P)
        self.cumulative_neighbor_count = np.zeros(n + 1, dtype=np.int64)
        self.cumulative_neighbor_count[1:] = np.cumsum(self.neighbor_count)
        sp = np.asarray(self.species, dtype=np.int32)
        self.neighbor_species = sp[self.structure_indices] if P else \
            np.zeros(0, np.int32)
        self.descriptor_calculators = descriptor_calculators
        self.descriptors = [self._compute_b2(d, compute_dervs)
                            for d in descriptor_calculators]
        self.energy = np.zeros(0)
        self.forces = np.zeros(0)
        self.stresses = np.zeros(0)

    def _compute_b2(self, b2, compute_dervs):
        L = lib()
        n = self.noa
        S, N, Lm = b2.descriptor_settings
        nh = (Lm + 1) ** 2
        nA = S * N * nh
        nd = b2.n_descriptors
        sp = np.asarray(self.species, dtype=np.int32)
        ch = np.asarray(b2.cutoff_hyps, dtype=np.float64)
        if ch.size == 0:
            ch = np.zeros(1)
        b2_count = np.zeros(n, dtype=np.int32)
        args_pre = (n, _ip(sp), _ip(self.neighbor_count),
                    _dp(self.relative_positions), _ip(self.structure_indices),
                    RADIAL_IDS[b2.radial_basis], CUTOFF_IDS[b2.cutoff_function],
                    b2.radial_hyps[0],
                    b2.radial_hyps[2] if len(b2.radial_hyps) > 2 else 0.0,
                    _dp(ch), len(b2.cutoff_hyps), S, N, Lm,
                    _dp(b2.cutoffs))
        Pb = L.orc_b2(*args_pre, _ip(b2_count), None, None, None, None, None,
                      None, None)
        b2_idx = np.zeros(Pb, dtype=np.int32)
        coords = np.zeros((Pb, 3))
        single = np.zeros((n, nA))
        B2 = np.zeros((n, nd))
        norms = np.zeros(n)
        dervs = np.zeros((3 * Pb, nd)) if compute_dervs else None
        fdots = np.zeros(3 * Pb) if compute_dervs else None
        L.orc_b2(*args_pre, _ip(b2_count), _ip(b2_idx), _dp(coords),
                 _dp(single), _dp(B2), _dp(norms), _dp(dervs), _dp(fdots))
        cum = np.zeros(n + 1, dtype=np.int64)
        cum[1:] = np.cumsum(b2_count)

        # Species regroup, b2.cpp:104-176.
        dv = DescriptorValues()
        dv.n_descriptors = nd
        dv.n_types = S
        dv.n_atoms = n
        dv.volume = self.volume
        dv.single_bond = single
        dv.atom_B2 = B2
        dv.atom_norms = norms
        dv.b2_count = b2_count
        dv.b2_cum = cum
        dv.b2_idx = b2_idx
        dv.b2_coords = coords
        dv.descriptors, dv.descriptor_force_dervs, dv.neighbor_coordinates = \
            [], [], []
        dv.descriptor_norms, dv.descriptor_force_dots = [], []
        dv.neighbor_counts, dv.cumulative_neighbor_counts = [], []
        dv.atom_indices, dv.neighbor_indices = [], []
        dv.n_clusters_by_type, dv.cumulative_type_count = [], [0]
        dv.n_neighbors_by_type = []
        dv.n_clusters = 0
        for s in range(S):
            atoms = np.nonzero(sp == s)[0]
            dv.n_clusters_by_type.append(len(atoms))
            dv.cumulative_type_count.append(dv.cumulative_type_count[-1] +
                                            len(atoms))
            dv.n_clusters += len(atoms)
            dv.descriptors.append(B2[atoms])
            dv.descriptor_norms.append(norms[atoms])
            dv.atom_indices.append(atoms.astype(np.int32))
            cnts = b2_count[atoms]
            dv.neighbor_counts.append(cnts.astype(np.int32))
            c2 = np.zeros(len(atoms), dtype=np.int32)
            if len(atoms):
                c2[1:] = np.cumsum(cnts)[:-1]
            dv.cumulative_neighbor_counts.append(c2)
            dv.n_neighbors_by_type.append(int(cnts.sum()))
            pair_rows = np.concatenate(
                [np.arange(cum[a], cum[a + 1]) for a in atoms]).astype(
                    np.int64) if len(atoms) else np.zeros(0, np.int64)
            dv.neighbor_indices.append(b2_idx[pair_rows])
            dv.neighbor_coordinates.append(coords[pair_rows])
            if compute_dervs:
                # contiguous per-atom blocks (b2.cpp:159-166 block copies)
                blocks = [dervs[3 * cum[a]:3 * cum[a + 1]] for a in atoms]
                dv.descriptor_force_dervs.append(
                    np.concatenate(blocks) if blocks else np.zeros((0, nd)))
                fblocks = [fdots[3 * cum[a]:3 * cum[a + 1]] for a in atoms]
                dv.descriptor_force_dots.append(
                    np.concatenate(fblocks) if fblocks else np.zeros(0))
        return dv


# ----------------------------------------------------------------- kernel
class NormalizedDotProduct:
    """normalized_dot_product.cpp:15-214."""

    def __init__(self, sigma, power):
        self.sigma = float(sigma)
        self.power = float(power)

    @property
    def kernel_hyperparameters(self):
        return np.array([self.sigma])

    def envs_envs(self, envs1, envs2, hyps=None):
        sig = self.sigma if hyps is None else hyps[0]
        sig_sq = sig * sig
        K = np.zeros((envs1.n_clusters, envs2.n_clusters))
        thr = 1e-8
        for s in range(envs1.n_types):
            d1, d2 = envs1.descriptors[s], envs2.descriptors[s]
            n1, n2 = envs1.descriptor_norms[s], envs2.descriptor_norms[s]
            if d1.shape[0] == 0 or d2.shape[0] == 0:
                continue
            dot = d1 @ d2.T
            nd = dot / np.outer(n1, n2)
            with np.errstate(invalid="ignore", divide="ignore"):
                k = sig_sq * np.power(nd, self.power)
            mask = (n1[:, None] >= thr) & (n2[None, :] >= thr)
            k = np.where(mask, k, 0.0)
            c1, c2 = envs1.cumulative_type_count[s], envs2.cumulative_type_count[s]
            K[c1:c1 + d1.shape[0], c2:c2 + d2.shape[0]] += k
        return K

    def envs_struc(self, envs, struc, hyps=None):
        sig = self.sigma if hyps is None else hyps[0]
        sig_sq = sig * sig
        n_atoms = struc.n_atoms
        K = np.zeros((envs.n_clusters, 1 + 3 * n_atoms + 6))
        for s in range(envs.n_types):
            S = envs.descriptors[s]
            if S.shape[0] == 0 or S.shape[1] == 0:
                continue
            D = struc.descriptors[s]
            dot_vals = np.ascontiguousarray(S @ D.T)
            fd = struc.descriptor_force_dervs[s]
            force_dot = np.ascontiguousarray(S @ fd.T) if fd.shape[0] else \
                np.zeros((S.shape[0], 0))
            Ms, Ns = S.shape[0], D.shape[0]
            if Ns == 0:
                continue
            sn = np.ascontiguousarray(envs.descriptor_norms[s])
            dn = np.ascontiguousarray(struc.descriptor_norms[s])
            sfd = np.ascontiguousarray(struc.descriptor_force_dots[s])
            nc = np.ascontiguousarray(struc.neighbor_counts[s], dtype=np.int32)
            cn = np.ascontiguousarray(struc.cumulative_neighbor_counts[s],
                                      dtype=np.int32)
            ai = np.ascontiguousarray(struc.atom_indices[s], dtype=np.int32)
            ni = np.ascontiguousarray(struc.neighbor_indices[s], dtype=np.int32)
            co = np.ascontiguousarray(struc.neighbor_coordinates[s])
            lib().orc_envs_struc_block(
                Ms, Ns, n_atoms, envs.cumulative_type_count[s], _dp(sn), _dp(dn),
                _dp(dot_vals), _dp(force_dot), _dp(sfd), _ip(nc), _ip(cn),
                _ip(ai), _ip(ni), _dp(co), sig_sq, self.power,
                1.0 / struc.volume, _dp(K))
        return K


    def struc_struc(self, struc1, struc2, hyps=None):
        """Structure-structure kernel (normalized_dot_product.cpp:216-448):
        (1 + 3 N1 + 6) x (1 + 3 N2 + 6), per species with dot_vals,
        force_dot_1/2 and force_force precomputed as the reference does."""
        sig = self.sigma if hyps is None else hyps[0]
        out = np.zeros((1 + 3 * struc1.n_atoms + 6, 1 + 3 * struc2.n_atoms + 6))
        c = np.ascontiguousarray
        for s in range(struc1.n_types):
            D1, D2 = c(struc1.descriptors[s]), c(struc2.descriptors[s])
            if D1.shape[0] == 0 or D2.shape[0] == 0:
                continue
            f1, f2 = struc1.descriptor_force_dervs[s], struc2.descriptor_force_dervs[s]
            side = []
            for st in (struc1, struc2):
                side += [c(st.descriptor_force_dots[s]),
                         c(st.neighbor_counts[s], np.int32),
                         c(st.cumulative_neighbor_counts[s], np.int32),
                         c(st.atom_indices[s], np.int32),
                         c(st.neighbor_indices[s], np.int32),
                         c(st.neighbor_coordinates[s])]
            args = [D1.shape[0], D2.shape[0], struc1.n_atoms, struc2.n_atoms,
                    _dp(c(struc1.descriptor_norms[s])),
                    _dp(c(struc2.descriptor_norms[s])), _dp(c(D1 @ D2.T)),
                    _dp(c(f1 @ D2.T)), _dp(c(f2 @ D1.T)), _dp(c(f1 @ f2.T)),
                    _dp(side[0]), _dp(side[6])]
            for k in (0, 6):
                args += [_ip(side[k + 1]), _ip(side[k + 2]), _ip(side[k + 3]),
                         _ip(side[k + 4]), _dp(side[k + 5])]
            args += [sig * sig, self.power, 1.0 / struc1.volume,
                     1.0 / struc2.volume, _dp(out)]
            if lib().orc_struc_struc_block(*args) != 0:
                raise ValueError(
                    "Dot product of descriptors is 0, and the negative power "
                    "function in force-force kernel diverges.")
        return out

    def self_kernel_struc(self, struc, hyps=None):
        """Prior variances of E, F, S (normalized_dot_product.cpp:450-586):
        [1 + 3N + 6], the per-species loop over atom pairs and neighbour
        entries with dot_vals, force_dot and force_force precomputed as the
        reference does."""
        sig = self.sigma if hyps is None else hyps[0]
        n_atoms = struc.n_atoms
        out = np.zeros(1 + 3 * n_atoms + 6)
        for s in range(struc.n_types):
            D = np.ascontiguousarray(struc.descriptors[s])
            Ns = D.shape[0]
            if Ns == 0:
                continue
            fd = struc.descriptor_force_dervs[s]
            dot_vals = np.ascontiguousarray(D @ D.T)
            force_dot = np.ascontiguousarray(fd @ D.T) if fd.shape[0] else \
                np.zeros((0, Ns))
            force_force = np.ascontiguousarray(fd @ fd.T) if fd.shape[0] else \
                np.zeros((0, 0))
            rc = lib().orc_self_kernel_block(
                Ns, n_atoms, _dp(np.ascontiguousarray(struc.descriptor_norms[s])),
                _dp(dot_vals), _dp(force_dot), _dp(force_force),
                _dp(np.ascontiguousarray(struc.descriptor_force_dots[s])),
                _ip(np.ascontiguousarray(struc.neighbor_counts[s], np.int32)),
                _ip(np.ascontiguousarray(struc.cumulative_neighbor_counts[s],
                                         np.int32)),
                _ip(np.ascontiguousarray(struc.atom_indices[s], np.int32)),
                _ip(np.ascontiguousarray(struc.neighbor_indices[s], np.int32)),
                _dp(np.ascontiguousarray(struc.neighbor_coordinates[s])),
                sig * sig, self.power, 1.0 / struc.volume, _dp(out))
            if rc != 0:
                raise ValueError(
                    "Dot product of descriptors is 0, and the negative power "
                    "function in force-force kernel diverges.")
        return out


# --------------------------------------------------------------- SparseGP
class SparseGP:
    """sparse_gp.cpp:14-757 (prediction + the QR solve)."""

    def __init__(self, kernels, energy_noise, force_noise, stress_noise):
        self.kernels = kernels
        self.n_kernels = len(kernels)
        self.Kuu_jitter = 1e-8
        self.energy_noise = energy_noise
        self.force_noise = force_noise
        self.stress_noise = stress_noise
        self.hyperparameters = np.concatenate(
            [k.kernel_hyperparameters for k in kernels] +
            [np.array([energy_noise, force_noise, stress_noise])])
        self.Kuu_kernels = [np.zeros((0, 0)) for _ in kernels]
        self.Kuf_kernels = [np.zeros((0, 0)) for _ in kernels]
        self.sparse_descriptors = []
        self.sparse_indices = []
        self.training_structures = []
        self.training_atom_indices = []
        self.label_count = [0]
        self.y = np.zeros(0)
        self.noise_vector = np.zeros(0)
        self.n_labels = 0
        self.n_sparse = 0
        self.n_strucs = 0
        self.L_inv = None

    @staticmethod
    def from_weights(kernels, sparse_descriptors, alpha, L_inv):
        """A solved model carrying given weights (no training data): per
        kernel a ClusterDescriptor-like object (n_types, n_descriptors,
        descriptors, descriptor_norms, n_clusters_by_type), alpha [M] and
        L_inv [M x M].  Prediction then follows sparse_gp.cpp:643-757 with
        exactly these weights, so another implementation's model can be
        checked against this oracle."""
        gp = SparseGP(kernels, 1.0, 1.0, 1.0)
        for i, sd in enumerate(sparse_descriptors):
            cd = ClusterDescriptor(sd.n_types, sd.n_descriptors)
            cd.descriptors = [np.asarray(d, np.float64).reshape(
                -1, sd.n_descriptors) for d in sd.descriptors]
            cd.descriptor_norms = [np.asarray(d, np.float64)
                                   for d in sd.descriptor_norms]
            cd.n_clusters_by_type = [len(d) for d in cd.descriptor_norms]
            for s in range(1, cd.n_types):
                cd.cumulative_type_count[s] = (cd.cumulative_type_count[s - 1]
                                               + cd.n_clusters_by_type[s - 1])
            cd.n_clusters = sum(cd.n_clusters_by_type)
            gp.sparse_descriptors.append(cd)
            gp.Kuu_kernels[i] = np.zeros((cd.n_clusters, cd.n_clusters))
        gp.n_sparse = sum(cd.n_clusters for cd in gp.sparse_descriptors)
        gp._stack_Kuu()
        gp.alpha = np.asarray(alpha, np.float64).copy()
        gp.L_inv = np.asarray(L_inv, np.float64).copy()
        return gp

    def initialize_sparse_descriptors(self, structure):
        if self.sparse_descriptors:
            return
        for dv in structure.descriptors:
            self.sparse_descriptors.append(
                ClusterDescriptor(dv.n_types, dv.n_descriptors))
            self.sparse_indices.append([])

    # sparse_gp.cpp:474-583
    def add_training_structure(self, structure, atom_indices=(-1,),
                               rel_e_noise=1.0, rel_f_noise=1.0,
                               rel_s_noise=1.0):
        self.initialize_sparse_descriptors(structure)
        n_atoms = structure.noa
        n_energy = structure.energy.size
        atom_indices = list(atom_indices)
        if atom_indices[0] == -1:
            atoms = list(range(n_atoms))
            n_force = structure.forces.size
        else:
            atoms = atom_indices
            n_force = 3 * len(atoms)
        self.training_atom_indices.append(atoms)
        n_stress = structure.stresses.size
        nl = n_energy + n_force + n_stress
        self.label_count.append(self.n_labels + nl)
        yy = np.zeros(nl)
        yy[:n_energy] = np.asarray(structure.energy).reshape(-1)
        f = np.asarray(structure.forces).reshape(-1)
        for a, at in enumerate(atoms):
            if n_force:
                yy[n_energy + 3 * a:n_energy + 3 * a + 3] = f[3 * at:3 * at + 3]
        yy[n_energy + n_force:] = np.asarray(structure.stresses).reshape(-1)
        self.y = np.concatenate([self.y, yy])
        nv = np.zeros(nl)
        nv[:n_energy] = 1 / (self.energy_noise ** 2 * rel_e_noise ** 2)
        nv[n_energy:n_energy + n_force] = 1 / (self.force_noise ** 2 *
                                               rel_f_noise ** 2)
        nv[n_energy + n_force:] = 1 / (self.stress_noise ** 2 * rel_s_noise ** 2)
        self.noise_vector = np.concatenate([self.noise_vector, nv])
        for i, k in enumerate(self.kernels):
            n_sparse = self.sparse_descriptors[i].n_clusters
            esk = k.envs_struc(self.sparse_descriptors[i],
                               structure.descriptors[i])
            blk = np.zeros((n_sparse, nl))
            blk[:, :n_energy] = esk[:, :n_energy]
            blk[:, n_energy + n_force:] = esk[:, 1 + 3 * n_atoms:1 + 3 * n_atoms +
                                              n_stress]
            for a, at in enumerate(atoms):
                if n_force:
                    blk[:, n_energy + 3 * a:n_energy + 3 * a + 3] = \
                        esk[:, 1 + 3 * at:1 + 3 * at + 3]
            old = self.Kuf_kernels[i]
            if old.shape[0] != n_sparse:
                old = np.zeros((n_sparse, self.n_labels))
            self.Kuf_kernels[i] = np.hstack([old, blk])
        self.n_labels += nl
        self.training_structures.append(structure)
        self.n_strucs += 1
        self._stack_Kuf()

    # sparse_gp.cpp:141-189
    def add_specific_environments(self, structure, atoms):
        self.initialize_sparse_descriptors(structure)
        atoms = list(atoms)
        indices_1 = []
        for i in range(self.n_kernels):
            self.sparse_indices[i].append(atoms)
            dv = structure.descriptors[i]
            ind2 = []
            for j in range(dv.n_types):
                ind3 = []
                for k in range(dv.n_clusters_by_type[j]):
                    a1 = int(dv.atom_indices[j][k])
                    for a2 in atoms:
                        if a1 == a2:
                            ind3.append(k)
                ind2.append(ind3)
            indices_1.append(ind2)
        clusters = [ClusterDescriptor.from_values(structure.descriptors[i],
                                                  indices_1[i])
                    for i in range(self.n_kernels)]
        self._update_Kuu(clusters)
        self._update_Kuf(clusters)
        self._stack_Kuu()
        self._stack_Kuf()
        for i in range(self.n_kernels):
            self.sparse_descriptors[i].add_clusters_by_type(
                structure.descriptors[i], indices_1[i])

    def add_all_environments(self, structure):
        self.initialize_sparse_descriptors(structure)
        clusters = [ClusterDescriptor.from_values(dv)
                    for dv in structure.descriptors]
        self._update_Kuu(clusters)
        self._update_Kuf(clusters)
        self._stack_Kuu()
        self._stack_Kuf()
        for i in range(self.n_kernels):
            dv = structure.descriptors[i]
            self.sparse_descriptors[i].add_clusters_by_type(
                dv, [list(range(dv.n_clusters_by_type[s]))
                     for s in range(dv.n_types)])
            self.sparse_indices[i].append(list(range(structure.noa)))

    # sparse_gp.cpp:343-400 (type-blocked Kuu growth)
    def _update_Kuu(self, clusters):
        for i, k in enumerate(self.kernels):
            sd, cd = self.sparse_descriptors[i], clusters[i]
            prev = k.envs_envs(sd, cd)
            selfb = k.envs_envs(cd, cd)
            ns, ne, nt = sd.n_clusters, cd.n_clusters, cd.n_types
            km = np.zeros((ns + ne, ns + ne))
            n1 = n2 = 0
            for j in range(nt):
                n3 = n4 = 0
                n5, n6 = sd.n_clusters_by_type[j], cd.n_clusters_by_type[j]
                for kk in range(nt):
                    n7, n8 = sd.n_clusters_by_type[kk], cd.n_clusters_by_type[kk]
                    km[n1 + n2:n1 + n2 + n5, n3 + n4:n3 + n4 + n7] = \
                        self.Kuu_kernels[i][n1:n1 + n5, n3:n3 + n7]
                    km[n1 + n2:n1 + n2 + n5, n3 + n4 + n7:n3 + n4 + n7 + n8] = \
                        prev[n1:n1 + n5, n4:n4 + n8]
                    km[n1 + n2 + n5:n1 + n2 + n5 + n6, n3 + n4:n3 + n4 + n7] = \
                        prev[n3:n3 + n7, n2:n2 + n6].T
                    km[n1 + n2 + n5:n1 + n2 + n5 + n6,
                       n3 + n4 + n7:n3 + n4 + n7 + n8] = \
                        selfb[n2:n2 + n6, n4:n4 + n8]
                    n3 += n7
                    n4 += n8
                n1 += n5
                n2 += n6
            self.Kuu_kernels[i] = km
            self.n_sparse += ne

    # sparse_gp.cpp:402-472
    def _update_Kuf(self, clusters):
        for i, k in enumerate(self.kernels):
            sd, cd = self.sparse_descriptors[i], clusters[i]
            ns, ne, nt = sd.n_clusters, cd.n_clusters, cd.n_types
            inds = [0]
            for j in range(nt):
                inds.append(inds[-1] + sd.n_clusters_by_type[j] +
                            cd.n_clusters_by_type[j])
            km = np.zeros((ns + ne, self.n_labels))
            for j, struc in enumerate(self.training_structures):
                n_atoms = struc.noa
                esk = k.envs_struc(cd, struc.descriptors[i])
                n1 = n2 = 0
                lc = self.label_count[j]
                for kk in range(nt):
                    cc = 0
                    u = inds[kk]
                    n3, n4 = sd.n_clusters_by_type[kk], cd.n_clusters_by_type[kk]
                    old = self.Kuf_kernels[i]
                    if struc.energy.size:
                        km[u:u + n3, lc] = old[n1:n1 + n3, lc] if n3 else 0
                        km[u + n3:u + n3 + n4, lc] = esk[n2:n2 + n4, 0]
                        cc += 1
                    if struc.forces.size:
                        for at in self.training_atom_indices[j]:
                            if n3:
                                km[u:u + n3, lc + cc:lc + cc + 3] = \
                                    old[n1:n1 + n3, lc + cc:lc + cc + 3]
                            km[u + n3:u + n3 + n4, lc + cc:lc + cc + 3] = \
                                esk[n2:n2 + n4, 1 + 3 * at:1 + 3 * at + 3]
                            cc += 3
                    if struc.stresses.size:
                        if n3:
                            km[u:u + n3, lc + cc:lc + cc + 6] = \
                                old[n1:n1 + n3, lc + cc:lc + cc + 6]
                        km[u + n3:u + n3 + n4, lc + cc:lc + cc + 6] = \
                            esk[n2:n2 + n4, 1 + 3 * n_atoms:1 + 3 * n_atoms + 6]
                    n1 += n3
                    n2 += n4
            self.Kuf_kernels[i] = km

    def _stack_Kuu(self):
        self.Kuu = sla.block_diag(*self.Kuu_kernels) if self.Kuu_kernels else \
            np.zeros((0, 0))

    def _stack_Kuf(self):
        self.Kuf = np.vstack([k if k.shape[1] == self.n_labels else
                              np.zeros((k.shape[0], self.n_labels))
                              for k in self.Kuf_kernels])

    # sparse_gp.cpp:607-641
    def update_matrices_QR(self):
        M = self.Kuu.shape[0]
        nsq = np.sqrt(self.noise_vector)
        Lc = np.linalg.cholesky(self.Kuu + self.Kuu_jitter * np.eye(M))
        self.L_inv = sla.solve_triangular(Lc, np.eye(M), lower=True)
        self.Kuu_inverse = self.L_inv.T @ self.L_inv
        A = np.vstack([nsq[:, None] * self.Kuf.T, Lc.T])
        b = np.concatenate([nsq * self.y, np.zeros(M)])
        Q, R = np.linalg.qr(A, mode="reduced")
        Qb = Q.T @ b
        self.R_inv = sla.solve_triangular(R, np.eye(M), lower=False)
        self.alpha = self.R_inv @ Qb
        self.Sigma = self.R_inv @ self.R_inv.T

    def _kernel_mat(self, structure):
        n_out = 1 + 3 * structure.noa + 6
        km = np.zeros((self.n_sparse, n_out))
        c = 0
        for i, k in enumerate(self.kernels):
            sz = self.Kuu_kernels[i].shape[0]
            km[c:c + sz] = k.envs_struc(self.sparse_descriptors[i],
                                        structure.descriptors[i])
            c += sz
        return km

    def _check(self):
        if self.L_inv is None or self.L_inv.shape[0] != self.Kuu.shape[0]:
            raise RuntimeError("L_inv must be up to date to make predictions. "
                               "Please call update_matrices_QR and try again.")

    def predict_mean(self, structure):
        self._check()
        structure.mean_efs = self._kernel_mat(structure).T @ self.alpha

    def predict_SOR(self, structure):
        self._check()
        km = self._kernel_mat(structure)
        structure.mean_efs = km.T @ self.alpha
        vs = km.T @ self.R_inv
        structure.variance_efs = np.einsum("ij,ij->i", vs, vs)

    def predict_DTC(self, structure):
        """sparse_gp.cpp:694-729: mean_efs, and variance_efs = K_self -
        diag(K^T Kuu^-1 K) + diag(K^T Sigma K)."""
        self._check()
        km = self._kernel_mat(structure)
        structure.mean_efs = km.T @ self.alpha
        K_self = np.zeros(km.shape[1])
        for i, k in enumerate(self.kernels):
            K_self += k.self_kernel_struc(structure.descriptors[i])
        Q_self = np.einsum("ij,ij->j", km, self.Kuu_inverse @ km)
        V_SOR = np.einsum("ij,ij->j", km, self.Sigma @ km)
        structure.variance_efs = K_self - Q_self + V_SOR

    # sparse_gp.cpp:94-139
    def compute_cluster_uncertainties(self, structure):
        self._check()
        out = []
        count = 0
        for i, k in enumerate(self.kernels):
            cd = ClusterDescriptor.from_values(structure.descriptors[i])
            Kself = _self_kernel(k, cd)
            Kus = k.envs_envs(cd, self.sparse_descriptors[i])
            nc = self.sparse_descriptors[i].n_clusters
            Lb = self.L_inv[count:count + nc, count:count + nc]
            count += nc
            Q1 = Lb @ Kus.T
            out.append(Kself - np.einsum("ij,ij->j", Q1, Q1))
        return out

    def predict_local_uncertainties(self, structure):
        self._check()
        structure.mean_efs = self._kernel_mat(structure).T @ self.alpha
        structure.local_uncertainties = self.compute_cluster_uncertainties(
            structure)


def _self_kernel(k, cd):
    """Diagonal of envs_envs(cd, cd) (sparse_gp.cpp:116-119) without the
    N x N matrix: sig^2 (d.d / |d||d|)^power, zero for norms < 1e-8."""
    out = []
    for s in range(cd.n_types):
        D, n = cd.descriptors[s], cd.descriptor_norms[s]
        dd = np.einsum("ij,ij->i", D, D)
        with np.errstate(invalid="ignore", divide="ignore"):
            v = k.sigma ** 2 * np.power(dd / (n * n), k.power)
        out.append(np.where(n >= 1e-8, v, 0.0))
    return np.concatenate(out) if out else np.zeros(0)


# --------------------------------------------------------- calculator post
def sort_variances(structure, variances):
    """calculator.py:188-206."""
    out = np.zeros(len(variances))
    dv = structure.descriptors[0]
    v = 0
    for s in range(dv.n_types):
        for a in dv.atom_indices[s]:
            out[a] = variances[v]
            v += 1
    return out


def calculator_results(structure, variance_type, sigma,
                       single_atom_energies=None):
    """SGP_Calculator.predict_on_structure post-processing (calculator.py:66-122)."""
    res = {}
    m = structure.mean_efs
    res["energy"] = m[0]
    res["forces"] = m[1:-6].reshape(-1, 3).copy()
    if single_atom_energies is not None:
        for s in structure.species:
            res["energy"] += single_atom_energies[s]
    fs = m[-6:]
    res["stress"] = -np.array([fs[0], fs[3], fs[5], fs[4], fs[2], fs[1]])
    if variance_type in ("SOR", "DTC"):
        v = structure.variance_efs[1:-6]
        res["stds"] = np.where(v > 0, np.sqrt(np.abs(v)),
                               -np.sqrt(np.abs(v))).reshape(-1, 3)
    elif variance_type == "local":
        v = sort_variances(structure, structure.local_uncertainties[0])
        stds = np.where(v > 0, np.sqrt(np.abs(v)), -np.sqrt(np.abs(v)))
        full = np.zeros((len(v), 3))
        full[:, 0] = stds / abs(sigma)
        res["stds"] = full
    return res


# ------------------------------------------------------------ mapped models
def mapping_coefficients(sgp, kernel_index=0):
    """NormalizedDotProduct::compute_map_coeff_pow1 / _pow2
    (normalized_dot_product.cpp:653-767): per species, over its non-empty
    sparse environments j in order, beta += sig2 p_k alpha_j (power 1) or
    beta(k<=l) += (k == l ? 1 : 2) sig2 p_k p_l alpha_j (power 2),
    p = s_j / |s_j|; the upper triangle row by row."""
    k = sgp.kernels[kernel_index]
    cd = sgp.sparse_descriptors[kernel_index]
    sig2 = k.sigma ** 2
    p = cd.n_descriptors
    alpha_ind = sum(sgp.sparse_descriptors[i].n_clusters
                    for i in range(kernel_index))
    if k.power == 1:
        out = np.zeros((cd.n_types, p))
    else:
        iu = np.triu_indices(p)
        fac = np.where(iu[0] == iu[1], 1.0, 2.0)
        out = np.zeros((cd.n_types, len(iu[0])))
    for s in range(cd.n_types):
        c = cd.cumulative_type_count[s]
        for j in range(cd.n_clusters_by_type[s]):
            nrm = cd.descriptor_norms[s][j]
            if nrm < 1e-8:
                continue
            a = sgp.alpha[alpha_ind + c + j]
            pv = cd.descriptors[s][j] / nrm
            if k.power == 1:
                out[s] += sig2 * pv * a
            else:
                out[s] += fac * (sig2 * pv[iu[0]] * pv[iu[1]] * a)
    return out


def varmap_coefficients(sgp, kernel_index=0):
    """NormalizedDotProduct::compute_varmap_coefficients
    (normalized_dot_product.cpp:769-830): Householder QR (LAPACK, standing in
    for Eigen's HouseholderQR) of [S^T; sqrt(jitter)/sigma I] per species;
    coefficient (i, j) = Q(i, j) for j < n_s, row-major p x p."""
    k = sgp.kernels[kernel_index]
    cd = sgp.sparse_descriptors[kernel_index]
    p = cd.n_descriptors
    jr = math.sqrt(sgp.Kuu_jitter)
    out = np.zeros((cd.n_types, p * p))
    for s in range(cd.n_types):
        n = cd.n_clusters_by_type[s]
        if n == 0:
            continue
        pi = np.array(cd.descriptors[s], dtype=np.float64)
        for i in range(n):
            if cd.descriptor_norms[s][i] >= 1e-8:
                pi[i] = pi[i] / cd.descriptor_norms[s][i]
        A = np.vstack([pi.T, jr * np.eye(n) / k.sigma])
        Q, _ = np.linalg.qr(A, mode="reduced")
        blk = np.zeros((p, p))
        w = min(n, p)
        blk[:, :w] = Q[:p, :w]
        out[s] = blk.reshape(-1)
    return out


def write_mapping_text(coeffs, power, descriptor_settings, radial_basis,
                       cutoff_function, cutoffs, contributor, date):
    """SparseGP::write_mapping_coefficients (sparse_gp.cpp:1199-1264) with
    NormalizedDotProduct::write_info (:832-835) and B2::write_to_file
    (b2.cpp:52-74), statement by statement."""
    o = ["DATE: ", date, " ", "CONTRIBUTOR: ", contributor, "\n"]
    o += ["%.0f" % power, " NormalizedDotProduct\n"]
    S, N, L = descriptor_settings
    o += [radial_basis, "\n", "%d %d %d " % (S, N, L), "%d" % coeffs.shape[1],
          "\n", cutoff_function, "\n"]
    for i in range(S):
        for j in range(S):
            o += ["%.2f" % cutoffs[i][j], " "]
    o += ["\n"]
    count = 0
    for i in range(coeffs.shape[0]):
        if count != 0:
            o += ["\n"]
        for j in range(coeffs.shape[1]):
            v = coeffs[i, j]
            o += ["  " if v > 0 else " ", "%.16e" % v]
            count += 1
            if count == 5:
                count = 0
                o += ["\n"]
    return "".join(o)


def mapped_energy_and_w(B2, beta, power, normalized=True):
    """compute_energy_and_u (lammps_descriptor.cpp:250-275): the local
    energy and w = dE/dB2 from one B2 vector and the species' beta (matrix
    for power 2, vector for power 1)."""
    n2 = float(B2 @ B2)
    if normalized:
        if power == 1:
            nrm = n2 ** 0.5
            e = float(B2 @ beta) / nrm
            w = beta / nrm - e * B2 / n2
        else:
            bp = beta @ B2
            e = float(B2 @ bp) / n2
            w = 2 * (bp - e * B2) / n2
    else:
        if power == 1:
            w = beta.copy()
            e = float(B2 @ w)
        else:
            bp = beta @ B2
            e = float(B2 @ bp)
            w = 2 * bp
    return e, w
