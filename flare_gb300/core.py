"""Drop-in classes for FLARE's sparse-GP prediction path on one GB300.

Names, constructor signatures, attributes and exception types follow the
reference's pybind11 module ``_C_flare`` (src/ace_binding.cpp:28-262):
``Structure``, ``DescriptorValues``, ``ClusterDescriptor``, ``B2``,
``NormalizedDotProduct`` and ``SparseGP``.  All numerical work runs in
libflaregb (CUDA, sm_103a) through the C ABI; torch is used only to own
device memory and streams.

Differences from the reference, by design:
  * ``Structure`` builds its neighbour list and descriptors on the GPU lazily
    (on first access, or when a SparseGP call needs them); prediction goes
    straight from positions to energy/forces/stress/variance in one pipeline.
  * The forward-mode descriptor gradients (``descriptor_force_dervs``) are
    only materialised for training (``add_training_structure``), never for
    prediction, which uses the reverse-mode adjoint.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr, stream_ptr

_prec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}
_default_precision = ["fp64"]


def set_precision(mode):
    """Select the prediction precision: "fp64" or "mixed"."""
    if mode not in _prec:
        raise ValueError(f"unknown precision {mode!r}")
    _default_precision[0] = mode


def get_precision():
    return _default_precision[0]


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("flare_gb300 needs a CUDA device (no CPU path)")
    return torch.device("cuda", torch.cuda.current_device())


# ------------------------------------------------------------------ B2
class B2:
    """B2(radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
    descriptor_settings[, cutoffs]) — src/flare_pp/descriptors/b2.cpp:13-50."""

    descriptor_name = "B2"

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings, cutoffs=None):
        self.radial_basis = str(radial_basis)
        self.cutoff_function = str(cutoff_function)
        self.radial_hyps = [float(x) for x in radial_hyps]
        self.cutoff_hyps = [float(x) for x in cutoff_hyps]
        self.descriptor_settings = [int(x) for x in descriptor_settings]
        if len(self.descriptor_settings) != 3:
            raise ValueError("descriptor_settings must be [n_species, n_max, l_max]")
        S = self.descriptor_settings[0]
        if cutoffs is None:
            cutoffs = np.full((S, S), self.radial_hyps[1])
        self.cutoffs = np.ascontiguousarray(np.asarray(cutoffs, np.float64))
        if self.cutoffs.shape != (S, S):
            raise ValueError("cutoffs must be n_species x n_species")
        if self.radial_basis not in _lib.RADIAL:
            raise ValueError(
                f"unknown radial basis {self.radial_basis!r} "
                f"(radial.cpp:381-408 names: {sorted(_lib.RADIAL)})")
        if self.cutoff_function not in _lib.CUTOFF:
            raise ValueError(f"unknown cutoff function {self.cutoff_function!r}")
        self._handle = None

    @property
    def handle(self):
        if self._handle is None:
            h = ctypes.c_void_p()
            rh = np.asarray(self.radial_hyps, np.float64)
            ch = np.asarray(self.cutoff_hyps if self.cutoff_hyps else [0.0],
                            np.float64)
            S, N, L = self.descriptor_settings
            check(lib().fgb_b2_create(
                ctypes.byref(h), _lib.RADIAL[self.radial_basis],
                _lib.CUTOFF[self.cutoff_function], ptr(rh), len(rh), ptr(ch),
                len(self.cutoff_hyps), S, N, L, ptr(self.cutoffs)), "B2")
            self._handle = h
            self._keep = (rh, ch)
        return self._handle

    @property
    def n_descriptors(self):
        S, N, L = self.descriptor_settings
        nr = S * N
        return nr * (nr + 1) // 2 * (L + 1)

    @property
    def n_single_bond(self):
        S, N, L = self.descriptor_settings
        return S * N * (L + 1) ** 2

    def __del__(self):
        if getattr(self, "_handle", None) is not None and _lib._lib is not None:
            _lib._lib.fgb_b2_destroy(self._handle)
            self._handle = None

    def __getstate__(self):
        d = dict(self.__dict__)
        d["_handle"] = None
        d.pop("_keep", None)
        return d

    def as_dict(self):
        return {"type": "B2", "radial_basis": self.radial_basis,
                "cutoff_function": self.cutoff_function,
                "radial_hyps": self.radial_hyps,
                "cutoff_hyps": self.cutoff_hyps,
                "descriptor_settings": self.descriptor_settings,
                "cutoffs": self.cutoffs.tolist()}


# ------------------------------------------------------------ kernel
class NormalizedDotProduct:
    """k = sigma^2 (d1.d2 / |d1||d2|)^power
    (src/flare_pp/kernels/normalized_dot_product.cpp:15-26)."""

    kernel_name = "NormalizedDotProduct"

    def __init__(self, sigma, power):
        self.sigma = float(sigma)
        self.power = float(power)

    @property
    def kernel_hyperparameters(self):
        return np.array([self.sigma])

    def envs_envs(self, envs1, envs2, hyps=None):
        """Kernel matrix between two ClusterDescriptors (FP64 on the GPU)."""
        sig = self.sigma if hyps is None else float(np.asarray(hyps)[0])
        return envs_envs_gpu(envs1, envs2, sig, self.power)

    def envs_struc(self, envs, struc, hyps=None):
        """Kernel matrix between a ClusterDescriptor and a structure
        (sparse rows x [energy, 3N forces, 6 stress]); ``struc`` is a
        Structure (FP64 on the GPU, stored-gradient form)."""
        sig = self.sigma if hyps is None else float(np.asarray(hyps)[0])
        return envs_struc_gpu(envs, struc, sig, self.power)

    def struc_struc(self, struc1, struc2, hyps=None):
        """Kernel between every output (energy, 3N forces, 6 stresses) of
        two structures, (1 + 3 N1 + 6) x (1 + 3 N2 + 6)
        (normalized_dot_product.cpp:216-448); Structures (FP64 on the
        GPU)."""
        sig = self.sigma if hyps is None else float(np.asarray(hyps)[0])
        calc = struc1.descriptor_calculators[0]
        out = torch.zeros((1 + 3 * struc1.noa + 6, 1 + 3 * struc2.noa + 6),
                          dtype=torch.float64, device=_device())
        d1, d2 = struc1._inputs(), struc2._inputs()
        check(lib().fgb_struc_struc(calc.handle, sig, self.power,
                                    struc1.nlist().h, ptr(d1["species"]),
                                    struc2.nlist().h, ptr(d2["species"]),
                                    ptr(out), stream_ptr()),
              "struc_struc")
        return out.cpu().numpy()

    def self_kernel_struc(self, struc, hyps=None, kernel_index=0):
        """Prior variances of a structure's energy, forces and stress
        [1 + 3N + 6] (normalized_dot_product.cpp:450-586; the C++ method
        behind predict_DTC); ``struc`` is a Structure (FP64 on the GPU) and
        ``kernel_index`` picks its descriptor calculator."""
        sig = self.sigma if hyps is None else float(np.asarray(hyps)[0])
        calc = struc.descriptor_calculators[kernel_index]
        out = torch.zeros(1 + 3 * struc.noa + 6, dtype=torch.float64,
                          device=_device())
        d = struc._inputs()
        check(lib().fgb_self_kernel_struc(calc.handle, sig, self.power,
                                          struc.nlist().h, ptr(d["species"]),
                                          ptr(out), stream_ptr()),
              "self_kernel_struc")
        return out.cpu().numpy()


# ------------------------------------------------------- descriptors
class DescriptorValues:
    """Per-species descriptor values of one structure (descriptor.h:31-57)."""

    def __init__(self):
        self.n_descriptors = 0
        self.n_types = 0
        self.n_atoms = 0
        self.volume = 0.0
        self.descriptors = []
        self.descriptor_norms = []
        self.atom_indices = []
        self.neighbor_counts = []
        self.cumulative_neighbor_counts = []
        self.neighbor_indices = []
        self.neighbor_coordinates = []
        self.n_clusters_by_type = []
        self.cumulative_type_count = [0]
        self.n_neighbors_by_type = []
        self.n_clusters = 0


class ClusterDescriptor:
    """Sparse-set style descriptor collection (descriptor.h:61-90)."""

    def __init__(self, n_types=0, n_descriptors=0):
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
        """descriptor.cpp:104-140."""
        for s in range(self.n_types):
            idx = np.asarray(clusters[s], dtype=np.int64)
            if idx.size:
                self.descriptors[s] = np.vstack([self.descriptors[s],
                                                 dv.descriptors[s][idx]])
                self.descriptor_norms[s] = np.concatenate(
                    [self.descriptor_norms[s], dv.descriptor_norms[s][idx]])
        for s in range(self.n_types):
            self.n_clusters_by_type[s] += len(clusters[s])
            self.n_clusters += len(clusters[s])
            if s > 0:
                self.cumulative_type_count[s] = (
                    self.cumulative_type_count[s - 1] +
                    self.n_clusters_by_type[s - 1])

    def add_clusters(self, dv, clusters):
        """descriptor.cpp:81-102: clusters given as structure-wide indices."""
        by_type = [[] for _ in range(dv.n_types)]
        for c in clusters:
            for s in range(dv.n_types):
                if dv.cumulative_type_count[s] <= c < dv.cumulative_type_count[s + 1]:
                    by_type[s].append(c - dv.cumulative_type_count[s])
                    break
        self.add_clusters_by_type(dv, by_type)

    def stacked(self):
        """(counts_by_species, rows) with species-grouped rows."""
        rows = np.vstack([d for d in self.descriptors]) if self.n_types else \
            np.zeros((0, self.n_descriptors))
        return np.asarray(self.n_clusters_by_type, np.int32), \
            np.ascontiguousarray(rows, dtype=np.float64)


# ---------------------------------------------------------- structure
class _NList:
    """Owner of an fgb_nlist_t handle."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().fgb_nlist_create(ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.fgb_nlist_destroy(self.h)
            self.h = None


class Structure:
    """Structure(cell, species, positions[, cutoff, descriptor_calculators])
    — src/flare_pp/structure.cpp:7-43."""

    def __init__(self, cell, species, positions, cutoff=None,
                 descriptor_calculators=None):
        self.cell = np.ascontiguousarray(np.asarray(cell, np.float64).reshape(3, 3))
        self.species = [int(s) for s in species]
        self.positions = np.ascontiguousarray(
            np.asarray(positions, np.float64).reshape(-1, 3))
        if self.positions.shape[0] != len(self.species):
            raise ValueError("positions and species disagree in length")
        self.noa = len(self.species)
        self.volume = abs(float(np.linalg.det(self.cell)))
        self.cell_transpose = self.cell.T.copy()
        self.cutoff = None if cutoff is None else float(cutoff)
        self.descriptor_calculators = list(descriptor_calculators or [])
        self.energy = np.zeros(0)
        self.forces = np.zeros(0)
        self.stresses = np.zeros(0)
        self.mean_efs = np.zeros(0)
        self.variance_efs = np.zeros(0)
        self.mean_contributions = []
        self.local_uncertainties = []
        self._nl = None
        self._dev = None
        self._descriptors = None
        self._dervs = {}

    # device copies of the inputs
    def _inputs(self):
        if self._dev is None:
            dev = _device()
            self._dev = {
                "pos": torch.from_numpy(self.positions).to(dev),
                "species": torch.tensor(self.species, dtype=torch.int32,
                                        device=dev),
                "offsets": np.array([0, self.noa], dtype=np.int32),
                "cell": np.ascontiguousarray(self.cell.reshape(-1)),
            }
        return self._dev

    def nlist(self):
        """Neighbour list (built once, on the GPU)."""
        if self._nl is None:
            if self.cutoff is None:
                raise ValueError("Structure has no cutoff")
            d = self._inputs()
            nl = _NList()
            check(lib().fgb_nlist_build(nl.h, 1, ptr(d["offsets"]),
                                        ptr(d["cell"]), ptr(d["pos"]),
                                        self.cutoff, stream_ptr()),
                  "Structure")
            self._nl = nl
        return self._nl

    def neighbor_arrays(self):
        """Reference-layout neighbour arrays (structure.cpp:93-117) as numpy:
        neighbor_count, cumulative_neighbor_count, structure_indices,
        neighbor_species, relative_positions (P x 4), shifts (P x 3),
        wrapped_positions."""
        nl = self.nlist()
        P = ctypes.c_longlong()
        n = ctypes.c_int()
        check(lib().fgb_nlist_size(nl.h, ctypes.byref(P), ctypes.byref(n)))
        P = P.value
        dev = _device()
        cnt = torch.zeros(max(self.noa, 1), dtype=torch.int32, device=dev)
        sidx = torch.zeros(max(P, 1), dtype=torch.int32, device=dev)
        sh = torch.zeros(max(3 * P, 1), dtype=torch.int32, device=dev)
        rel = torch.zeros(max(4 * P, 1), dtype=torch.float64, device=dev)
        wr = torch.zeros(max(3 * self.noa, 1), dtype=torch.float64, device=dev)
        check(lib().fgb_nlist_export(nl.h, ptr(cnt), ptr(sidx), ptr(sh),
                                     ptr(rel), ptr(wr), stream_ptr()))
        torch.cuda.current_stream().synchronize()
        out = {
            "neighbor_count": cnt.cpu().numpy()[:self.noa],
            "structure_indices": sidx.cpu().numpy()[:P],
            "shifts": sh.cpu().numpy()[:3 * P].reshape(P, 3),
            "relative_positions": rel.cpu().numpy()[:4 * P].reshape(P, 4),
            "wrapped_positions": wr.cpu().numpy()[:3 * self.noa].reshape(-1, 3),
        }
        c = np.zeros(self.noa + 1, dtype=np.int64)
        c[1:] = np.cumsum(out["neighbor_count"])
        out["cumulative_neighbor_count"] = c
        sp = np.asarray(self.species, np.int32)
        out["neighbor_species"] = sp[out["structure_indices"]] if P else \
            np.zeros(0, np.int32)
        return out

    @property
    def wrapped_positions(self):
        return self.neighbor_arrays()["wrapped_positions"]

    @property
    def n_neighbors(self):
        P = ctypes.c_longlong()
        check(lib().fgb_nlist_size(self.nlist().h, ctypes.byref(P), None))
        return P.value

    # ----------------------------------------------------- descriptors
    def b2_values(self, k=0):
        """(B2 [N x n_d], norms [N]) as device tensors, atom order."""
        calc = self.descriptor_calculators[k]
        d = self._inputs()
        dev = _device()
        B = torch.zeros((max(self.noa, 1), calc.n_descriptors),
                        dtype=torch.float64, device=dev)
        nrm = torch.zeros(max(self.noa, 1), dtype=torch.float64, device=dev)
        check(lib().fgb_b2_forward(calc.handle, self.nlist().h, ptr(d["species"]),
                                   ptr(B), ptr(nrm), stream_ptr()), "B2")
        return B[:self.noa], nrm[:self.noa]

    @property
    def descriptors(self):
        if self._descriptors is None:
            self._descriptors = [self._regroup(k) for k in
                                 range(len(self.descriptor_calculators))]
        return self._descriptors

    def compute_descriptors(self):
        self._descriptors = None
        return self.descriptors

    def _regroup(self, k):
        """Species regroup of B2 values (b2.cpp:104-176)."""
        calc = self.descriptor_calculators[k]
        B, nrm = self.b2_values(k)
        B = B.cpu().numpy()
        nrm = nrm.cpu().numpy()
        S = calc.descriptor_settings[0]
        sp = np.asarray(self.species)
        dv = DescriptorValues()
        dv.n_descriptors = calc.n_descriptors
        dv.n_types = S
        dv.n_atoms = self.noa
        dv.volume = self.volume
        for s in range(S):
            atoms = np.nonzero(sp == s)[0]
            dv.n_clusters_by_type.append(len(atoms))
            dv.cumulative_type_count.append(dv.cumulative_type_count[-1] +
                                            len(atoms))
            dv.n_clusters += len(atoms)
            dv.descriptors.append(B[atoms])
            dv.descriptor_norms.append(nrm[atoms])
            dv.atom_indices.append(atoms.astype(np.int32))
        return dv


# ------------------------------------------------------- GPU kernels
def envs_envs_gpu(envs1, envs2, sigma, power):
    """envs_envs (normalized_dot_product.cpp:28-89) in FP64."""
    dev = _device()
    K = torch.zeros((envs1.n_clusters, envs2.n_clusters), dtype=torch.float64,
                    device=dev)
    sig2 = sigma * sigma
    for s in range(envs1.n_types):
        d1 = torch.from_numpy(np.ascontiguousarray(envs1.descriptors[s])).to(dev)
        d2 = torch.from_numpy(np.ascontiguousarray(envs2.descriptors[s])).to(dev)
        if d1.shape[0] == 0 or d2.shape[0] == 0:
            continue
        n1 = torch.from_numpy(np.ascontiguousarray(
            envs1.descriptor_norms[s], dtype=np.float64)).to(dev)
        n2 = torch.from_numpy(np.ascontiguousarray(
            envs2.descriptor_norms[s], dtype=np.float64)).to(dev)
        blk = _kernel_block(d1, n1, d2, n2, sig2, power)
        c1, c2 = envs1.cumulative_type_count[s], envs2.cumulative_type_count[s]
        K[c1:c1 + d1.shape[0], c2:c2 + d2.shape[0]] = blk
    return K.cpu().numpy()


def _kernel_block(d1, n1, d2, n2, sig2, power):
    return _KernelBlock.run(d1, n1, d2, n2, sig2, power)


class _KernelBlock:
    """Dense FP64 kernel block via the model path (one species)."""

    @staticmethod
    def run(d1, n1, d2, n2, sig2, power):
        out = torch.empty((d1.shape[0], d2.shape[0]), dtype=torch.float64,
                          device=d1.device)
        check(lib().fgb_envs_envs(ptr(d1), ptr(n1), d1.shape[0], ptr(d2),
                                  ptr(n2), d2.shape[0], d1.shape[1], sig2,
                                  power, ptr(out), stream_ptr()), "envs_envs")
        return out


def _envs_struc_device(envs, struc, sigma, power, k=0):
    """envs_struc (normalized_dot_product.cpp:117-214) in FP64 on the GPU,
    stored-gradient form, as a device tensor; ``struc`` is a Structure and
    ``k`` the index of its descriptor calculator."""
    calc = struc.descriptor_calculators[k]
    counts, rows = envs.stacked()
    M = int(counts.sum())
    ncol = 1 + 3 * struc.noa + 6
    dev = _device()
    out = torch.zeros((M, ncol), dtype=torch.float64, device=dev)
    if M == 0:
        return out
    d_rows = torch.from_numpy(rows).to(dev)
    d = struc._inputs()
    check(lib().fgb_envs_struc(calc.handle, float(sigma), float(power),
                               ptr(counts), ptr(d_rows), struc.nlist().h,
                               ptr(d["species"]), ptr(out), stream_ptr()),
          "envs_struc")
    return out


def envs_struc_gpu(envs, struc, sigma, power, k=0):
    """envs_struc (normalized_dot_product.cpp:117-214) in FP64 on the GPU,
    stored-gradient form; ``struc`` is a Structure."""
    return _envs_struc_device(envs, struc, sigma, power, k).cpu().numpy()



# ------------------------------------------------------------ training
class _Training:
    """Kuu / Kuf / label bookkeeping of SparseGP (sparse_gp.cpp:141-641)."""

    def _init_training(self):
        self.training_atom_indices = []
        self.Kuu_kernels = [np.zeros((0, 0)) for _ in self.kernels]
        self.Kuf_kernels = [np.zeros((0, 0)) for _ in self.kernels]
        self.Kuu = np.zeros((0, 0))
        self.Kuf = np.zeros((0, 0))
        self.label_count = [0]
        self.y = np.zeros(0)
        self.noise_vector = np.zeros(0)
        # per label 1/rel_noise^2 of its kind, zero elsewhere
        # (sparse_gp.cpp:518-532), for set_hyperparameters
        self.e_noise_one = np.zeros(0)
        self.f_noise_one = np.zeros(0)
        self.s_noise_one = np.zeros(0)
        self.n_labels = 0
        self.n_strucs = 0
        self.n_energy_labels = 0
        self.n_force_labels = 0
        self.n_stress_labels = 0

    @property
    def n_sparse(self):
        return sum(sd.n_clusters for sd in self.sparse_descriptors)

    def _calcs(self, structure):
        self._calculators = list(structure.descriptor_calculators)
        return self._calculators

    def initialize_sparse_descriptors(self, structure):
        """sparse_gp.cpp:59-71."""
        if self.sparse_descriptors:
            return
        for calc in self._calcs(structure):
            self.sparse_descriptors.append(
                ClusterDescriptor(calc.descriptor_settings[0],
                                  calc.n_descriptors))
            self.sparse_indices.append([])

    def add_training_structure(self, structure, atom_indices=(-1,),
                               rel_e_noise=1.0, rel_f_noise=1.0,
                               rel_s_noise=1.0):
        """sparse_gp.cpp:474-583."""
        self.initialize_sparse_descriptors(structure)
        n_atoms = structure.noa
        energy = np.asarray(structure.energy, np.float64).reshape(-1)
        forces = np.asarray(structure.forces, np.float64).reshape(-1)
        stresses = np.asarray(structure.stresses, np.float64).reshape(-1)
        n_energy = energy.size
        atom_indices = list(np.asarray(atom_indices).reshape(-1))
        if atom_indices[0] == -1:
            atoms = list(range(n_atoms))
            n_force = forces.size
        else:
            atoms = [int(a) for a in atom_indices]
            n_force = 3 * len(atoms)
        self.training_atom_indices.append(atoms)
        n_stress = stresses.size
        nl = n_energy + n_force + n_stress
        self.label_count.append(self.n_labels + nl)
        yy = np.zeros(nl)
        yy[:n_energy] = energy
        if n_force:
            for a, at in enumerate(atoms):
                yy[n_energy + 3 * a:n_energy + 3 * a + 3] = forces[3 * at:3 * at + 3]
        yy[n_energy + n_force:] = stresses
        self.y = np.concatenate([self.y, yy])
        nv = np.zeros(nl)
        nv[:n_energy] = 1 / (self.energy_noise ** 2 * rel_e_noise ** 2)
        nv[n_energy:n_energy + n_force] = 1 / (self.force_noise ** 2 *
                                               rel_f_noise ** 2)
        nv[n_energy + n_force:] = 1 / (self.stress_noise ** 2 * rel_s_noise ** 2)
        self.noise_vector = np.concatenate([self.noise_vector, nv])
        ones = [np.zeros(nl) for _ in range(3)]
        ones[0][:n_energy] = 1 / (rel_e_noise * rel_e_noise)
        ones[1][n_energy:n_energy + n_force] = 1 / (rel_f_noise * rel_f_noise)
        ones[2][n_energy + n_force:] = 1 / (rel_s_noise * rel_s_noise)
        self.e_noise_one = np.concatenate([self.e_noise_one, ones[0]])
        self.f_noise_one = np.concatenate([self.f_noise_one, ones[1]])
        self.s_noise_one = np.concatenate([self.s_noise_one, ones[2]])
        for i, k in enumerate(self.kernels):
            n_sparse = self.sparse_descriptors[i].n_clusters
            blk = np.zeros((n_sparse, nl))
            if n_sparse:
                esk = envs_struc_gpu(self.sparse_descriptors[i], structure,
                                     k.sigma, k.power, i)
                blk[:, :n_energy] = esk[:, :n_energy]
                blk[:, n_energy + n_force:] = \
                    esk[:, 1 + 3 * n_atoms:1 + 3 * n_atoms + n_stress]
                if n_force:
                    ats = np.asarray(atoms, np.int64)
                    cols = (1 + 3 * ats[:, None] +
                            np.arange(3)[None, :]).reshape(-1)
                    blk[:, n_energy:n_energy + cols.size] = esk[:, cols]
            old = self.Kuf_kernels[i]
            if old.shape != (n_sparse, self.n_labels):
                old = np.zeros((n_sparse, self.n_labels))
            self.Kuf_kernels[i] = np.hstack([old, blk])
        self.n_energy_labels += n_energy
        self.n_force_labels += n_force
        self.n_stress_labels += n_stress
        self.n_labels += nl
        self.training_structures.append(structure)
        self.n_strucs += 1
        self._stack_Kuf()

    def _add_clusters(self, structure, clusters_by_kernel):
        clusters = [ClusterDescriptor.from_values(structure.descriptors[i],
                                                  clusters_by_kernel[i])
                    for i in range(self.n_kernels)]
        self._update_Kuu(clusters)
        self._update_Kuf(clusters)
        self._stack_Kuu()
        self._stack_Kuf()
        for i in range(self.n_kernels):
            self.sparse_descriptors[i].add_clusters_by_type(
                structure.descriptors[i], clusters_by_kernel[i])
        self.alpha = None
        self._model = None

    def _specific_by_kernel(self, structure, atoms):
        """Per kernel and species, the cluster indices of ``atoms``
        (sparse_gp.cpp:148-168); records them in sparse_indices."""
        atoms = [int(a) for a in atoms]
        by_kernel = []
        for i in range(self.n_kernels):
            self.sparse_indices[i].append(atoms)
            dv = structure.descriptors[i]
            by_type = []
            for j in range(dv.n_types):
                ind = []
                for kk in range(dv.n_clusters_by_type[j]):
                    a1 = int(dv.atom_indices[j][kk])
                    ind.extend(kk for a2 in atoms if a1 == a2)
                by_type.append(ind)
            by_kernel.append(by_type)
        return by_kernel

    def add_specific_environments(self, structure, atoms):
        """sparse_gp.cpp:141-189."""
        self.initialize_sparse_descriptors(structure)
        self._add_clusters(structure,
                           self._specific_by_kernel(structure, atoms))

    def add_environments_batch(self, items):
        """``add_specific_environments`` for several ``(structure, atoms)``
        at once: the same Kuu, Kuf and sparse set as the calls in sequence,
        with the new rows computed in one pass over the training structures
        (one envs_struc per training structure instead of one per call)."""
        items = [(s, a) for s, a in items if len(a)]
        if not items:
            return
        for s, _ in items:
            self.initialize_sparse_descriptors(s)
        picks = [self._specific_by_kernel(s, a) for s, a in items]
        clusters = []
        for i in range(self.n_kernels):
            dv0 = items[0][0].descriptors[i]
            cd = ClusterDescriptor(dv0.n_types, dv0.n_descriptors)
            for (s, _), bk in zip(items, picks):
                cd.add_clusters_by_type(s.descriptors[i], bk[i])
            clusters.append(cd)
        self._update_Kuu(clusters)
        self._update_Kuf(clusters)
        self._stack_Kuu()
        self._stack_Kuf()
        for i in range(self.n_kernels):
            for (s, _), bk in zip(items, picks):
                self.sparse_descriptors[i].add_clusters_by_type(
                    s.descriptors[i], bk[i])
        self.alpha = None
        self._model = None

    def add_all_environments(self, structure):
        """sparse_gp.cpp:307-341."""
        self.initialize_sparse_descriptors(structure)
        by_kernel = [[list(range(dv.n_clusters_by_type[s]))
                      for s in range(dv.n_types)]
                     for dv in structure.descriptors[:self.n_kernels]]
        self._add_clusters(structure, by_kernel)
        for i in range(self.n_kernels):
            self.sparse_indices[i].append(list(range(structure.noa)))

    def _clusters_to_atoms(self, dv, clusters):
        out = []
        for c in clusters:
            for j in range(dv.n_types):
                if dv.cumulative_type_count[j] <= c < dv.cumulative_type_count[j + 1]:
                    out.append(int(dv.atom_indices[j][c - dv.cumulative_type_count[j]]))
                    break
        return out

    def _by_type(self, dv, clusters):
        by_type = [[] for _ in range(dv.n_types)]
        for c in clusters:
            for j in range(dv.n_types):
                if dv.cumulative_type_count[j] <= c < dv.cumulative_type_count[j + 1]:
                    by_type[j].append(c - dv.cumulative_type_count[j])
                    break
        return by_type

    def add_random_environments(self, structure, n_added, seed=None):
        """sparse_gp.cpp:256-305 (the reference shuffles with an unseeded
        std::random_shuffle; here a numpy generator, seedable)."""
        self.initialize_sparse_descriptors(structure)
        r = np.random.Generator(np.random.PCG64(seed))
        by_kernel, picked = [], []
        for i in range(self.n_kernels):
            dv = structure.descriptors[i]
            order = r.permutation(dv.n_clusters)
            chosen = order[:min(int(n_added[i]), dv.n_clusters)].tolist()
            picked.append(chosen)
            by_kernel.append(self._by_type(dv, chosen))
        self._add_clusters(structure, by_kernel)
        for i in range(self.n_kernels):
            self.sparse_indices[i].append(
                self._clusters_to_atoms(structure.descriptors[i], picked[i]))

    def add_uncertain_environments(self, structure, n_added):
        """sparse_gp.cpp:191-254: the n_added clusters of largest local
        variance (stable sort, descending)."""
        if len(n_added) != self.n_kernels:
            raise RuntimeError(
                "n_added must have the same size as the number of kernels")
        self.initialize_sparse_descriptors(structure)
        variances = self.compute_cluster_uncertainties(structure)
        by_kernel, picked = [], []
        for i in range(self.n_kernels):
            v = np.asarray(variances[i])
            order = sorted(range(len(v)), key=lambda q: -v[q])
            chosen = order[:min(int(n_added[i]), len(order))]
            picked.append(chosen)
            by_kernel.append(self._by_type(structure.descriptors[i], chosen))
        self._add_clusters(structure, by_kernel)
        for i in range(self.n_kernels):
            self.sparse_indices[i].append(
                self._clusters_to_atoms(structure.descriptors[i], picked[i]))

    def _update_Kuu(self, clusters):
        """sparse_gp.cpp:343-400 (type-blocked growth of Kuu)."""
        for i, k in enumerate(self.kernels):
            sd, cd = self.sparse_descriptors[i], clusters[i]
            prev = k.envs_envs(sd, cd) if sd.n_clusters and cd.n_clusters else \
                np.zeros((sd.n_clusters, cd.n_clusters))
            selfb = k.envs_envs(cd, cd) if cd.n_clusters else np.zeros((0, 0))
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

    def _update_Kuf(self, clusters):
        """sparse_gp.cpp:402-472: new sparse rows against every training
        structure."""
        for i, k in enumerate(self.kernels):
            sd, cd = self.sparse_descriptors[i], clusters[i]
            ns, ne, nt = sd.n_clusters, cd.n_clusters, cd.n_types
            inds = [0]
            for j in range(nt):
                inds.append(inds[-1] + sd.n_clusters_by_type[j] +
                            cd.n_clusters_by_type[j])
            km = np.zeros((ns + ne, self.n_labels))
            old = self.Kuf_kernels[i]
            if old.shape != (ns, self.n_labels):
                old = np.zeros((ns, self.n_labels))
            for j, struc in enumerate(self.training_structures):
                n_atoms = struc.noa
                esk = envs_struc_gpu(cd, struc, k.sigma, k.power, i) if ne else \
                    np.zeros((0, 1 + 3 * n_atoms + 6))
                n1 = n2 = 0
                lc = self.label_count[j]
                ne_j = np.asarray(struc.energy).size
                nf_j = np.asarray(struc.forces).size
                ns_j = np.asarray(struc.stresses).size
                for kk in range(nt):
                    cc = 0
                    u = inds[kk]
                    n3, n4 = sd.n_clusters_by_type[kk], cd.n_clusters_by_type[kk]
                    if ne_j:
                        km[u:u + n3, lc] = old[n1:n1 + n3, lc]
                        km[u + n3:u + n3 + n4, lc] = esk[n2:n2 + n4, 0]
                        cc += 1
                    if nf_j:
                        ats = np.asarray(self.training_atom_indices[j],
                                         np.int64)
                        cols = (1 + 3 * ats[:, None] +
                                np.arange(3)[None, :]).reshape(-1)
                        w = cols.size
                        km[u:u + n3, lc + cc:lc + cc + w] = \
                            old[n1:n1 + n3, lc + cc:lc + cc + w]
                        km[u + n3:u + n3 + n4, lc + cc:lc + cc + w] = \
                            esk[n2:n2 + n4, cols]
                        cc += w
                    if ns_j:
                        km[u:u + n3, lc + cc:lc + cc + 6] = \
                            old[n1:n1 + n3, lc + cc:lc + cc + 6]
                        km[u + n3:u + n3 + n4, lc + cc:lc + cc + 6] = \
                            esk[n2:n2 + n4, 1 + 3 * n_atoms:1 + 3 * n_atoms + 6]
                    n1 += n3
                    n2 += n4
            self.Kuf_kernels[i] = km

    def _stack_Kuu(self):
        import scipy.linalg as sla
        self.Kuu = sla.block_diag(*self.Kuu_kernels)

    def _stack_Kuf(self):
        self.Kuf = np.vstack([k if k.shape[1] == self.n_labels else
                              np.zeros((k.shape[0], self.n_labels))
                              for k in self.Kuf_kernels])

    def set_hyperparameters(self, hyps):
        """sparse_gp.cpp:1163-1198: new kernel hyperparameters and noises.
        The NormalizedDotProduct kernel matrices scale by (sigma_new /
        sigma_old)^2 (Kuu_grad / Kuf_grad, normalized_dot_product.cpp:
        588-623); the noise vector is rebuilt from the per-label relative
        noises, then update_matrices_QR."""
        hyps = np.asarray(hyps, np.float64).reshape(-1)
        idx = 0
        for i, k in enumerate(self.kernels):
            n = len(k.kernel_hyperparameters)
            new = hyps[idx:idx + n]
            f = new[0] * new[0] / (k.sigma * k.sigma)
            self.Kuu_kernels[i] = self.Kuu_kernels[i] * f
            self.Kuf_kernels[i] = self.Kuf_kernels[i] * f
            k.sigma = float(new[0])
            idx += n
        self._stack_Kuu()
        self._stack_Kuf()
        self.energy_noise = float(hyps[idx])
        self.force_noise = float(hyps[idx + 1])
        self.stress_noise = float(hyps[idx + 2])
        self.noise_vector = (self.e_noise_one / self.energy_noise ** 2 +
                             self.f_noise_one / self.force_noise ** 2 +
                             self.s_noise_one / self.stress_noise ** 2)
        self.update_matrices_QR()

    def update_matrices_QR(self):
        """sparse_gp.cpp:607-641 on the GPU in FP64 (fgb_solve_qr)."""
        M = self.Kuu.shape[0]
        if M == 0:
            raise RuntimeError("no sparse environments")
        dev = _device()
        Kuu = torch.from_numpy(np.ascontiguousarray(self.Kuu)).to(dev)
        Kuf = torch.from_numpy(np.ascontiguousarray(self.Kuf)).to(dev)
        y = torch.from_numpy(np.ascontiguousarray(self.y)).to(dev)
        nv = torch.from_numpy(np.ascontiguousarray(self.noise_vector)).to(dev)
        alpha = torch.zeros(M, dtype=torch.float64, device=dev)
        Li = torch.zeros((M, M), dtype=torch.float64, device=dev)
        Ri = torch.zeros((M, M), dtype=torch.float64, device=dev)
        check(lib().fgb_solve_qr(M, int(self.n_labels), ptr(Kuu), ptr(Kuf),
                                 ptr(y), ptr(nv), float(self.Kuu_jitter),
                                 ptr(alpha), ptr(Li), ptr(Ri), stream_ptr()),
              "update_matrices_QR")
        self.alpha = alpha.cpu().numpy()
        self.L_inv = Li.cpu().numpy()
        self.R_inv = Ri.cpu().numpy()
        # Kuu_inverse = L_inv^T L_inv and Sigma = R_inv R_inv^T
        # (sparse_gp.cpp:619, 640) are formed on the GPU when first read
        self._Kuu_inverse = None
        self._Sigma = None
        self._model = None

    def _solve_product(self, which):
        dev = _device()
        src = self.L_inv if which == "Kuu_inverse" else self.R_inv
        Li = torch.from_numpy(np.ascontiguousarray(src, np.float64)).to(dev)
        Ri = Li
        M = Li.shape[0]
        out = torch.empty((M, M), dtype=torch.float64, device=dev)
        check(lib().fgb_solve_products(
            M, ptr(Li), ptr(Ri), ptr(out) if which == "Kuu_inverse" else None,
            ptr(out) if which == "Sigma" else None, stream_ptr()),
            which)
        return out.cpu().numpy()

    @property
    def Kuu_inverse(self):
        """L_inv^T L_inv (sparse_gp.cpp:619), formed on the GPU at FP64
        level when first read after a solve."""
        if self._Kuu_inverse is None and self.L_inv is not None:
            self._Kuu_inverse = self._solve_product("Kuu_inverse")
        return self._Kuu_inverse

    @Kuu_inverse.setter
    def Kuu_inverse(self, v):
        self._Kuu_inverse = v

    @property
    def Sigma(self):
        """R_inv R_inv^T (sparse_gp.cpp:640), formed on the GPU at FP64
        level when first read after a solve."""
        if self._Sigma is None and self.R_inv is not None:
            self._Sigma = self._solve_product("Sigma")
        return self._Sigma

    @Sigma.setter
    def Sigma(self, v):
        self._Sigma = v


# -------------------------------------------------------------- model
class _Model:
    """Owner of an fgb_model_t (device-resident sparse set, alpha, L_inv)."""

    def __init__(self, b2, sigma, power):
        h = ctypes.c_void_p()
        check(lib().fgb_model_create(ctypes.byref(h), b2.handle, float(sigma),
                                     float(power)), "SparseGP")
        self.h = h
        self.b2 = b2

    def set(self, counts, desc, alpha=None, L_inv=None):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        desc = np.ascontiguousarray(desc, dtype=np.float64)
        a = None if alpha is None else np.ascontiguousarray(alpha, np.float64)
        L = None if L_inv is None else np.ascontiguousarray(L_inv, np.float64)
        check(lib().fgb_model_set(self.h, ptr(counts), ptr(desc), ptr(a),
                                  ptr(L)), "SparseGP")

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.fgb_model_destroy(self.h)
            self.h = None


def pack_structures(structures):
    """Packed batch inputs: atom offsets, cells, positions, species (host)."""
    offsets = np.zeros(len(structures) + 1, dtype=np.int32)
    for k, s in enumerate(structures):
        offsets[k + 1] = offsets[k] + s.noa
    cells = np.ascontiguousarray(np.stack([s.cell.reshape(-1)
                                           for s in structures]))
    pos = np.ascontiguousarray(np.concatenate([s.positions for s in structures]))
    sp = np.ascontiguousarray(np.concatenate(
        [np.asarray(s.species, np.int32) for s in structures]))
    return offsets, cells, pos, sp


class SparseGP(_Training):
    """SparseGP(kernels, energy_noise, force_noise, stress_noise) —
    src/flare_pp/bffs/sparse_gp.cpp:14-58.  Training bookkeeping (Kuu, Kuf,
    labels) mirrors sparse_gp.cpp:141-641 with the kernel blocks and the QR
    solve on the GPU in FP64; prediction runs the fused GPU pipeline."""

    def __init__(self, kernels=(), energy_noise=1.0, force_noise=1.0,
                 stress_noise=1.0):
        self.kernels = list(kernels)
        self.n_kernels = len(self.kernels)
        self.energy_noise = float(energy_noise)
        self.force_noise = float(force_noise)
        self.stress_noise = float(stress_noise)
        self.Kuu_jitter = 1e-8
        self.sparse_descriptors = []
        self.sparse_indices = []
        self.training_structures = []
        self._init_training()
        self.alpha = None
        self.L_inv = None
        self.R_inv = None
        self._Sigma = None
        self._Kuu_inverse = None
        self._model = None
        self._model_key = None

    @property
    def hyperparameters(self):
        return np.concatenate([k.kernel_hyperparameters for k in self.kernels] +
                              [np.array([self.energy_noise, self.force_noise,
                                         self.stress_noise])])

    # -------------------------------------------------- device model
    def set_weights(self, sparse_descriptors, alpha, L_inv, calculators):
        """Install solved weights (alpha, L_inv) and the sparse set
        (list of ClusterDescriptor, one per kernel)."""
        self.sparse_descriptors = list(sparse_descriptors)
        self.alpha = np.asarray(alpha, np.float64)
        self.L_inv = np.asarray(L_inv, np.float64)
        self._Kuu_inverse = None
        self._Sigma = None
        self._calculators = list(calculators)
        self._model = None

    def _kernel_blocks(self):
        """(first row, rows) of each kernel's sparse set in alpha and L_inv
        (sparse_gp.cpp:94-139, 643-665: kernels are stacked in order)."""
        out, c = [], 0
        for cd in self.sparse_descriptors[:self.n_kernels]:
            n = int(np.sum(cd.n_clusters_by_type))
            out.append((c, n))
            c += n
        return out

    def _device_models(self, structure_calcs=None):
        """One device model per kernel: its descriptor calculator, sparse
        set, alpha segment and L_inv diagonal block.  The mean is the sum
        of the kernels' terms and each kernel's local variance uses its own
        diagonal block, exactly as predict_mean and
        compute_cluster_uncertainties do (sparse_gp.cpp:94-139, 643-665)."""
        if self.alpha is None or self.L_inv is None:
            raise RuntimeError(
                "L_inv must be up to date to make predictions. Please call "
                "update_matrices_QR and try again.")
        if self._model is None:
            calcs = list(structure_calcs or self._calculators)
            if len(calcs) < self.n_kernels:
                raise ValueError("a structure needs one descriptor calculator "
                                 "per kernel")
            models = []
            for i, ((c0, n), k) in enumerate(zip(self._kernel_blocks(),
                                                 self.kernels)):
                m = _Model(calcs[i], k.sigma, k.power)
                counts, desc = self.sparse_descriptors[i].stacked()
                m.set(counts, desc, self.alpha[c0:c0 + n],
                      self.L_inv[c0:c0 + n, c0:c0 + n])
                if self.R_inv is not None and self.n_kernels == 1:
                    R = np.ascontiguousarray(self.R_inv[:n, :n], np.float64)
                    check(lib().fgb_model_set_R_inv(m.h, ptr(R)), "SparseGP")
                slices = getattr(self, "_slices", None)
                if slices:
                    check(lib().fgb_model_set_slices(m.h, *slices),
                          "set_slices")
                models.append(m)
            self._model = models
        return self._model

    def _device_model(self, structure_calcs=None):
        """The device model of a single-kernel SparseGP (the mapped,
        MD-ensemble, serving and autograd front-ends take one kernel)."""
        if self.n_kernels != 1:
            raise NotImplementedError(
                "this operation takes a single-kernel SparseGP; prediction "
                "(predict_mean / predict_local_uncertainties / predict_SOR / "
                "predict_DTC / predict_batch) takes any number of kernels")
        return self._device_models(structure_calcs)[0]

    def predict_batch(self, structures, want=0xF, precision=None,
                      stream=None):
        """Batched prediction on the GPU.  Returns dict of numpy arrays:
        energy [S], forces [N, 3], stress [S, 6] (flare order), local_var
        [N] (atom order; the first kernel's) and local_vars (one [N] array
        per kernel).  With several kernels each runs the fused pipeline on
        its own descriptor and the mean terms are summed."""
        if not structures:
            return {}
        calcs = structures[0].descriptor_calculators
        models = self._device_models(calcs)
        offsets, cells, pos, sp = pack_structures(structures)
        dev = _device()
        N = int(offsets[-1])
        S = len(structures)
        d_pos = torch.from_numpy(pos).to(dev)
        d_sp = torch.from_numpy(sp).to(dev)
        prec = _prec[precision or _default_precision[0]]
        cutoff = structures[0].cutoff
        for s in structures:
            if s.cutoff != cutoff:
                raise ValueError("a batch must share one structure cutoff")
        out = None
        local_vars = []
        for m in models:
            e = torch.zeros(S, dtype=torch.float64, device=dev)
            f = torch.zeros((max(N, 1), 3), dtype=torch.float64, device=dev)
            st = torch.zeros((S, 6), dtype=torch.float64, device=dev)
            v = torch.zeros(max(N, 1), dtype=torch.float64, device=dev)
            check(lib().fgb_predict(m.h, S, ptr(offsets), ptr(cells),
                                    ptr(d_pos), ptr(d_sp), cutoff, int(want),
                                    prec, ptr(e), ptr(f), ptr(st), ptr(v),
                                    stream_ptr(stream)),
                  "predict")
            if out is None:
                out = [e, f, st]
            else:
                out[0] += e
                out[1] += f
                out[2] += st
            local_vars.append(v)
        torch.cuda.current_stream().synchronize()
        lv = [v.cpu().numpy()[:N] for v in local_vars]
        return {"energy": out[0].cpu().numpy(),
                "forces": out[1].cpu().numpy()[:N],
                "stress": out[2].cpu().numpy(), "local_var": lv[0],
                "local_vars": lv, "offsets": offsets}

    def _predict_one(self, structure, want):
        r = self.predict_batch([structure], want)
        structure.mean_efs = np.concatenate(
            [r["energy"][:1], r["forces"].reshape(-1), r["stress"][0]])
        return r

    def predict_mean(self, structure):
        """sparse_gp.cpp:643-665: mean_efs = [E, F (3N), stress (6)]."""
        self._predict_one(structure, _lib.FGB_WANT_ENERGY |
                          _lib.FGB_WANT_FORCES | _lib.FGB_WANT_STRESS)

    def predict_local_uncertainties(self, structure):
        """sparse_gp.cpp:731-757: mean_efs plus per-atom local variances,
        one array per kernel (each stored in its descriptor's
        species-sorted order, as the reference does)."""
        r = self._predict_one(structure, 0xF)
        sp = np.asarray(structure.species)
        out = []
        for i, v in enumerate(r["local_vars"]):
            S = structure.descriptor_calculators[i].descriptor_settings[0]
            order = np.concatenate([np.nonzero(sp == s)[0] for s in range(S)])
            out.append(v[order])
        structure.local_uncertainties = out

    def _stacked_kernel_matrix(self, structure):
        """The kernels' envs_struc blocks stacked in kernel order on the
        device, [n_sparse x (1 + 3N + 6)] (sparse_gp.cpp:667-692)."""
        blocks = []
        for i, k in enumerate(self.kernels):
            blocks.append(_envs_struc_device(self.sparse_descriptors[i],
                                             structure, k.sigma, k.power, i))
        return torch.cat(blocks, 0)

    def _check_solved(self):
        if self.R_inv is None:
            raise RuntimeError(
                "L_inv must be up to date to make predictions. Please call "
                "update_matrices_QR and try again.")

    def predict_SOR(self, structure):
        """sparse_gp.cpp:667-692: mean_efs and the SOR variances
        diag(K^T R_inv R_inv^T K) over all 1 + 3N + 6 outputs (FP64).  One
        kernel: the fused fgb_predict_sor.  Several: K stacked over the
        kernels (each block from the GPU envs_struc), then K^T alpha and
        the rows of K^T R_inv as plain FP64 GEMMs (cuBLAS)."""
        self._check_solved()
        if self.n_kernels != 1:
            K = self._stacked_kernel_matrix(structure)
            alpha = torch.from_numpy(np.asarray(self.alpha)).to(K.device)
            Ri = torch.from_numpy(np.ascontiguousarray(self.R_inv)).to(K.device)
            vs = K.T @ Ri
            structure.mean_efs = (K.T @ alpha).cpu().numpy()
            structure.variance_efs = (vs * vs).sum(1).cpu().numpy()
            return
        m = self._device_model(structure.descriptor_calculators)
        dev = _device()
        n_out = 1 + 3 * structure.noa + 6
        mean = torch.zeros(n_out, dtype=torch.float64, device=dev)
        var = torch.zeros(n_out, dtype=torch.float64, device=dev)
        d = structure._inputs()
        check(lib().fgb_predict_sor(m.h, structure.nlist().h, ptr(d["species"]),
                                    ptr(mean), ptr(var), stream_ptr()),
              "predict_SOR")
        structure.mean_efs = mean.cpu().numpy()
        structure.variance_efs = var.cpu().numpy()

    def predict_DTC(self, structure):
        """sparse_gp.cpp:694-729: mean_efs and the DTC variances K_self -
        diag(K^T Kuu^-1 K) + diag(K^T Sigma K) over all 1 + 3N + 6 outputs
        (FP64; K_self is NormalizedDotProduct::self_kernel_struc, summed
        over the kernels).  Several kernels: K stacked as in predict_SOR,
        diag(K^T Kuu^-1 K) = |L_inv K|^2 and diag(K^T Sigma K) = |R_inv^T
        K|^2 per column."""
        self._check_solved()
        if self.n_kernels != 1:
            K = self._stacked_kernel_matrix(structure)
            dev = K.device
            alpha = torch.from_numpy(np.asarray(self.alpha)).to(dev)
            Li = torch.from_numpy(np.ascontiguousarray(self.L_inv)).to(dev)
            Ri = torch.from_numpy(np.ascontiguousarray(self.R_inv)).to(dev)
            kself = sum(torch.from_numpy(k.self_kernel_struc(structure,
                                                             kernel_index=i))
                        for i, k in enumerate(self.kernels)).to(dev)
            q = Li @ K
            v = Ri.T @ K
            structure.mean_efs = (K.T @ alpha).cpu().numpy()
            structure.variance_efs = (kself - (q * q).sum(0) +
                                      (v * v).sum(0)).cpu().numpy()
            return
        m = self._device_model(structure.descriptor_calculators)
        dev = _device()
        n_out = 1 + 3 * structure.noa + 6
        mean = torch.zeros(n_out, dtype=torch.float64, device=dev)
        var = torch.zeros(n_out, dtype=torch.float64, device=dev)
        d = structure._inputs()
        check(lib().fgb_predict_dtc(m.h, structure.nlist().h, ptr(d["species"]),
                                    ptr(mean), ptr(var), stream_ptr()),
              "predict_DTC")
        structure.mean_efs = mean.cpu().numpy()
        structure.variance_efs = var.cpu().numpy()

    def mixed_plan(self, kernel_index=0):
        """The mixed path's precision plan for one kernel of this model:
        slices of the kernel GEMM (9, 8 or 7) and of the variance GEMM (9,
        8, 7 or 6) with the largest energy (eV/atom) and local-variance
        differences to 9 slices measured on the sparse set when they were
        chosen, and the fold guard (largest folded coefficient, whether the
        descriptor and forces run at FP64 level)."""
        m = self._device_models()[kernel_index]
        S, Sv, fp64 = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        est, vest = ctypes.c_double(0.0), ctypes.c_double(0.0)
        fmax = ctypes.c_double(0.0)
        check(lib().fgb_model_mixed_plan(m.h, None, None, ctypes.byref(fmax),
                                         ctypes.byref(fp64), stream_ptr()),
              "mixed_plan")
        check(lib().fgb_model_slice_plan(m.h, ctypes.byref(S),
                                         ctypes.byref(Sv), ctypes.byref(est),
                                         ctypes.byref(vest), stream_ptr()),
              "mixed_plan")
        return {"kernel_slices": S.value, "variance_slices": Sv.value,
                "slice_err_ev_per_atom": est.value,
                "variance_slice_err": vest.value,
                "fold_max": fmax.value, "fp64_forces": bool(fp64.value)}

    def set_slices(self, kernel=0, variance=0):
        """Force the mixed path's slice counts (kernel GEMM 7-9, variance
        GEMM 6-9; 0 = the fewest the model's error probes allow)."""
        self._slices = (int(kernel), int(variance))
        for m in self._model or []:
            check(lib().fgb_model_set_slices(m.h, *self._slices),
                  "set_slices")

    # -------------------------------------------------- mapped models
    def write_mapping_coefficients(self, file_name, contributor,
                                   kernel_index=0):
        """lmp.flare coefficients (sparse_gp.cpp:1199-1264); flare_gb300.mapped."""
        from . import mapped
        return mapped.write_mapping_coefficients(self, file_name, contributor,
                                                 kernel_index)

    def write_varmap_coefficients(self, file_name, contributor,
                                  kernel_index=0):
        """Power-1 variance map (sparse_gp.cpp:1266-1335)."""
        from . import mapped
        return mapped.write_varmap_coefficients(self, file_name, contributor,
                                                kernel_index)

    def write_L_inverse(self, file_name, contributor):
        """L_inv blocks for compute flare/std/atom (sparse_gp.cpp:1337-1391)."""
        from . import mapped
        mapped.write_L_inverse(self, file_name, contributor)

    def write_sparse_descriptors(self, file_name, contributor):
        """Sparse descriptors for compute flare/std/atom (sparse_gp.cpp:1393-1466)."""
        from . import mapped
        mapped.write_sparse_descriptors(self, file_name, contributor)

    def compute_cluster_uncertainties(self, structure):
        """sparse_gp.cpp:94-139 (species-sorted variances)."""
        r = self.predict_batch([structure], _lib.FGB_WANT_LOCAL_VAR)
        sp = np.asarray(structure.species)
        out = []
        for i, v in enumerate(r["local_vars"]):
            S = structure.descriptor_calculators[i].descriptor_settings[0]
            order = np.concatenate([np.nonzero(sp == s)[0] for s in range(S)])
            out.append(v[order])
        return out
