"""SGP_Wrapper: the reference's Python model wrapper
(flare/bffs/sgp/sparse_gp.py:17-420) over the GPU SparseGP.

Same constructor, properties, ``update_db`` modes and JSON round trip
(``as_dict``/``from_dict``/``write_model``/``from_file``: the model is
rebuilt by replaying ``update_db`` on the stored training structures, then
``update_matrices_QR``).  Training structures are written in the layout
the reference writes them in: ASE's ``Atoms.todict()`` (numbers, positions,
cell, pbc, info with rel_efs_noise) with the labels under ``results``
(energy as a list of zero or one totals, forces N x 3, stress as six values
or an empty list), which ``FLARE_Atoms.from_dict`` reads
(flare/atoms.py:162-183, flare/bffs/sgp/sparse_gp.py:190-211, 273-309).
ASE itself is optional here: the records are plain dicts.  Hyperparameter
optimisation (``train``) is outside the prediction path and raises
NotImplementedError.
"""
import json
import warnings

import numpy as np

from .core import B2, NormalizedDotProduct, SparseGP, Structure


class _NumpyEncoder(json.JSONEncoder):
    def default(self, o):
        if isinstance(o, np.ndarray):
            return o.tolist()
        if isinstance(o, (np.integer,)):
            return int(o)
        if isinstance(o, (np.floating,)):
            return float(o)
        return super().default(o)


class SGP_Wrapper:
    def __init__(self, kernels, descriptor_calculators, cutoff, sigma_e,
                 sigma_f, sigma_s, species_map, variance_type="SOR",
                 single_atom_energies=None, energy_training=True,
                 force_training=True, stress_training=True, max_iterations=10,
                 opt_method="BFGS", bounds=None):
        self.sparse_gp = SparseGP(kernels, sigma_e, sigma_f, sigma_s)
        self.descriptor_calculators = descriptor_calculators
        self.cutoff = cutoff
        self.hyps_mask = None
        self.species_map = species_map
        self.variance_type = variance_type
        self.single_atom_energies = single_atom_energies
        self.energy_training = energy_training
        self.force_training = force_training
        self.stress_training = stress_training
        self.max_iterations = max_iterations
        self.opt_method = opt_method
        self.bounds = bounds
        self.atom_indices = []
        self.rel_efs_noise = []
        self.hyp_labels = ["Hyp" + str(n) for n in range(len(self.hyps))]
        self._training_dicts = []

    @property
    def training_data(self):
        return self.sparse_gp.training_structures

    @property
    def hyps(self):
        return self.sparse_gp.hyperparameters

    @property
    def hyps_and_labels(self):
        return self.hyps, self.hyp_labels

    @property
    def force_noise(self):
        return self.sparse_gp.force_noise

    def __len__(self):
        return len(self.training_data)

    def check_L_alpha(self):
        pass

    def set_L_alpha(self):
        pass

    def train(self, logger_name=None):
        raise NotImplementedError(
            "hyperparameter optimisation (likelihood and its gradient, "
            "sparse_gp.cpp:759-1161) is not part of the GPU prediction path")

    # sparse_gp.py:321-415
    def update_db(self, structure, forces, custom_range=(), energy=None,
                  stress=None, mode="specific", sgp=None, update_qr=True,
                  atom_indices=(-1,), rel_e_noise=1, rel_f_noise=1,
                  rel_s_noise=1):
        numbers = getattr(structure, "numbers", None)
        if numbers is not None and not isinstance(structure, Structure):
            coded = [self.species_map[int(z)] for z in numbers]
        else:
            coded = list(structure.species)
        cell = np.asarray(structure.cell, np.float64)
        positions = np.asarray(structure.positions, np.float64)
        desc = Structure(cell, coded, positions, self.cutoff,
                         self.descriptor_calculators)
        if energy is not None and self.energy_training:
            sae = 0.0
            if self.single_atom_energies is not None:
                sae = sum(self.single_atom_energies[s] for s in coded)
            desc.energy = np.array([[energy - sae]])
        if forces is not None and self.force_training:
            desc.forces = np.asarray(forces, np.float64).reshape(-1)
        if stress is not None and self.stress_training:
            st = np.asarray(stress, dtype=object)
            if st.ndim > 0 and st.size and all(v is not None for v in st.ravel()):
                desc.stresses = np.asarray(stress, np.float64).reshape(-1)
        if sgp is None:
            sgp = self.sparse_gp
            self.atom_indices.append(list(np.asarray(atom_indices).reshape(-1)))
        sgp.add_training_structure(desc, atom_indices, rel_e_noise,
                                   rel_f_noise, rel_s_noise)
        self.rel_efs_noise.append([rel_e_noise, rel_f_noise, rel_s_noise])
        self._training_dicts.append({
            "cell": cell, "numbers": self._numbers(coded), "positions": positions,
            "energy": None if energy is None else float(energy),
            "forces": None if forces is None else np.asarray(forces).reshape(-1, 3),
            "stress": None if stress is None else np.asarray(stress, dtype=object),
            "rel_efs_noise": [rel_e_noise, rel_f_noise, rel_s_noise]})
        if mode == "all":
            if not custom_range:
                sgp.add_all_environments(desc)
            else:
                raise Exception("Set mode='specific' for a user-defined custom_range")
        elif mode == "uncertain":
            if len(custom_range) == 1:
                sgp.add_uncertain_environments(desc, custom_range)
            else:
                raise Exception("The custom_range should be set as [n_added] "
                                "if mode='uncertain'")
        elif mode == "specific":
            if len(custom_range) == 0:
                warnings.warn("The mode='specific' but no custom_range is "
                              "given, will not add sparse envs")
            else:
                sgp.add_specific_environments(desc, custom_range)
        elif mode == "random":
            if len(custom_range) == 1:
                sgp.add_random_environments(desc, custom_range)
            else:
                raise Exception("The custom_range should be set as [n_added] "
                                "if mode='random'")
        else:
            raise NotImplementedError
        if update_qr:
            sgp.update_matrices_QR()

    def write_mapping_coefficients(self, filename, contributor, kernel_idx):
        """flare/bffs/sgp/sparse_gp.py:429-430."""
        self.sparse_gp.write_mapping_coefficients(filename, contributor,
                                                  kernel_idx)

    def write_varmap_coefficients(self, filename, contributor, kernel_idx):
        """flare/bffs/sgp/sparse_gp.py:432-495: the variance map of the
        power-1 model with this sparse set, sigma and jitter (which is all
        it depends on; the reference rebuilds and retrains that model)."""
        assert len(self.sparse_gp.kernels) == 1 and kernel_idx == 0, \
            "Not support multiple kernels"
        return self.sparse_gp.write_varmap_coefficients(filename, contributor,
                                                        kernel_idx)

    def _numbers(self, coded):
        inv = {v: k for k, v in self.species_map.items()}
        return [int(inv[s]) for s in coded]

    # sparse_gp.py:136-213
    def as_dict(self):
        out = {}
        skip = {"sparse_gp", "descriptor_calculators", "_training_dicts"}
        for key, val in vars(self).items():
            if key not in skip:
                out[key] = val
        assert len(self.descriptor_calculators) == 1
        out["descriptor_calculators"] = [self.descriptor_calculators[0].as_dict()]
        out["hyps"], out["hyp_labels"] = self.hyps_and_labels
        out["Kuu_jitter"] = self.sparse_gp.Kuu_jitter
        out["kernels"] = [("NormalizedDotProduct", k.sigma, k.power)
                          for k in self.sparse_gp.kernels]
        out["training_structures"] = [
            _training_record(d, self.energy_training, self.stress_training)
            for d in self._training_dicts]
        out["sparse_indice"] = self.sparse_gp.sparse_indices
        return out

    # sparse_gp.py:215-313
    @staticmethod
    def from_dict(in_dict):
        kl = in_dict["kernels"]
        assert len(kl) == 1 and kl[0][0] == "NormalizedDotProduct"
        kernel = NormalizedDotProduct(float(kl[0][1]), int(kl[0][2]))
        bd = in_dict["descriptor_calculators"][0]
        assert bd["type"] == "B2"
        calc = B2(bd["radial_basis"], bd["cutoff_function"], bd["radial_hyps"],
                  bd["cutoff_hyps"], bd["descriptor_settings"], bd["cutoffs"])
        sae = in_dict.get("single_atom_energies")
        if sae is not None:
            sae = {int(k): v for k, v in sae.items()}
        species_map = {int(k): v for k, v in in_dict["species_map"].items()}
        gp = SGP_Wrapper([kernel], [calc], in_dict["cutoff"],
                         in_dict["hyps"][-3], in_dict["hyps"][-2],
                         in_dict["hyps"][-1], species_map,
                         variance_type=in_dict["variance_type"],
                         single_atom_energies=sae,
                         energy_training=in_dict["energy_training"],
                         force_training=in_dict["force_training"],
                         stress_training=in_dict["stress_training"],
                         max_iterations=in_dict["max_iterations"],
                         opt_method=in_dict["opt_method"],
                         bounds=in_dict["bounds"])
        gp.sparse_gp.Kuu_jitter = in_dict["Kuu_jitter"]
        for s, td in enumerate(in_dict["training_structures"]):
            custom_range = in_dict["sparse_indice"][0][s]
            atom_indices = in_dict["atom_indices"][s] if "atom_indices" in in_dict \
                else [-1]
            forces, energy, stress, rel = _read_training_record(td)
            if not in_dict["stress_training"]:
                stress = None
            gp.update_db(_Atoms(td), forces, custom_range=custom_range,
                         energy=energy, stress=stress, mode="specific",
                         sgp=None, update_qr=False, atom_indices=atom_indices,
                         rel_e_noise=rel[0], rel_f_noise=rel[1],
                         rel_s_noise=rel[2])
        gp.sparse_gp.update_matrices_QR()
        return gp, [kernel]

    def write_model(self, name):
        if not name.endswith(".json"):
            name += ".json"
        with open(name, "w") as f:
            json.dump(self.as_dict(), f, cls=_NumpyEncoder)

    @staticmethod
    def from_file(filename):
        with open(filename) as f:
            in_dict = json.loads(f.readline())
        return SGP_Wrapper.from_dict(in_dict)

    def __deepcopy__(self, memo):
        return SGP_Wrapper.from_dict(json.loads(json.dumps(
            self.as_dict(), cls=_NumpyEncoder)))[0]


def _training_record(d, energy_training, stress_training):
    """One training structure in the reference's file layout: ASE's
    ``Atoms.todict()`` plus ``results`` (sparse_gp.py:190-211).  The energy
    is the total as labelled (single-atom energies included); an energy or
    stress that is not trained on is written as an empty list, as the
    reference's empty label vectors are.  Structures given without forces
    carry an empty force list: the reference's reader passes it on as an
    empty label vector (``FLARE_Atoms.from_dict`` then ``update_db``,
    sparse_gp.py:273-309), so neither reader trains on force labels that
    were never given."""
    n = len(d["numbers"])
    energy = [] if d["energy"] is None or not energy_training \
        else [float(d["energy"])]
    stress = []
    if d["stress"] is not None and stress_training:
        st = [None if v is None else float(v) for v in np.ravel(d["stress"])]
        if st and all(v is not None for v in st):
            stress = st
    info = {"rel_efs_noise": [float(v) for v in d["rel_efs_noise"]]}
    if d["forces"] is None:
        forces = np.zeros((0,))
    else:
        forces = np.asarray(d["forces"], np.float64).reshape(n, 3)
    return {"numbers": [int(z) for z in d["numbers"]],
            "positions": np.asarray(d["positions"], np.float64).tolist(),
            "cell": np.asarray(d["cell"], np.float64).tolist(),
            "pbc": [True, True, True], "info": info,
            "results": {"energy": energy, "forces": forces.tolist(),
                        "stress": stress}}


def _read_training_record(td):
    """(forces, energy, stress, rel_efs_noise) of one stored training
    structure, as the reference's reader takes them (sparse_gp.py:273-309):
    labels from ``results`` (the reference's layout), or from the top level
    (the flat layout earlier versions of this package wrote)."""
    info = td.get("info") or {}
    rel = list(info.get("rel_efs_noise", [1, 1, 1]))
    if "results" in td:
        res = td["results"]
        e = res.get("energy")
        e = np.ravel(np.asarray([] if e is None else e, np.float64))
        energy = float(e[0]) if e.size else None
        forces = res.get("forces")
        # an empty list is the reference's empty force-label vector;
        # has_forces marks the zero-filled records older versions wrote
        if forces is not None and np.size(forces) == 0:
            forces = None
        if not info.get("has_forces", True):
            forces = None
        st = res.get("stress")
        stress = None if st is None or np.size(st) == 0 else st
    else:
        energy, forces, stress = td.get("energy"), td.get("forces"), \
            td.get("stress")
    return forces, energy, stress, rel


class _Atoms:
    """Minimal atoms record (cell, numbers, positions) used on reload."""

    def __init__(self, d):
        self.cell = np.asarray(d["cell"], np.float64)
        self.numbers = [int(z) for z in d["numbers"]]
        self.positions = np.asarray(d["positions"], np.float64)
