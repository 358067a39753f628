"""SGP_Calculator: the reference's ASE calculator
(flare/bffs/sgp/calculator.py:16-206) on the GPU SparseGP.

``calculate(atoms)`` accepts an ASE ``Atoms`` or any object with ``numbers``,
``cell`` and ``positions``; ASE's ``Calculator`` is used as the base class
when it is installed, a minimal stand-in otherwise.  Results match the
reference's post-processing: energy plus single-atom energies, forces,
stress in ASE order -[xx, yy, zz, yz, xz, xy], and ``stds`` (per force
component for SOR, per atom in column 0 — divided by |sigma| — for "local").
"""
import json
from copy import deepcopy

import numpy as np

from .core import Structure
from .sparse_gp import SGP_Wrapper, _NumpyEncoder

try:  # pragma: no cover - ASE is optional
    from ase.calculators.calculator import Calculator, all_changes
except Exception:  # noqa: BLE001
    all_changes = ["positions", "numbers", "cell", "pbc"]

    class Calculator:
        """Minimal stand-in for ase.calculators.calculator.Calculator."""

        implemented_properties = []

        def __init__(self, **kwargs):
            self.results = {}
            self.atoms = None

        def calculate(self, atoms=None, properties=None,
                      system_changes=all_changes):
            if atoms is not None:
                self.atoms = atoms

        def get_property(self, name, atoms=None, allow_calculation=True):
            self.calculate(atoms)
            return self.results[name]

        def get_potential_energy(self, atoms=None):
            return self.get_property("energy", atoms)

        def get_forces(self, atoms=None):
            return self.get_property("forces", atoms)

        def get_stress(self, atoms=None):
            return self.get_property("stress", atoms)


def sort_variances(structure, variances):
    """calculator.py:188-206: species-sorted variances back to atom order."""
    assert len(variances) == structure.noa
    out = np.zeros(len(variances))
    dv = structure.descriptors[0]
    v = 0
    for s in range(dv.n_types):
        for a in dv.atom_indices[s]:
            out[a] = variances[v]
            v += 1
    return out


def _signed_sqrt(v):
    v = np.asarray(v, np.float64)
    return np.where(v > 0, np.sqrt(np.abs(v)), -np.sqrt(np.abs(v)))


class SGP_Calculator(Calculator):
    implemented_properties = ["energy", "forces", "stress", "stds"]

    def __init__(self, sgp_model, use_mapping=False):
        super().__init__()
        self.gp_model = sgp_model
        self.results = {}
        self.use_mapping = use_mapping
        self.mgp_model = None

    def calculate(self, atoms=None, properties=None,
                  system_changes=all_changes):
        super().calculate(atoms=atoms, properties=properties,
                          system_changes=system_changes)
        coded = [self.gp_model.species_map[int(z)] for z in atoms.numbers]
        structure = Structure(np.asarray(atoms.cell, np.float64), coded,
                              np.asarray(atoms.positions, np.float64),
                              self.gp_model.cutoff,
                              self.gp_model.descriptor_calculators)
        self.predict_on_structure(structure)

    def predict_on_structure(self, structure):
        vt = self.gp_model.variance_type
        sgp = self.gp_model.sparse_gp
        if vt == "SOR":
            sgp.predict_SOR(structure)
        elif vt == "DTC":
            sgp.predict_DTC(structure)
        elif vt == "local":
            sgp.predict_local_uncertainties(structure)
        m = structure.mean_efs
        self.results["energy"] = deepcopy(m[0])
        self.results["forces"] = deepcopy(m[1:-6].reshape(-1, 3))
        if self.gp_model.single_atom_energies is not None:
            for spec in structure.species:
                self.results["energy"] += self.gp_model.single_atom_energies[spec]
        fs = m[-6:]
        self.results["stress"] = -np.array([fs[0], fs[3], fs[5], fs[4], fs[2],
                                            fs[1]])
        if vt in ("SOR", "DTC"):
            self.results["stds"] = _signed_sqrt(
                structure.variance_efs[1:-6]).reshape(-1, 3)
        elif vt == "local":
            v = sort_variances(structure, structure.local_uncertainties[0])
            full = np.zeros((len(v), 3))
            full[:, 0] = _signed_sqrt(v) / np.abs(self.gp_model.hyps[0])
            self.results["stds"] = full

    def build_map(self, filename="lmp.flare", contributor="user",
                  map_uncertainty=False):
        """calculator.py:169-185: the LAMMPS potential file and the files of
        its uncertainty compute (variance map, or L_inv and sparse
        descriptors)."""
        self.gp_model.sparse_gp.write_mapping_coefficients(filename,
                                                           contributor, 0)
        if map_uncertainty:
            self.gp_model.write_varmap_coefficients(f"map_unc_{filename}",
                                                    contributor, 0)
        else:
            self.gp_model.sparse_gp.write_L_inverse(f"L_inv_{filename}",
                                                    contributor)
            self.gp_model.sparse_gp.write_sparse_descriptors(
                f"sparse_desc_{filename}", contributor)

    def get_uncertainties(self, atoms):
        return self.get_property("stds", atoms)

    def calculation_required(self, atoms, quantities):
        return True

    def as_dict(self):
        return {"class": self.__class__.__name__,
                "gp_model": self.gp_model.as_dict(),
                "use_mapping": self.use_mapping,
                "results": self.results}

    @staticmethod
    def from_dict(dct):
        sgp, _ = SGP_Wrapper.from_dict(dct["gp_model"])
        calc = SGP_Calculator(sgp, use_mapping=dct["use_mapping"])
        calc.results = dct.get("results", {})
        return calc

    def write_model(self, name):
        if not name.endswith(".json"):
            name += ".json"
        with open(name, "w") as f:
            json.dump(self.as_dict(), f, cls=_NumpyEncoder)

    @staticmethod
    def from_file(name):
        with open(name) as f:
            d = json.loads(f.readline())
        sgp, kernels = SGP_Wrapper.from_dict(d["gp_model"])
        return SGP_Calculator(sgp, use_mapping=d["use_mapping"]), kernels
