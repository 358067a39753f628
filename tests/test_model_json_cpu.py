"""CPU: the model file's training-structure records (SGP_Wrapper.as_dict /
from_dict, flare/bffs/sgp/sparse_gp.py:136-313).  Records are written in
the reference's layout — ASE's Atoms.todict() with the labels under
"results" (flare/atoms.py:64-79, 162-183) — and read back from that layout
and from the flat layout earlier versions of this package wrote."""
import json

import numpy as np

from flare_gb300.sparse_gp import (_Atoms, _NumpyEncoder, _read_training_record,
                                   _training_record)

CELL = np.diag([5.0, 6.0, 7.0])
POS = np.array([[0.1, 0.2, 0.3], [1.4, 2.5, 3.6], [4.0, 0.5, 6.1]])
FORCES = np.array([[0.5, -0.25, 1.0], [-1.5, 2.0, 0.125], [1.0, -1.75, -1.125]])


def _stored(**kw):
    d = {"cell": CELL, "numbers": [13, 29, 13], "positions": POS,
         "energy": -12.5, "forces": FORCES,
         "stress": np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6], dtype=object),
         "rel_efs_noise": [1, 0.5, 2]}
    d.update(kw)
    return d


def _through_json(rec):
    return json.loads(json.dumps(rec, cls=_NumpyEncoder))


def test_record_has_reference_layout():
    rec = _through_json(_training_record(_stored(), True, True))
    assert set(rec) == {"numbers", "positions", "cell", "pbc", "info", "results"}
    assert rec["results"]["energy"] == [-12.5]
    assert np.array_equal(rec["results"]["forces"], FORCES)
    assert rec["results"]["stress"] == [0.1, 0.2, 0.3, 0.4, 0.5, 0.6]
    assert rec["info"] == {"rel_efs_noise": [1.0, 0.5, 2.0]}
    assert rec["numbers"] == [13, 29, 13] and rec["pbc"] == [True] * 3


def test_record_round_trip():
    forces, energy, stress, rel = _read_training_record(
        _through_json(_training_record(_stored(), True, True)))
    assert energy == -12.5 and rel == [1.0, 0.5, 2.0]
    assert np.array_equal(forces, FORCES)
    assert np.array_equal(np.asarray(stress, np.float64),
                          [0.1, 0.2, 0.3, 0.4, 0.5, 0.6])
    a = _Atoms(_through_json(_training_record(_stored(), True, True)))
    assert np.array_equal(a.cell, CELL) and np.array_equal(a.positions, POS)
    assert a.numbers == [13, 29, 13]


def test_untrained_and_missing_labels():
    # energy / stress not trained on: written empty, read back as None
    rec = _through_json(_training_record(_stored(), False, False))
    assert rec["results"]["energy"] == [] and rec["results"]["stress"] == []
    forces, energy, stress, _ = _read_training_record(rec)
    assert energy is None and stress is None and np.array_equal(forces, FORCES)
    # no energy, no forces, a stress with missing components
    rec = _through_json(_training_record(
        _stored(energy=None, forces=None,
                stress=np.array([1.0, None, 2.0, 3.0, 4.0, 5.0], dtype=object)),
        True, True))
    # no fake labels: the force list is empty, and read the way the
    # reference reads it (np.array of the list, reshape(-1)) it gives no
    # force label at all
    assert rec["results"]["forces"] == []
    assert "has_forces" not in rec["info"]
    assert np.array(rec["results"]["forces"]).reshape(-1).size == 0
    forces, energy, stress, _ = _read_training_record(rec)
    assert forces is None and energy is None and stress is None
    # records older versions wrote: zero forces marked has_forces = False
    rec["results"]["forces"] = np.zeros((3, 3)).tolist()
    rec["info"]["has_forces"] = False
    forces, _, _, _ = _read_training_record(rec)
    assert forces is None


def test_reads_reference_written_record():
    # a record as FLARE_Atoms.as_dict writes it: label_setter's full results
    # dict, energy as a one-element list (struc.energy + single-atom sum)
    rec = {"numbers": [8, 1, 1], "positions": POS.tolist(),
           "cell": CELL.tolist(), "pbc": [True, True, True],
           "info": {"rel_efs_noise": [1, 1, 1]},
           "results": {"forces": FORCES.tolist(), "energy": [-3.25],
                       "stress": [], "stds": np.zeros((3, 3)).tolist(),
                       "local_energy_stds": [0, 0, 0],
                       "stress_stds": [0] * 6}}
    forces, energy, stress, rel = _read_training_record(rec)
    assert energy == -3.25 and stress is None and rel == [1, 1, 1]
    assert np.array_equal(forces, FORCES)
    # no info: the reference's default noise factors
    rec.pop("info")
    rec["results"]["energy"] = []
    _, energy, _, rel = _read_training_record(rec)
    assert energy is None and rel == [1, 1, 1]


def test_reads_flat_record():
    rec = {"cell": CELL.tolist(), "numbers": [13, 29, 13],
           "positions": POS.tolist(), "energy": -1.0,
           "forces": FORCES.tolist(), "stress": None,
           "info": {"rel_efs_noise": [2, 1, 1]}}
    forces, energy, stress, rel = _read_training_record(rec)
    assert energy == -1.0 and stress is None and rel == [2, 1, 1]
    assert np.array_equal(forces, FORCES)


def test_model_dict_has_every_key_the_reference_reads():
    """The keys SGP_Wrapper.from_dict reads (sparse_gp.py:215-313) are all
    written, and the dict survives JSON (an empty model: no GPU needed)."""
    import flare_gb300 as fg
    from flare_gb300.sparse_gp import SGP_Wrapper
    b2 = fg.B2("chebyshev", "quadratic", [0, 5], [], [2, 4, 3])
    w = SGP_Wrapper([fg.NormalizedDotProduct(2.0, 2)], [b2], 5.0, 0.01, 0.1,
                    0.001, {13: 0, 29: 1}, single_atom_energies={0: -1.5, 1: 2})
    d = json.loads(json.dumps(w.as_dict(), cls=_NumpyEncoder))
    for key in ("kernels", "descriptor_calculators", "single_atom_energies",
                "species_map", "cutoff", "hyps", "variance_type",
                "energy_training", "force_training", "stress_training",
                "max_iterations", "opt_method", "bounds", "Kuu_jitter",
                "training_structures", "sparse_indice"):
        assert key in d, key
    assert d["kernels"] == [["NormalizedDotProduct", 2.0, 2]]
    assert d["hyps"][-3:] == [0.01, 0.1, 0.001] and d["hyps"][0] == 2.0
    bd = d["descriptor_calculators"][0]
    assert bd["type"] == "B2" and bd["radial_basis"] == "chebyshev"
    assert bd["cutoff_hyps"] == [] and bd["cutoffs"] == [[5.0, 5.0]] * 2
    assert {int(k): v for k, v in d["species_map"].items()} == {13: 0, 29: 1}
    assert d["training_structures"] == []
