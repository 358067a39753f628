"""Uncertainty-aware molecular dynamics on the GPU: an ensemble of replicas
advanced by velocity Verlet with sparse-GP forces, every atom's local std
checked each step, and the sparse set grown from the most uncertain
environments followed by the FP64 re-solve.

The reference runs this loop in its OTF learner (flare/learners/otf.py:
507-521 computes forces and uncertainties per step through SGP_Calculator;
:548-600 adds uncertain environments and calls update_matrices_QR) with an
ASE integrator on the host, one structure at a time.  Here the replicas
live on the device (``fgb_md_*``): one batched prediction per step for all
of them.
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib
from ._lib import check, lib, ptr

# (eV/A)/amu in A/fs^2; kinetic energy m v^2 / 2 in eV is (amu A^2/fs^2) / KACCEL
KACCEL = 9.64853321e-3
KB_EV = 8.617333262e-5          # Boltzmann constant, eV/K


def maxwell_boltzmann(species, masses, temperature, seed):
    """Velocities (A/fs) from the Maxwell-Boltzmann distribution at
    ``temperature`` (K), centre-of-mass momentum removed."""
    r = np.random.Generator(np.random.PCG64(seed))
    m = np.asarray(masses, np.float64)[np.asarray(species)]
    sd = np.sqrt(KB_EV * temperature * KACCEL / m)
    v = r.normal(size=(len(m), 3)) * sd[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    return v


class Ensemble:
    """Replicas (lists of ``(cell, species, positions)`` with one atom
    count) of one sparse-GP model, advanced together on the GPU."""

    def __init__(self, sgp, descriptor_calculators, replicas, masses,
                 temperature=None, velocities=None, seed=0, cutoff=None,
                 precision="mixed", graphs=True, pair_margin=0.25):
        if not replicas:
            raise ValueError("no replicas")
        n = len(replicas[0][1])
        if any(len(sp) != n for _, sp, _ in replicas):
            raise ValueError("all replicas must have the same atom count")
        self.sgp = sgp
        self.calcs = list(descriptor_calculators)
        self.R, self.N = len(replicas), n
        self.masses = np.ascontiguousarray(masses, np.float64)
        # the structure cutoff: the largest per-species-pair cutoff
        self.cutoff = float(cutoff if cutoff is not None else
                            max(float(np.max(c.cutoffs)) for c in self.calcs))
        self.cells = np.ascontiguousarray(
            np.stack([np.asarray(c, np.float64).reshape(9)
                      for c, _, _ in replicas]))
        self.species = np.ascontiguousarray(
            np.concatenate([np.asarray(sp) for _, sp, _ in replicas]),
            np.int32)
        pos = np.ascontiguousarray(
            np.concatenate([np.asarray(p, np.float64).reshape(-1, 3)
                            for _, _, p in replicas]))
        if velocities is None:
            if temperature is None:
                raise ValueError("give velocities or a temperature")
            velocities = np.concatenate([
                maxwell_boltzmann(sp, self.masses, temperature, seed + k)
                for k, (_, sp, _) in enumerate(replicas)])
        vel = np.ascontiguousarray(velocities, np.float64).reshape(-1, 3)
        self._prec = {"fp64": _lib.FGB_PREC_FP64,
                      "mixed": _lib.FGB_PREC_MIXED}[precision]
        self._model = sgp._device_model(self.calcs)
        h = ctypes.c_void_p()
        check(lib().fgb_md_create(ctypes.byref(h), self._model.h, self.R,
                                  self.N, ptr(self.cells), ptr(pos), ptr(vel),
                                  ptr(self.species), ptr(self.masses),
                                  self.cutoff, self._prec), "Ensemble")
        self.h = h
        self.steps_done = 0
        self.set_graphs(graphs, pair_margin)

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.fgb_md_destroy(self.h)
            self.h = None

    def step(self, n_steps=1, dt=1.0, std_threshold=0.05):
        """Advance every replica by ``n_steps`` velocity-Verlet steps of
        ``dt`` fs, counting atoms whose local std exceeds the threshold."""
        check(lib().fgb_md_step(self.h, int(n_steps), float(dt),
                                float(std_threshold), _lib.stream_ptr()),
              "Ensemble.step")
        self.steps_done += n_steps

    def set_graphs(self, enable=True, pair_margin=0.25):
        """Replay CUDA-graph-captured steps (``enable``) with a pair
        capacity of the last full step's pairs x (1 + ``pair_margin``)."""
        check(lib().fgb_md_set_graphs(self.h, int(bool(enable)),
                                      float(pair_margin)), "Ensemble")

    def stats(self):
        """Replayed steps, full steps, graph captures, rolled-back chunks."""
        out = np.zeros(4, np.int64)
        check(lib().fgb_md_stats(self.h, ptr(out)), "Ensemble.stats")
        return dict(zip(("replayed", "full", "captures", "rollbacks"),
                        (int(x) for x in out)))

    def state(self):
        NT = self.R * self.N
        out = {k: np.zeros(s) for k, s in
               (("positions", (NT, 3)), ("velocities", (NT, 3)),
                ("forces", (NT, 3)), ("local_var", NT), ("energy", self.R),
                ("kinetic", self.R), ("max_std", self.R))}
        flagged = np.zeros(self.R, np.int64)
        check(lib().fgb_md_read(self.h, ptr(out["positions"]),
                                ptr(out["velocities"]), ptr(out["forces"]),
                                ptr(out["local_var"]), ptr(out["energy"]),
                                ptr(out["kinetic"]), ptr(out["max_std"]),
                                ptr(flagged), _lib.stream_ptr()),
              "Ensemble.state")
        out["flagged"] = flagged
        v = out["local_var"]
        sig = abs(self.sgp.kernels[0].sigma)
        out["std"] = np.sign(v) * np.sqrt(np.abs(v)) / sig
        dof = 3 * self.N - 3
        out["temperature"] = 2.0 * out["kinetic"] / (dof * KB_EV)
        return out

    def uncertain_environments(self, n):
        """The ``n`` (replica, atom) pairs with the largest local std,
        largest first (ties by position in the ensemble)."""
        std = self.state()["std"]
        order = np.lexsort((np.arange(std.size), -std))[:n]
        return [(int(a // self.N), int(a % self.N)) for a in order]

    def grow_sparse_set(self, n_new):
        """Add the ``n_new`` most uncertain environments to the sparse set
        (their replicas' current configurations), re-solve the model in
        FP64 (update_matrices_QR) and continue with it.  Returns timings."""
        from .core import Structure
        t0 = time.perf_counter()
        picks = self.uncertain_environments(n_new)
        st = self.state()
        pos = st["positions"].reshape(self.R, self.N, 3)
        by_rep = {}
        for r, a in picks:
            by_rep.setdefault(r, []).append(a)
        m_before = self.sgp.n_sparse
        items = []
        for r in sorted(by_rep):
            sp = self.species[r * self.N:(r + 1) * self.N]
            s = Structure(self.cells[r].reshape(3, 3), sp.tolist(), pos[r],
                          self.cutoff, self.calcs)
            items.append((s, sorted(by_rep[r])))
        self.sgp.add_environments_batch(items)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        self.sgp.update_matrices_QR()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        # the ensemble copies the new model's weights into its own replica
        new = self.sgp._device_model(self.calcs)
        check(lib().fgb_md_set_model(self.h, new.h), "Ensemble")
        self._model = new
        return {"sparse_before": int(m_before),
                "sparse_after": int(self.sgp.n_sparse),
                "n_labels": int(self.sgp.n_labels),
                "add_environments_s": t1 - t0, "resolve_fp64_s": t2 - t1,
                "replicas_touched": len(by_rep)}
