"""Benchmark: atoms/s for energy + forces + local std on the 2-species
1,000-atom alloy workload (flare_gb300.workloads.ALLOY), one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed] [--batch B]

A step is one batched pass of the prediction pipeline (neighbours, B2,
kernel against the 2,000-environment sparse set, reverse-mode adjoint forces
and stress, local variance) over B structures of 1,000 atoms.  `value` is
timed with CUDA events per step on the launching stream with inputs resident
in HBM (L2 flushed between steps by a 256 MiB write); `e2e` is the same step
through the C ABI with host buffers (pinned H2D of positions/species, D2H of
energy/forces/stress/variances inside the timed region).  `--impl reference`
times the FP64 CPU oracle (a restatement of the reference's flare_pp
algorithm; the reference itself cannot be built here) on the host cores.
Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("atoms/s (E+F+std) mixed-prec/adjoint vs FP64 plain on 1 GB300 at "
          "stated err; p99")
WORKLOAD = ("alloy1000: 2-species random alloy, 1000-atom cubic cell, 0.06 "
            "atoms/A^3, B2 n_max=8 l_max=4 rc=5.5, NormalizedDotProduct "
            "sigma=2 power=2, 2000 sparse envs (1000/species), 10 LJ-labelled "
            "training structures")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--batch", type=int, default=32,
                    help="structures (1000 atoms each) per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true")
    ap.add_argument("--oracle-weights", default=None,
                    help=argparse.SUPPRESS)
    ap.add_argument("--requests", type=int, default=0,
                    help="serve workload: number of requests (default 4096)")
    ap.add_argument("--replicas", type=int, default=0,
                    help="md workload: number of replicas (default 256)")
    ap.add_argument("--workload", default="alloy1000",
                    choices=["alloy1000", "fcc256", "fcc1m", "md", "serve",
                             "mapped"],
                    help="fcc1m: one 1,048,576-atom structure, E+F+virial, "
                         "peak device memory (reported as a side record)")
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n > 0 else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seeds(seed0, rank, n):
    """Seeds of one rank's n structures: disjoint across ranks, so every
    rank predicts its own units with no exchange (weak scaling)."""
    return [seed0 + rank * 100000 + i for i in range(n)]


# ------------------------------------------------------------ CPU oracle
def oracle_model():
    """FP64 CPU oracle model of the same sizes (M = 2000, n_d = 680) from
    two training structures; prediction cost does not depend on the
    training-set size."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from flare_gb300 import workloads as wl
    c = wl.ALLOY
    b2 = oracle.B2Settings("chebyshev", "quadratic", [0.0, c["rc"]], [],
                           [2, c["n_max"], c["l_max"]])
    k = oracle.NormalizedDotProduct(c["sigma"], c["power"])
    gp = oracle.SparseGP([k], c["sigma_e_per_atom"] * c["n_atoms"],
                         c["sigma_f"], c["sigma_s"])
    n_train = 2
    data = [wl.alloy_structure(c["train_seed0"] + t) for t in range(n_train)]
    sparse = wl.alloy_sparse_choice(n_train, [d[1] for d in data],
                                    c["sparse_per_species"], c["sparse_seed"])
    for t, (cell, sp, pos) in enumerate(data):
        st = oracle.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = wl.alloy_labels(cell, sp, pos)
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(st, sparse[t])
    gp.update_matrices_QR()
    return oracle, gp, b2


def oracle_step(oracle, gp, b2, seed):
    """One structure through the oracle: Structure (neighbours, B2 with
    stored gradients), predict_local_uncertainties, calculator results."""
    from flare_gb300 import workloads as wl
    cell, sp, pos = wl.alloy_structure(seed)
    st = oracle.Structure(cell, sp, pos, wl.ALLOY["rc"], [b2])
    gp.predict_local_uncertainties(st)
    oracle.calculator_results(st, "local", wl.ALLOY["sigma"])
    return len(sp)


def oracle_reference(gp, b2, struct):
    """E, F [N, 3], stress [6] and local variances (input order) of one
    structure from the FP64 CPU oracle carrying the GPU model's sparse set,
    alpha and L_inv (no training on the host)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from flare_gb300 import workloads as wl
    k = gp.kernels[0]
    ogp = oracle.SparseGP.from_weights(
        [oracle.NormalizedDotProduct(k.sigma, k.power)],
        gp.sparse_descriptors, gp.alpha, gp.L_inv)
    ob2 = oracle.B2Settings("chebyshev", "quadratic", [0.0, wl.ALLOY["rc"]],
                            [], [2, wl.ALLOY["n_max"], wl.ALLOY["l_max"]])
    cell, sp, pos = struct
    st = oracle.Structure(cell, sp, pos, wl.ALLOY["rc"], [ob2])
    ogp.predict_local_uncertainties(st)
    m = st.mean_efs
    return (m[0], m[1:-6].reshape(-1, 3), m[-6:],
            oracle.sort_variances(st, st.local_uncertainties[0]))


def _oracle_3species_model(cells, per_cell_sparse, lj_eps, lj_sigma, seed):
    """FP64 CPU oracle model with the 3-species descriptor of the serving
    and MD workloads (B2 [3, 8, 4], rc 5.5 A, n_d 1,500): LJ-labelled
    training cells and `per_cell_sparse` seeded sparse atoms per cell."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from flare_gb300 import synthetic as syn
    from flare_gb300 import workloads as wl
    c = wl.MD3
    b2 = oracle.B2Settings("chebyshev", "quadratic", [0.0, c["rc"]], [],
                           [3, c["n_max"], c["l_max"]])
    gp = oracle.SparseGP([oracle.NormalizedDotProduct(c["sigma"], c["power"])],
                         c["sigma_e_per_atom"] * len(cells[0][1]),
                         c["sigma_f"], c["sigma_s"])
    r = syn.rng(seed)
    for cell, sp, pos in cells:
        st = oracle.Structure(cell, sp, pos, c["rc"], [b2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, lj_eps, lj_sigma, c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        gp.add_training_structure(st)
        gp.add_specific_environments(
            st, sorted(r.choice(len(sp), size=per_cell_sparse,
                                replace=False).tolist()))
    gp.update_matrices_QR()
    return oracle, gp, b2


def cpu_serve_sweep(sizes=(32, 64, 128, 256, 512, 1024)):
    """The FP64 CPU oracle on one request per size (E + F + stress + local
    std, as the server answers), with a 3-species model of 600 sparse
    environments (the served model has 3,000: the oracle's stored-gradient
    envs_struc scales with M x 3P)."""
    from flare_gb300 import synthetic as syn
    from flare_gb300 import workloads as wl
    cells = [syn.rsa_alloy(500, density=0.07, fractions=(1 / 3,) * 3,
                           dmin=1.8, seed=4700 + t) for t in range(2)]
    oracle, gp, b2 = _oracle_3species_model(cells, 300, wl.MD3["eps"],
                                            wl.MD3["lj_sigma"], 4710)
    out = []
    for k, n in enumerate((sizes[0],) + tuple(sizes)):
        cell, sp, pos = syn.rsa_alloy(n, density=0.07, fractions=(1 / 3,) * 3,
                                      dmin=1.8, seed=4800 + k)
        t0 = time.perf_counter()
        st = oracle.Structure(cell, sp, pos, wl.MD3["rc"], [b2])
        gp.predict_local_uncertainties(st)
        oracle.calculator_results(st, "local", wl.MD3["sigma"])
        dt = time.perf_counter() - t0
        if k > 0:           # the first request warms up
            out.append({"atoms": n, "ms": 1e3 * dt, "atoms_per_s": n / dt})
    return {"kind": "port", "cores": cpu_cores(), "sparse_envs": gp.n_sparse,
            "sample": "one request per size after one warm-up; FP64 CPU "
                      "oracle (brute-force neighbours, stored-gradient B2, "
                      "envs_struc, K^T alpha, local variance)",
            "requests": out}


def cpu_md_step():
    """The FP64 CPU oracle's prediction for one md3 replica (2,000 atoms, 3
    species; forces and local variance are what a step needs) with a model
    of 1,000 sparse environments (the ensemble's has 8,000)."""
    from flare_gb300 import workloads as wl
    c = wl.MD3
    cells = [wl.md_cell(c["train_seed0"])]
    oracle, gp, b2 = _oracle_3species_model(cells, 1000, c["eps"],
                                            c["lj_sigma"], 5610)
    cell, sp, pos = wl.md_cell(c["replica_seed0"])
    times = []
    for _ in range(2):      # the first warms up
        t0 = time.perf_counter()
        st = oracle.Structure(cell, sp, pos, c["rc"], [b2])
        gp.predict_local_uncertainties(st)
        times.append(time.perf_counter() - t0)
    return {"kind": "port", "cores": cpu_cores(), "sparse_envs": gp.n_sparse,
            "replica_step_ms": 1e3 * times[-1],
            "atom_steps_per_s": c["n_atoms"] / times[-1],
            "sample": "one 2,000-atom replica's forces and local variance "
                      "after one warm-up, FP64 CPU oracle"}


def cpu_cores():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def time_oracle(n_structures, warm=1):
    oracle, gp, b2 = oracle_model()
    for w in range(warm):
        oracle_step(oracle, gp, b2, 2100 + w)
    times = []
    atoms = 0
    for k in range(n_structures):
        t0 = time.perf_counter()
        atoms += oracle_step(oracle, gp, b2, 2100 + k)
        times.append(time.perf_counter() - t0)
    sd = gp.sparse_descriptors[0]
    weights = {"alpha": gp.alpha, "L_inv": gp.L_inv}
    for s_ in range(sd.n_types):
        weights[f"desc{s_}"] = sd.descriptors[s_]
        weights[f"norm{s_}"] = sd.descriptor_norms[s_]
    return atoms / sum(times), times, weights


def oracle_model_from_weights(path):
    """The oracle model from saved weights (no training)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from types import SimpleNamespace
    from flare_gb300 import workloads as wl
    c = wl.ALLOY
    z = np.load(path)
    nt = 2
    sd = SimpleNamespace(n_types=nt, n_descriptors=z["desc0"].shape[1],
                         descriptors=[z[f"desc{s}"] for s in range(nt)],
                         descriptor_norms=[z[f"norm{s}"] for s in range(nt)])
    gp = oracle.SparseGP.from_weights(
        [oracle.NormalizedDotProduct(c["sigma"], c["power"])], [sd],
        z["alpha"], z["L_inv"])
    b2 = oracle.B2Settings("chebyshev", "quadratic", [0.0, c["rc"]], [],
                           [2, c["n_max"], c["l_max"]])
    return oracle, gp, b2


def time_oracle_one_thread(weights):
    """The oracle on one host thread (OpenMP and BLAS pinned to 1 in a child
    process that loads the model's weights): one structure after one
    warm-up."""
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "oracle_weights.npz")
        np.savez(path, **weights)
        env = dict(os.environ)
        for k_ in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS",
                   "MKL_NUM_THREADS", "BLIS_NUM_THREADS"):
            env[k_] = "1"
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"),
                            "--impl", "reference", "--steps", "1",
                            "--warmup", "1", "--oracle-weights", path],
                           env=env, capture_output=True, text=True,
                           timeout=600)
    for line in r.stdout.splitlines():
        if line.startswith("{"):
            d = json.loads(line)
            return {"value": d["value"], "unit": "atoms/s", "cores": 1,
                    "sample": "one 1000-atom alloy structure after one "
                              "warm-up, OMP and BLAS threads 1"}
    return {"error": (r.stderr or r.stdout)[-300:]}


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = cpu_cores()
    if args.oracle_weights:
        oracle, gp, b2 = oracle_model_from_weights(args.oracle_weights)
    else:
        oracle, gp, b2 = oracle_model()
    for w in range(args.warmup):
        oracle_step(oracle, gp, b2, 2100 + w)
    times, atoms = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        atoms += oracle_step(oracle, gp, b2, 2100 + k)
        times.append(time.perf_counter() - t0)
    v = atoms / sum(times)
    sample = ("one 1000-atom alloy structure per step: neighbours (brute "
              "force), B2 with stored gradients, envs_struc, K^T alpha, local "
              "variance via L_inv; FP64, OpenMP + BLAS threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "atoms/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "atoms_per_step": 1000,
                   "implementation": "FP64 CPU oracle restating flare_pp "
                                     "(reference unbuildable: Eigen/json "
                                     "fetched at configure time)"},
        "cpu_baseline": {"value": v, "unit": "atoms/s", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "atoms/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


# ------------------------------------------------------------- GPU arm
def timed_steps(torch, stream, flush, step, steps):
    """Per-step milliseconds from CUDA events on the launching stream; L2 is
    flushed (a 256 MiB write) before every step, outside the events."""
    per = []
    for _ in range(steps):
        flush.fill_(1.0)
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        torch.cuda.nvtx.range_push("timed_step")
        step()
        torch.cuda.nvtx.range_pop()
        s1.record(stream)
        s1.synchronize()
        per.append(s0.elapsed_time(s1))
    return per


def read_stages(L):
    """{stage name: (total ms, launches)} from the library's stage profiler."""
    import ctypes
    nst = L.fgb_profile_n_stages()
    ms = ctypes_array("d", nst)
    ln = ctypes_array("q", nst)
    L.fgb_profile_read(ctypes.cast(ms, ctypes.c_void_p),
                       ctypes.cast(ln, ctypes.c_void_p), nst)
    return {L.fgb_profile_stage_name(i).decode(): (ms[i], ln[i])
            for i in range(nst)}


def clocks_path(name):
    """Where a run's nvidia-smi clock samples go: $FGB_CLOCKS_DIR (created
    if needed) or the temporary directory."""
    import tempfile
    d = os.environ.get("FGB_CLOCKS_DIR") or tempfile.gettempdir()
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, name)


class Clocks:
    """nvidia-smi clock samples during a timed region: sampling starts (and
    its first line is written) before the region, every 20 ms; the summary
    keeps the samples taken after that first line, i.e. inside the region."""

    def __init__(self, path):
        self.path = path
        self.p = None
        self.skip = 0

    def _lines(self):
        try:
            with open(self.path) as f:
                return f.read().count("\n")
        except Exception:
            return 0

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while self._lines() == 0 and time.time() - t0 < 5.0:
                time.sleep(0.005)
            self.skip = self._lines()
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self, dev_index=0):
        try:
            lines = open(self.path).read().splitlines()
        except Exception:
            return None
        # (line number, fields): the lines before `skip` were written before
        # the timed region began
        rows = [(k, [x.strip() for x in l.split(",")])
                for k, l in enumerate(lines)]

        def numeric(r):
            try:
                float(r[1]), float(r[2])
                return True
            except ValueError:
                return False
        rows = [(k, r) for k, r in rows if len(r) >= 9 and numeric(r)]
        rows = [(k, r) for k, r in rows if r[0] == str(dev_index)] or rows
        inside = [(k, r) for k, r in rows if k >= self.skip]
        # samples from inside the region (if there are none, those written
        # before it, and samples_in_region says so)
        rows = [r for _, r in (inside or rows)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx,
                "reasons": reasons, "samples": len(rows),
                "samples_in_region": len(inside)}


def measure_fp64_peak(torch):
    """cuBLAS DGEMM throughput (TFLOP/s), best of 5 on 8192^3."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def run_ours(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    import flare_gb300 as fg
    from flare_gb300 import _lib
    from flare_gb300 import workloads as wl
    L = _lib.lib()
    c = wl.ALLOY
    t_setup = time.time()
    gp, b2, k = wl.build_alloy_model()
    model = gp._device_model([b2])
    train_s = time.time() - t_setup

    B = args.batch
    structs = [wl.alloy_structure(sd)
               for sd in rank_seeds(c["test_seed0"], rank, B)]
    offsets = np.zeros(B + 1, dtype=np.int32)
    for i, s in enumerate(structs):
        offsets[i + 1] = offsets[i] + len(s[1])
    cells = np.ascontiguousarray(np.stack([s[0].reshape(-1) for s in structs]))
    pos = np.ascontiguousarray(np.concatenate([s[2] for s in structs]))
    sp = np.ascontiguousarray(np.concatenate([s[1] for s in structs]).astype(np.int32))
    N = int(offsets[-1])
    dev = torch.device("cuda", local)
    d_pos = torch.from_numpy(pos).to(dev)
    d_sp = torch.from_numpy(sp).to(dev)
    out = {k_: torch.zeros(n, dtype=torch.float64, device=dev)
           for k_, n in (("e", B), ("f", 3 * N), ("s", 6 * B), ("v", N))}
    stream = torch.cuda.current_stream()
    sptr = _lib.stream_ptr(stream)
    prec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}[args.precision]
    want = 0xF
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(precision=prec):
        _lib.check(L.fgb_predict(model.h, B, _lib.ptr(offsets), _lib.ptr(cells),
                                 _lib.ptr(d_pos), _lib.ptr(d_sp), c["rc"], want,
                                 precision, _lib.ptr(out["e"]),
                                 _lib.ptr(out["f"]), _lib.ptr(out["s"]),
                                 _lib.ptr(out["v"]), sptr))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # ---- timed region: device-resident inputs, stage profiler off
    L.fgb_profile_enable(0)
    clocks = Clocks(clocks_path(f"clocks_rank{rank}.csv"))
    barrier(world)
    torch.cuda.synchronize()
    with clocks:
        per = timed_steps(torch, stream, flush, step, args.steps)
    torch.cuda.synchronize()
    barrier(world)
    total_ms = sum(per)
    total_ms_max = max_over_ranks(total_ms, world)
    atoms_all = N * args.steps * world
    value = atoms_all / (total_ms_max * 1e-3)
    res_e = out["e"].cpu().numpy().copy()
    res_f = out["f"].cpu().numpy().copy()
    res_s = out["s"].cpu().numpy().copy()
    res_v = out["v"].cpu().numpy().copy()

    # ---- stage split: the same steps again with the per-stage CUDA-event
    # profiler on (events on the launching stream); not part of `value`
    L.fgb_profile_reset()
    L.fgb_profile_enable(1)
    prof_per = timed_steps(torch, stream, flush, step, args.steps)
    torch.cuda.synchronize()
    L.fgb_profile_enable(0)
    stage = read_stages(L)

    # ---- errors of this precision against the FP64 path (same batch), and
    # the fused FP64 path's own throughput on it (CUDA events, same flush)
    errors = None
    fp64_fused = None
    nat = np.diff(offsets)
    std = lambda v: np.where(v > 0, np.sqrt(np.abs(v)),
                             -np.sqrt(np.abs(v))) / c["sigma"]
    if args.precision != "fp64":
        step(_lib.FGB_PREC_FP64)
        torch.cuda.synchronize()
        k64 = max(3, min(args.steps, 5))
        per64 = timed_steps(torch, stream, flush,
                            lambda: step(_lib.FGB_PREC_FP64), k64)
        fp64_fused = {"value": N * k64 / (sum(per64) * 1e-3),
                      "unit": "atoms/s", "steps": k64,
                      "sample": f"the same {B}-structure batch through the "
                                "fused FP64 path (neighbours, FP64 B2, FP64 "
                                "SIMT GEMMs, FP64 adjoint), CUDA events"}
        e64 = out["e"].cpu().numpy()
        f64 = out["f"].cpu().numpy()
        s64 = out["s"].cpu().numpy()
        v64 = out["v"].cpu().numpy()
        errors = {
            "energy_ev_per_atom_max": float(np.max(np.abs(res_e - e64) / nat)),
            "force_mae_ev_per_a": float(np.mean(np.abs(res_f - f64))),
            "force_max_ev_per_a": float(np.max(np.abs(res_f - f64))),
            "stress_max_ev_per_a3": float(np.max(np.abs(res_s - s64))),
            "local_std_max_abs": float(np.max(np.abs(std(res_v) - std(v64)))),
            "reference": "FP64 path of this library on the same batch"}
    # against the FP64 CPU oracle carrying this model's weights, on the
    # batch's first structure (rank 0)
    errors_oracle = None
    if rank == 0 and not args.no_oracle_check:
        n0 = int(nat[0])
        E, F, Sg, V = oracle_reference(gp, b2, structs[0])
        errors_oracle = {
            "structure": "batch structure 0 (seed %d, %d atoms)"
                         % (c["test_seed0"], n0),
            "energy_ev_per_atom": float(abs(res_e[0] - E) / n0),
            "force_mae_ev_per_a": float(np.mean(np.abs(res_f[:3 * n0] -
                                                       F.reshape(-1)))),
            "force_max_ev_per_a": float(np.max(np.abs(res_f[:3 * n0] -
                                                      F.reshape(-1)))),
            "stress_max_ev_per_a3": float(np.max(np.abs(res_s[:6] - Sg))),
            "local_var_max_abs": float(np.max(np.abs(res_v[:n0] - V))),
            "local_std_max_abs": float(np.max(np.abs(std(res_v[:n0]) -
                                                     std(V)))),
            "reference": "FP64 CPU oracle (restatement of flare_pp's "
                         "predict_local_uncertainties) with this model's "
                         "sparse set, alpha and L_inv"}

    # ---- e2e through the host-buffer C ABI (pinned buffers)
    h_pos = torch.from_numpy(pos).pin_memory()
    h_sp = torch.from_numpy(sp).pin_memory()
    h_out = {k_: torch.zeros(n, dtype=torch.float64).pin_memory()
             for k_, n in (("e", B), ("f", 3 * N), ("s", 6 * B), ("v", N))}

    def step_host():
        _lib.check(L.fgb_predict_host(
            model.h, B, _lib.ptr(offsets), _lib.ptr(cells), _lib.ptr(h_pos),
            _lib.ptr(h_sp), c["rc"], want, prec, _lib.ptr(h_out["e"]),
            _lib.ptr(h_out["f"]), _lib.ptr(h_out["s"]), _lib.ptr(h_out["v"]),
            sptr))

    for _ in range(max(1, args.warmup)):
        step_host()
    e2e = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_host()
        e2e.append(time.perf_counter() - t0)
    e2e_max = max_over_ranks(sum(e2e), world)
    e2e_value = atoms_all / e2e_max
    h2d = pos.nbytes + sp.nbytes + cells.nbytes + offsets.nbytes
    d2h = 8 * (B + 3 * N + 6 * B + N)

    guard = None
    if args.precision == "mixed":
        import ctypes
        fmax, f64 = ctypes.c_double(0.0), ctypes.c_int(0)
        sl, est = ctypes.c_int(0), ctypes.c_double(0.0)
        _lib.check(L.fgb_model_mixed_plan(model.h, ctypes.byref(sl),
                                          ctypes.byref(est), ctypes.byref(fmax),
                                          ctypes.byref(f64), sptr))
        slv, vest = ctypes.c_int(0), ctypes.c_double(0.0)
        _lib.check(L.fgb_model_slice_plan(model.h, None, ctypes.byref(slv),
                                          None, ctypes.byref(vest), sptr))
        guard = {"kernel_slices": sl.value,
                 "slice_err_ev_per_atom": est.value,
                 "variance_slices": slv.value,
                 "variance_slice_err": vest.value,
                 "fold_max": fmax.value,
                 "force_stage": "fp64-level" if f64.value else "fp32-level",
                 "fold_threshold": 200.0}

    # ---- dominant kernel roofline.  Algorithmic FLOP per launch: the
    # kernel GEMM c = d^ . s^ is 2 M_s n_d per atom of species s (one launch
    # per species and row chunk), counted once whatever precision scheme
    # carries it; the time is the GEMM kernel's own launches (the row
    # slicing is a stage of its own).
    sizes = species_sizes(sp, offsets, gp)
    nd_ = b2.n_descriptors
    fp64_flops = {"kernel_gemm": sum(2.0 * n_s * m_s * nd_ for n_s, m_s in sizes),
                  "adjoint_gemm": sum(2.0 * n_s * m_s * nd_ for n_s, m_s in sizes),
                  "variance_gemm": sum(1.0 * n_s * m_s * (m_s + 1)
                                       for n_s, m_s in sizes)}
    tensor = args.precision == "mixed" and oz_eligible(gp, b2)
    gemm_stage = max(fp64_flops, key=lambda s_: stage.get(s_, (0, 0))[0])
    st_ms, st_n = stage[gemm_stage]
    launches_per_step = st_n / args.steps
    avg_ms = st_ms / st_n
    alg = fp64_flops[gemm_stage] / max(launches_per_step, 1)
    achieved = alg / (avg_ms * 1e-3) / 1e12
    fp64_peak = measure_fp64_peak(torch)
    if tensor:
        # executed on the tensor pipe: S(S+1)/2 BF16 slice products per
        # FP64-level product (S slices of 6 bits, a + b <= S + 1)
        S_ = (guard["variance_slices"] if gemm_stage == "variance_gemm"
              else guard["kernel_slices"]) if guard else 9
        products = S_ * (S_ + 1) // 2
        peak, peak_src = bf16_peak()
        roofline = {"kernel": gemm_stage + " (k_oz_gemm, tcgen05, exact BF16 "
                              "slicing)",
                    "bound": "tensor", "achieved": achieved,
                    "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak,
                    "traffic": None,
                    "traffic_note": "DRAM bytes are not measured in this run; "
                                    "the ncu capture of this kernel is "
                                    "summarised under profiles/",
                    "peak_source": peak_src,
                    "flop_per_launch_algorithmic": alg,
                    "avg_launch_ms": avg_ms,
                    "launches_per_step": launches_per_step,
                    "slices": S_, "products_per_fp64_product": products,
                    "slice_products_tflops": products * achieved,
                    "slice_products_frac": products * achieved / peak,
                    "fp64_dgemm_measured_tflops": fp64_peak,
                    "vs_fp64_dgemm": achieved / fp64_peak,
                    "note": "achieved = algorithmic FLOP (2 M_s n_d per atom, "
                            "counted once) / the GEMM kernel's mean launch "
                            "time; the kernel carries it at FP64-level "
                            "accuracy as products_per_fp64_product BF16 "
                            "slice products (slice_products_frac = tensor "
                            "pipe work against the same peak)"}
    else:
        roofline = {"kernel": gemm_stage, "bound": "tensor",
                    "achieved": achieved, "peak": fp64_peak,
                    "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                    "traffic": None,
                    "peak_source": "FP64 cuBLAS DGEMM 8192^3 measured in this "
                                   "run (FP64 has no entry in the measured-peaks "
                                   "file)",
                    "flop_per_launch_algorithmic": alg, "avg_launch_ms": avg_ms,
                    "launches_per_step": launches_per_step}
    gpu_launches = int(sum(v[1] for v in stage.values()))

    result = {
        "metric": METRIC, "value": value, "unit": "atoms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "structures_per_step": B,
                   "atoms_per_step": N, "precision": args.precision,
                   "l2": "flushed between steps (256 MiB write)",
                   "train_setup_s": round(train_s, 1)},
        "latency_ms": {"p50": float(np.percentile(per, 50)),
                       "p99": float(np.percentile(per, 99)),
                       "per_step": [round(x, 3) for x in per]},
        "e2e": {"value": e2e_value, "unit": "atoms/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "p50_ms": 1e3 * float(np.percentile(e2e, 50)),
                "p99_ms": 1e3 * float(np.percentile(e2e, 99))},
        "roofline": roofline,
        "stages_ms_per_step": {k_: round(v[0] / args.steps, 4)
                               for k_, v in stage.items() if v[1]},
        "stage_split": {"source": "a second pass of the same steps with the "
                                  "per-stage CUDA-event profiler on",
                        "ms_per_step": sum(prof_per) / args.steps},
        "errors_vs_oracle": errors_oracle,
        "gpu_launches": gpu_launches,
        "errors_vs_fp64": errors,
        "mixed_plan": guard,
        "clocks": clocks.summary(local),
        "autotune": autotune_table(),
    }
    if rank == 0 and not args.no_plain:
        result["fp64_plain"] = time_plain(L, _lib, model, structs[:6], b2, c,
                                          torch)
        if result["fp64_plain"] and fp64_fused:
            result["fp64_plain"]["mixed_over_plain"] = \
                value / world / result["fp64_plain"]["value"]
    if fp64_fused:
        fp64_fused["mixed_over_fused_fp64"] = value / world / fp64_fused["value"]
        result["fp64_fused"] = fp64_fused
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, ts, weights = time_oracle(2)
            result["cpu_baseline"] = {
                "value": v, "unit": "atoms/s", "cores": cpu_cores(),
                "kind": "port",
                "sample": "2 alloy structures (2000 atoms) through the FP64 "
                          "CPU oracle (brute-force neighbours, stored-gradient "
                          "B2, envs_struc, local variance), after 1 warm-up"}
            result["cpu_baseline"]["one_thread"] = time_oracle_one_thread(
                weights)
        except Exception as ex:  # report, never hide
            result["cpu_baseline"] = {"error": repr(ex)}
    if rank == 0:
        result["sample_energy_per_atom"] = float(res_e[0] / 1000)
        print(json.dumps(result), flush=True)



def oz_eligible(gp, b2):
    # the mixed path runs the kernel and variance GEMMs on the tensor cores
    # for powers 1 and 2 (any n_d: K runs in exact segments)
    return gp.kernels[0].power in (1.0, 2.0)




def bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), \
                "MEASURED_PEAKS.json bf16_tflops (burst, measured)"
    except Exception:
        return 1900.0, "fallback 1.9 PFLOP/s bf16 (measured-peaks file absent)"


def ctypes_array(code, n):
    import ctypes
    t = {"d": ctypes.c_double, "q": ctypes.c_longlong}[code]
    return (t * n)()


def species_sizes(sp, offsets, gp):
    sd = gp.sparse_descriptors[0]
    out = []
    for s in range(sd.n_types):
        out.append((int((sp == s).sum()), int(sd.n_clusters_by_type[s])))
    return out


def time_plain(L, _lib, model, structs, b2, c, torch):
    """The plain FP64 GPU form of the reference algorithm (stored forward
    gradients, envs_struc GEMM + scatter, K^T alpha, variance), one
    structure per call: the first structure warms up, the others are timed
    with CUDA events on the launching stream (the neighbour list is built
    outside the events, as the reference's Structure does before
    prediction)."""
    import flare_gb300 as fg
    stream = torch.cuda.current_stream()
    times, atoms = [], 0
    for i, (cell, sp, pos) in enumerate(structs):
        st = fg.Structure(cell, sp, pos, c["rc"], [b2])
        nl = st.nlist()
        d = st._inputs()
        N = st.noa
        mean = torch.zeros(1 + 3 * N + 6, dtype=torch.float64, device="cuda")
        var = torch.zeros(N, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        _lib.check(L.fgb_predict_plain(model.h, nl.h, _lib.ptr(d["species"]),
                                       _lib.ptr(mean), _lib.ptr(var),
                                       _lib.stream_ptr(stream)))
        s1.record(stream)
        s1.synchronize()
        if i > 0:            # first one warms up
            times.append(s0.elapsed_time(s1) * 1e-3)
            atoms += N
    if not times:
        return None
    return {"value": atoms / sum(times), "unit": "atoms/s",
            "sample": f"{len(times)} structures after 1 warm-up, CUDA events"}


def run_fcc256(args):
    """fcc256, the reference's small CPU-runnable case: energy, forces,
    stress and local variance of 256-atom FCC cells in FP64 through
    SparseGP.predict_batch (host arrays in and out, so this is end to end),
    64 cells per call and one per call; the mixed path on the same calls;
    the plain FP64 GPU form; and the FP64 CPU oracle on the host cores, with
    the GPU's FP64 results checked against it."""
    import torch
    import flare_gb300 as fg
    from flare_gb300 import _lib
    from flare_gb300 import synthetic as syn
    from flare_gb300 import workloads as wl
    L = _lib.lib()
    c = wl.FCC256
    t0 = time.time()
    gp, b2, k = wl.build_fcc256_model()
    train_s = time.time() - t0
    B = 64
    structs = [wl.fcc256_structure(c["test_seed0"] + i) for i in range(B)]
    fgs = [fg.Structure(cl, sp, ps, c["rc"], [b2]) for cl, sp, ps in structs]

    def timed(batch, prec):
        for _ in range(max(args.warmup, 1)):
            gp.predict_batch(batch, precision=prec)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            r = gp.predict_batch(batch, precision=prec)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t1) / args.steps
        return dt, r

    f64_b, r64 = timed(fgs, "fp64")
    f64_1, _ = timed(fgs[:1], "fp64")
    mix_b, rmx = timed(fgs, "mixed")
    plain = time_plain(L, _lib, gp._device_model([b2]), structs[:3], b2, c,
                       torch)
    # FP64 CPU oracle: the same model trained on the host
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ob2 = oracle.B2Settings("chebyshev", "quadratic", [0.0, c["rc"]], [],
                            [1, c["n_max"], c["l_max"]])
    ogp = oracle.SparseGP([oracle.NormalizedDotProduct(c["sigma"], c["power"])],
                          c["sigma_e"], c["sigma_f"], c["sigma_s"])
    sparse = wl.fcc256_sparse_choice()
    for t in range(c["n_train"]):
        cell, sp, pos = wl.fcc256_structure(c["train_seed0"] + t)
        st = oracle.Structure(cell, sp, pos, c["rc"], [ob2])
        E, F, _ = syn.lennard_jones(cell, sp, pos, [0.4], [2.6], c["rc"])
        st.energy = np.array([E])
        st.forces = F.reshape(-1)
        ogp.add_training_structure(st)
        ogp.add_specific_environments(st, sparse[t])
    ogp.update_matrices_QR()
    cpu_t = []
    for i in range(3):
        cell, sp, pos = structs[i]
        t1 = time.perf_counter()
        st = oracle.Structure(cell, sp, pos, c["rc"], [ob2])
        ogp.predict_local_uncertainties(st)
        cpu_t.append(time.perf_counter() - t1)
        if i == 0:
            ref_e, ref_f = st.mean_efs[0], st.mean_efs[1:-6].reshape(-1, 3)
    cpu_v = 256 * 2 / sum(cpu_t[1:])
    print(json.dumps({
        "metric": "atoms/s (E+F+S+local std) in FP64, 256-atom FCC",
        "value": B * 256 / f64_b, "unit": "atoms/s",
        "config": {"workload": "fcc256: 4x4x4 FCC cells, a 4.05, sigma 0.05; "
                               "B2 [1,8,3] rc 5.0; NormalizedDotProduct sigma 2 "
                               "power 2; 20 LJ-labelled training cells, 200 "
                               "sparse envs", "structures_per_call": B,
                   "calls": args.steps, "timing": "wall clock around "
                   "SparseGP.predict_batch (host arrays in and out)"},
        "fp64_ms_per_call": 1e3 * f64_b,
        "fp64_one_structure_ms": 1e3 * f64_1,
        "mixed": {"value": B * 256 / mix_b, "ms_per_call": 1e3 * mix_b,
                  "energy_ev_per_atom_max":
                      float(np.max(np.abs(rmx["energy"] - r64["energy"])) / 256),
                  "force_mae_ev_per_a":
                      float(np.mean(np.abs(rmx["forces"] - r64["forces"])))},
        "fp64_plain": plain,
        "cpu_oracle": {"value": cpu_v, "unit": "atoms/s", "cores": cpu_cores(),
                       "sample": "2 structures after 1 warm-up"},
        "fp64_vs_oracle": {
            "energy_ev": float(abs(r64["energy"][0] - ref_e)),
            "force_max_ev_per_a": float(np.max(np.abs(
                r64["forces"][:256] - ref_f)))},
        "train_setup_s": round(train_s, 1),
    }), flush=True)


def run_fcc1m(args):
    """One 1,048,576-atom FCC structure: energy, forces and virial through
    the reverse-mode adjoint (mixed and FP64), device memory, and the
    footprint the stored forward-mode gradients would need."""
    import torch
    import flare_gb300 as fg
    from flare_gb300 import _lib
    from flare_gb300 import workloads as wl
    L = _lib.lib()
    c = wl.FCC1M
    t0 = time.time()
    gp, b2, k = wl.build_fcc_model()
    train_s = time.time() - t0
    cell, sp, pos = wl.fcc_structure()
    N = len(sp)
    free0, total = torch.cuda.mem_get_info()
    out = {}
    for prec in ("mixed", "fp64"):
        s = fg.Structure(cell, sp, pos, c["rc"], [b2])
        torch.cuda.synchronize()
        times = []
        for rep in range(max(1, args.steps)):
            t1 = time.perf_counter()
            r = gp.predict_batch([s], want=7, precision=prec)
            times.append(time.perf_counter() - t1)
        free1, _ = torch.cuda.mem_get_info()
        out[prec] = {"seconds": float(np.median(times)),
                     "atoms_per_s": N / float(np.median(times)),
                     "energy_ev": float(r["energy"][0]),
                     "stress_flare_order": [float(x) for x in r["stress"][0]],
                     "device_bytes_in_use": int(total - free1),
                     "device_bytes_added": int(free0 - free1)}
    P = fg.Structure(cell, sp, pos, c["rc"], []).n_neighbors
    nd = b2.n_descriptors
    M = gp.n_sparse
    print(json.dumps({
        "workload": "fcc1m: 1,048,576-atom FCC (64^3 cells, a = 4.05, sigma "
                    "0.08), B2 n_max 10 l_max 6 rc 5.0, 4000 sparse envs",
        "n_atoms": N, "n_pairs": int(P), "train_setup_s": round(train_s, 1),
        "adjoint": out,
        "stored_forward_mode_bytes": {
            "dB2_dr_3P_x_nd_fp64": 3 * int(P) * nd * 8,
            "envs_struc_force_kernel_3P_x_M_fp64": 3 * int(P) * M * 8,
            "device_total_bytes": int(total),
            "fits": 3 * int(P) * nd * 8 < total},
        "energy_difference_mixed_vs_fp64_ev_per_atom":
            abs(out["mixed"]["energy_ev"] - out["fp64"]["energy_ev"]) / N,
    }), flush=True)


def run_serve(args):
    """Serving stream (serve3): requests of 32-4096 atoms and 1-3 species
    through the continuous-batching server; first all at once (saturation
    throughput), then Poisson arrivals at 0.25-4x that rate, each with
    throughput and p50/p99 latency (submit to result, server clock)."""
    import threading
    import torch
    from flare_gb300 import workloads as wl
    from flare_gb300.serving import Server
    c = wl.SERVE3
    n_req = args.requests or c["n_requests"]
    t0 = time.time()
    reqs = wl.serve_requests(n_req)          # spawned workers
    gen_s = time.time() - t0
    t0 = time.time()
    gp, b2, k = wl.build_serve_model()
    train_s = time.time() - t0
    atoms = np.array([len(r[1]) for r in reqs])
    srv = Server(gp, b2, c["rc"], n_workers=2, memory_budget_gb=16.0,
                 max_structures=64, precision=args.precision)
    for q in range(min(8, n_req)):            # warm-up: model set-up, kernels
        srv.result(srv.submit(*reqs[q]))

    def run(times):
        """Submit request q at times[q] (s from start); wait for all."""
        ids = [None] * n_req
        start = time.perf_counter()

        def producer():
            for q in range(n_req):
                while True:
                    dt = times[q] - (time.perf_counter() - start)
                    if dt <= 0:
                        break
                    time.sleep(min(dt, 2e-4) if dt > 2e-4 else 0)
                ids[q] = srv.submit(*reqs[q])
        b0 = srv.stats()["batches"]
        th = threading.Thread(target=producer)
        th.start()
        th.join()
        lat = np.array([srv.result(i)["latency_ms"] for i in ids])
        span = time.perf_counter() - start
        return {"requests": n_req, "seconds": span,
                "atoms_per_s": float(atoms.sum() / span),
                "requests_per_s": n_req / span,
                "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)),
                "batches": srv.stats()["batches"] - b0}

    with Clocks(clocks_path("clocks_serve.csv")) as clocks:
        sat = run(np.zeros(n_req))
        lam = sat["requests_per_s"]
        sweep = []
        rng_ = np.random.Generator(np.random.PCG64(4500))
        for f in (0.25, 0.5, 1.0, 2.0, 4.0):
            gaps = rng_.exponential(1.0 / (f * lam), size=n_req)
            r = run(np.cumsum(gaps) - gaps[0])
            r["offered_rate_x_saturation"] = f
            sweep.append(r)
    srv.close()
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_serve_sweep()
        except Exception as ex:  # report, never hide
            cpu = {"error": repr(ex)}
    print(json.dumps({
        "metric": "serving atoms/s (E+F+stress+local std per request) with "
                  "p50/p99 latency",
        "value": sat["atoms_per_s"], "unit": "atoms/s",
        "precision": args.precision,
        "config": {"workload": "serve3: %d requests, 32-4096 atoms "
                               "(log-uniform), 1-3 species, density "
                               "0.05-0.09; B2 [3,8,4] rc 5.5 (n_d 1500), "
                               "1000 sparse envs per species; 2 workers, "
                               "<= 64 structures per batch" % n_req,
                   "atoms_total": int(atoms.sum()),
                   "atoms_mean": float(atoms.mean())},
        "saturation": sat, "poisson_sweep": sweep, "cpu_baseline": cpu,
        "mixed_plan": gp.mixed_plan() if args.precision == "mixed" else None,
        "setup_s": {"train_fp64": round(train_s, 1),
                    "request_generation": round(gen_s, 1)},
        "clocks": clocks.summary(),
    }), flush=True)


def autotune_table():
    """Tile shapes the autotuner chose for the sliced GEMMs (per shape:
    operation, rows bucket, columns, depth, choice, ms per candidate)."""
    from flare_gb300 import autotune
    return [{**e, "ms": [round(x, 4) for x in e["ms"]]}
            for e in autotune.table()]


def run_mapped(args):
    """Evaluation from mapping coefficients (the LAMMPS pair style's model):
    the alloy1000 power-2 model written to an lmp.flare file and read back,
    energies + forces + stresses of 32 structures per call, device-resident
    inputs, against the same model's sparse-GP prediction (E+F+S, FP64)."""
    import tempfile
    import torch
    from flare_gb300 import _lib
    from flare_gb300 import workloads as wl
    from flare_gb300.mapped import MappedPotential
    L = _lib.lib()
    c = wl.ALLOY
    gp, b2, k = wl.build_alloy_model()
    model = gp._device_model([b2])
    with tempfile.TemporaryDirectory() as td:
        t0 = time.time()
        path = os.path.join(td, "lmp.flare")
        gp.write_mapping_coefficients(path, "bench", 0)
        write_s = time.time() - t0
        size = os.path.getsize(path)
        pot = MappedPotential(path)
    B = args.batch
    structs = [wl.alloy_structure(c["test_seed0"] + i) for i in range(B)]
    offsets = np.zeros(B + 1, dtype=np.int32)
    for i, s_ in enumerate(structs):
        offsets[i + 1] = offsets[i] + len(s_[1])
    cells = np.ascontiguousarray(np.stack([s_[0].reshape(-1) for s_ in structs]))
    pos = np.ascontiguousarray(np.concatenate([s_[2] for s_ in structs]))
    sp = np.ascontiguousarray(np.concatenate([s_[1] for s_ in structs]).astype(np.int32))
    N = int(offsets[-1])
    dev = torch.device("cuda", 0)
    d_pos = torch.from_numpy(pos).to(dev)
    d_sp = torch.from_numpy(sp).to(dev)
    out = {k_: torch.zeros(n, dtype=torch.float64, device=dev)
           for k_, n in (("e", B), ("f", 3 * N), ("s", 6 * B), ("a", N),
                         ("e2", B), ("f2", 3 * N), ("s2", 6 * B), ("v", N))}
    sptr = _lib.stream_ptr(torch.cuda.current_stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    mprec = {"fp64": _lib.FGB_PREC_FP64, "mixed": _lib.FGB_PREC_MIXED}

    def mapped_step(precision=args.precision):
        _lib.check(L.fgb_mapped_predict(
            pot.h, B, _lib.ptr(offsets), _lib.ptr(cells), _lib.ptr(d_pos),
            _lib.ptr(d_sp), c["rc"], 0x7, _lib.ptr(out["e"]), _lib.ptr(out["f"]),
            _lib.ptr(out["s"]), _lib.ptr(out["a"]), None, mprec[precision],
            sptr))

    def gp_step(prec):
        _lib.check(L.fgb_predict(model.h, B, _lib.ptr(offsets), _lib.ptr(cells),
                                 _lib.ptr(d_pos), _lib.ptr(d_sp), c["rc"], 0x7,
                                 prec, _lib.ptr(out["e2"]), _lib.ptr(out["f2"]),
                                 _lib.ptr(out["s2"]), None, sptr))

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        per = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            per.append(e0.elapsed_time(e1))
        return float(np.median(per))

    clocks = Clocks(clocks_path("clocks_mapped.csv"))
    os.makedirs(os.path.dirname(clocks.path), exist_ok=True)
    with clocks:
        ms_map = timed(mapped_step)
    other = "fp64" if args.precision == "mixed" else "mixed"
    ms_map_other = timed(lambda: mapped_step(other))
    ms_gp64 = timed(lambda: gp_step(_lib.FGB_PREC_FP64))
    ms_gpmx = timed(lambda: gp_step(_lib.FGB_PREC_MIXED))
    mapped_step()
    gp_step(_lib.FGB_PREC_FP64)
    torch.cuda.synchronize()
    e_err = float((out["e"] - out["e2"]).abs().max()) / 1000
    f_err = float((out["f"] - out["f2"]).abs().max())
    f_mae = float((out["f"] - out["f2"]).abs().mean())
    print(json.dumps({
        "metric": "mapped evaluation atoms/s (E+F+S from lmp.flare coefficients)",
        "value": N / (ms_map * 1e-3), "unit": "atoms/s",
        "ms_per_step": ms_map, "steps": args.steps,
        "warmup": max(args.warmup, 3), "precision": args.precision,
        "dtype": "f64 (exact-slicing tensor-core Y = B2 beta)" if args.precision == "fp64"
                 else "f64+df+f32 (double-float descriptor, FP32 adjoint, FP64-level Y)",
        "other_precision_ms_per_step": {other: ms_map_other},
        "config": {"workload": "alloy1000 power-2 model mapped: %d structures x "
                               "1000 atoms, B2 [2,8,4] rc 5.5 (n_d 680)" % B,
                   "atoms_per_step": N, "l2": "flushed between steps"},
        "coefficient_file": {"bytes": size, "write_s": round(write_s, 2)},
        "same_model_sparse_gp_ms_per_step": {"fp64": ms_gp64, "mixed": ms_gpmx,
                                             "want": "E+F+S"},
        "mapped_vs_fp64_gp": {"energy_ev_per_atom_max": e_err,
                              "force_max_ev_per_a": f_err,
                              "force_mae_ev_per_a": f_mae},
        "clocks": clocks.summary(),
    }), flush=True)


def run_md(args):
    """Uncertainty-aware MD ensemble (md3): replicas advanced together by
    velocity Verlet with forces and local std every step; then the sparse
    set grows by the most uncertain environments and is re-solved in FP64."""
    import torch
    from flare_gb300 import workloads as wl
    from flare_gb300.md import Ensemble
    c = wl.MD3
    R = args.replicas or c["n_replicas"]
    t0 = time.time()
    reps = wl.md_replicas(R)           # spawned workers, before CUDA work
    gen_s = time.time() - t0
    t0 = time.time()
    gp, b2, k = wl.build_md_model()
    train_s = time.time() - t0
    ens = Ensemble(gp, [b2], reps, c["masses"], temperature=c["temperature"],
                   seed=c["velocity_seed0"], precision=args.precision)
    N = R * c["n_atoms"]
    s0 = ens.state()
    ens.step(max(args.warmup, 1), dt=c["dt"], std_threshold=c["std_threshold"])
    e0 = ens.state()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(clocks_path("clocks_md.csv"))
    os.makedirs(os.path.dirname(clocks.path), exist_ok=True)
    # the timed steps in chunks of up to 100, with the ensemble's state read
    # between chunks (outside the events): drift, temperature and the
    # flagged fraction along the run
    chunk = min(100, args.steps)
    ms = 0.0
    track = []
    prev = e0
    done = 0
    with clocks:
        while done < args.steps:
            n = min(chunk, args.steps - done)
            ev0.record()
            ens.step(n, dt=c["dt"], std_threshold=c["std_threshold"])
            ev1.record()
            torch.cuda.synchronize()
            ms += ev0.elapsed_time(ev1)
            done += n
            cur = ens.state()
            tot = cur["energy"] + cur["kinetic"]
            tot0 = e0["energy"] + e0["kinetic"]
            track.append({
                "step": done,
                "temperature_K": float(cur["temperature"].mean()),
                "flagged_fraction": float((cur["flagged"] - prev["flagged"])
                                          .sum() / (n * N)),
                "drift_ev_per_atom_mean": float(np.mean(tot - tot0) /
                                                c["n_atoms"]),
                "drift_ev_per_atom_max_abs": float(np.max(np.abs(tot - tot0))
                                                   / c["n_atoms"]),
                "median_std_over_sigma": float(np.median(cur["std"]))})
            prev = cur
    s1 = ens.state()
    stats = ens.stats()
    flagged = int(s1["flagged"].sum() - e0["flagged"].sum())
    drift = (s1["energy"] + s1["kinetic"]) - (e0["energy"] + e0["kinetic"])
    # up to 50 steps without graph replay (full, checked steps)
    n_full = min(args.steps, 50)
    ens.set_graphs(False)
    torch.cuda.synchronize()
    ev0.record()
    ens.step(n_full, dt=c["dt"], std_threshold=c["std_threshold"])
    ev1.record()
    torch.cuda.synchronize()
    ms_full = ev0.elapsed_time(ev1)
    ens.set_graphs(True)
    before = ens.state()
    ens.step(1, dt=c["dt"], std_threshold=c["std_threshold"])
    flag_before = float((ens.state()["flagged"] - before["flagged"]).sum() / N)
    grow = ens.grow_sparse_set(c["n_grow"])
    torch.cuda.synchronize()
    before = ens.state()
    ev0.record()
    ens.step(1, dt=c["dt"], std_threshold=c["std_threshold"])
    ev1.record()
    torch.cuda.synchronize()
    ms_after = ev0.elapsed_time(ev1)
    flag_after = float((ens.state()["flagged"] - before["flagged"]).sum() / N)
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_md_step()
        except Exception as ex:  # report, never hide
            cpu = {"error": repr(ex)}
    print(json.dumps({
        "metric": "MD ensemble atom-steps/s (forces + local std every step)",
        "value": N * args.steps / (ms * 1e-3), "unit": "atom-steps/s",
        "ms_per_step": ms / args.steps, "steps": args.steps,
        "warmup": max(args.warmup, 1), "precision": args.precision,
        "config": {"workload": "md3: %d replicas x 2000 atoms, 3 species "
                               "(0.5/0.3/0.2, 27/58/1 amu), 1200 K, dt 1 fs, "
                               "B2 [3,8,4] rc 5.5 (n_d 1500), %d sparse envs"
                               % (R, grow["sparse_before"]),
                   "replicas": R, "atoms": N},
        "seconds_for_1000_steps": ms / args.steps,
        "graph_replay": {"ms_per_step_replayed": ms / args.steps,
                         "ms_per_step_full": ms_full / n_full,
                         "counters_timed_region": stats},
        "flagged_atom_steps_per_step": flagged / args.steps,
        "flag_threshold_std_over_sigma": c["std_threshold"],
        "max_std_over_sigma": float(s1["max_std"].max()),
        "temperature_K": {"start": float(s0["temperature"].mean()),
                          "end": float(s1["temperature"].mean())},
        "total_energy_drift_ev_per_atom": {
            "mean": float(np.mean(drift) / c["n_atoms"]),
            "max_abs": float(np.max(np.abs(drift)) / c["n_atoms"])},
        "track": track,
        "sparse_update": grow,
        "flagged_fraction_step_before_update": flag_before,
        "flagged_fraction_step_after_update": flag_after,
        "ms_per_step_after_update": ms_after,
        "cpu_baseline": cpu,
        # the grown model's plan (the timed steps ran the 8,000-env model)
        "mixed_plan_after_update": (gp.mixed_plan()
                                    if args.precision == "mixed" else None),
        "autotune": autotune_table(),
        "setup_s": {"train_fp64": round(train_s, 1),
                    "replica_generation": round(gen_s, 1)},
        "clocks": clocks.summary(),
    }), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus if args.impl == "ours" else 0)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "fcc1m":
        run_fcc1m(args)
        return
    if args.workload == "fcc256":
        run_fcc256(args)
        return
    if args.workload == "md":
        run_md(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "mapped":
        run_mapped(args)
        return
    run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
