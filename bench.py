#!/usr/bin/env python
"""Benchmark of the GB300 PDOS indirect solver.

Default workload (single GPU): batched solving with a learned warm start on
the parametrised factor-model portfolio family -- n = 2,000 assets, k = 200
factors, F at 20 % density shared by the family (N = 2,201 variables,
m = 4,402 rows, about 86,400 nonzeros per instance); per instance
mu = mu0 + 0.1 N(0,1) and D scaled entrywise by U[0.8, 1.2]; EPS_ABS 1e-4,
FP32 storage with FP64 reductions; seeded synthetic data.  The warm-start
network (4000 -> 1024 -> 1024 -> 11005, BF16) is trained inside the run on
GPU-solver solutions of a reduced training set (16,384 instances, --train)
solved at EPS_ABS 1e-5.  One step = one batch of held-out instances (--batch):
network inference on the device-resident features, warm start, batched
ADMM until every instance passes the DIMACS test (instances that do not are
re-solved from the cold start).

JSON line (rank 0):
  value    solves/s of that step with problem data and features resident in
           HBM (device time, CUDA events), whole job over all ranks
  plain_gpu_admm  the same instances solved one at a time by the
           single-instance GPU engine from the cold start (problem resident)
  batched_cold    the batch from the cold start, no network
  e2e      solves/s through the public API with host buffers: batch set-up
           (H2D of every instance and device set-up), H2D of the features,
           inference, warm start, solve, D2H of every x, s, y
  roofline the batch kernel (the whole fused ADMM iteration; all of the
           solve's device time): algorithmic bytes of the products it ran
           (values and indices of A and A', pointers, gathered and written
           vectors) / its device time, against the measured HBM copy peak;
           the CG products alone are timed beside it (spmv_products), and
           the network's forward pass against the measured BF16 peak
           (network_forward: TMA-fed tcgen05 kernel; mma.sync beside it)
  cpu_baseline  the oracle (C restatement of the reference, 1 core) solving
           a few held-out instances from the cold start
--impl reference runs that CPU solver on all host cores instead.
Other workloads (--workload): the single-instance configurations
(portfolio_n200k_fp64 and its random-cone-split twin
portfolio_n200k_split_fp64, portfolio_n100_fp64, random_socp_m600k_fp32),
batches of uneven portfolio instances (portfolio_mix_batch, n <= 2,000; and
portfolio_uneven_full, n up to 20,000 at full size, set up in waves).
Multi-GPU (torchrun): batch workloads shard the instances across ranks (no
collective); single-instance workloads run replicas.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the BASELINE single-instance configuration (FP64 plain GPU ADMM)
    # NORMALIZE=0 is the reference binding's default; this seeded instance
    # reaches EPS 1e-4 in 1700 ADMM iterations (20 CG iterations each) on
    # the FP64 path, which follows the reference's iterate sequence; the CPU
    # arm extrapolates its per-iteration time with that count.
    "portfolio_n200k_fp64": dict(gen="portfolio", n=200_000, k=2_000, density=0.05, seed=1,
                                 precision="fp64", iters_per_solve=1700,
                                 params=dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                             MAX_ITERS=2000, NORMALIZE=0)),
    # the same instance with its second-order cone cut into cones of random
    # sizes U[2, 64] (6,126 small cones instead of one of 202,001 rows); it
    # reaches EPS 1e-4 in 1358 ADMM iterations on the FP64 path
    "portfolio_n200k_split_fp64": dict(gen="portfolio", n=200_000, k=2_000, density=0.05, seed=1,
                                       soc_split=True, precision="fp64", iters_per_solve=1358,
                                       params=dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                                   MAX_ITERS=2000, NORMALIZE=0)),
    # the small CPU-runnable case
    "portfolio_n100_fp64": dict(gen="portfolio", n=100, k=10, density=0.5, seed=0, precision="fp64",
                                params=dict(EPS_ABS=5e-3, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                            MAX_ITERS=2000, NORMALIZE=0)),
    # mixed precision random feasible SOCP, built around a known optimum; the
    # reference's own iteration needs thousands of ADMM iterations on this
    # family (1,307 at m = 6,000, 3,789 at m = 30,000) and does not converge
    # with NORMALIZE=1 within 4,000
    "random_socp_m600k_fp32": dict(gen="random", m=600_000, n=200_000, nnz_per_col=20, seed=2,
                                   precision="fp32", iters_per_solve=3146,  # the GPU solve's count
                                   params=dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                               MAX_ITERS=30000, NORMALIZE=0)),
}
# batched workloads (many instances per step)
_BATCH_PARAMS = dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4, MAX_ITERS=4000, NORMALIZE=0)
BATCH_WORKLOADS = {
    # parametrised family with the learned warm start (F shared, mu and D
    # perturbed per instance); the network is trained on 50,000 GPU
    # solutions at EPS 1e-5, as the configuration states
    "portfolio_family_warmstart": dict(kind="family", n=2000, k=200, density=0.2, seed=0,
                                       precision="fp32", batch=4096, train=50000, train_eps=1e-5,
                                       epochs=40, hidden=1024, params=_BATCH_PARAMS),
    # uneven instances: n ~ U[50, 2000], k = ceil(n/10), F at 20 %
    "portfolio_mix_batch": dict(kind="mix", batch=4096, n_lo=50, n_hi=2000, density=0.2, seed=2,
                                precision="fp32", params=_BATCH_PARAMS),
    # the uneven batch at its full size: 4,096 instances with n ~ U[50, 20,000]
    # (about 1.1e10 nonzeros), generated on the host cores and set up on the
    # device in waves of 256 instances, never all on the host at once
    "portfolio_uneven_full": dict(kind="mix_waves", batch=4096, n_lo=50, n_hi=20000, density=0.2, seed=3,
                                  precision="fp32", params=_BATCH_PARAMS, wave=256,
                                  # mean ADMM iterations of each n-decile in the batch's cold solve
                                  # (measured on one GB300), for the reference arm's extrapolation
                                  iters_by_decile=[291, 417, 491, 583, 636, 702, 758, 811, 865, 912]),
}
DEFAULT_WORKLOAD = "portfolio_family_warmstart"


def make_problem(wl):
    from pdos_gb300.generators import portfolio, random_feasible
    if wl["gen"] == "portfolio":
        return portfolio(wl["n"], wl["k"], wl["density"], seed=wl["seed"], params=wl["params"],
                         random_soc_split=wl.get("soc_split", False))
    return random_feasible(wl["m"], wl["n"], wl["nnz_per_col"], seed=wl["seed"], params=wl["params"])


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def committed_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of this
    workload (profiles/traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        d = json.load(fh)
    return d.get(workload, {}).get(kernel)


def batch_traffic(workload, algorithmic_bytes, kernel="batch_admm_kernel"):
    """DRAM bytes of the batch kernel over a solve: the committed ncu ratio of
    DRAM bytes to algorithmic bytes (a smaller launch of the same kernel)
    times this solve's algorithmic bytes, or None."""
    d = committed_traffic(workload, kernel)
    if not isinstance(d, dict) or "dram_bytes_per_algorithmic_byte" not in d:
        return None
    return d["dram_bytes_per_algorithmic_byte"] * algorithmic_bytes


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------ CPU oracle
def cpu_sample(prob, sample_iters):
    """Time the oracle (the reference's algorithm in C, 1 core): set-up only,
    then set-up + `sample_iters` ADMM iterations."""
    from oracle import oracle as O
    O.build_port()
    t0 = time.perf_counter()
    O.port_solve(prob.with_params(MAX_ITERS=0))
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.port_solve(prob.with_params(MAX_ITERS=sample_iters))
    t_all = time.perf_counter() - t0
    t_iter = max(t_all - t_setup, 1e-9) / sample_iters
    return t_setup, t_iter


def cpu_solves_per_s(t_setup, t_iter, iters_per_solve):
    return 1.0 / (t_setup + t_iter * iters_per_solve)


# --------------------------------------------------------------- helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def spmv_bytes(prob, which, sv):
    """Algorithmic bytes of one launch of a CG SpMV kernel: matrix values and
    4-byte indices, the gathered vector once, 8 bytes of per-row layout data
    (length and row id), and the epilogue's element-wise streams.  Padding
    and split-row partial sums are overhead, not counted."""
    nnz, m, N = prob.nnz, prob.m, prob.n
    if which == 0:  # u = A p: gather p (N), write u (m)
        return nnz * (sv + 4) + N * sv + m * sv + 8 * m
    # t = p + A'u: gather u (m), read p, write t (N)
    return nnz * (sv + 4) + m * sv + 2 * N * sv + 8 * N


def single_instance_spmv(device, reps=20):
    """The single-instance FP64 engine's SpMV kernels on the n = 200,000
    portfolio (k = 2,000, F at 5 %: 20.6M nonzeros, A and A' 0.5 GB, far
    above L2), timed with CUDA events on the workspace stream, against two
    ceilings: the measured HBM copy rate and the device's FP64 FMA rate
    (one FMA per nonzero), both expressed in GB/s of the kernel's
    algorithmic bytes."""
    from pdos_gb300.solver import Workspace, fp64_fma_rate
    wl = WORKLOADS["portfolio_n200k_fp64"]
    prob = make_problem(wl)
    fma = fp64_fma_rate(device)
    peak, peak_kind = measured_peaks()
    out = {"workload": "portfolio_n200k_fp64", "nnz": prob.nnz, "n_vars": prob.n, "m_rows": prob.m,
           "fp64_fma_per_s": fma, "hbm_peak_gbs": peak, "hbm_peak_kind": peak_kind}
    with Workspace(prob, "fp64", device=device) as w:
        for which, name in ((4, "u = A p"), (5, "t = p + A'u")):
            ms = w.time_kernel(which, reps)
            pass_ms = w.time_kernel(which - 4, reps)
            nbytes = spmv_bytes(prob, which - 4, 8)
            achieved = nbytes / (ms / 1e3) / 1e9
            fp64_gbs = nbytes / (prob.nnz / fma) / 1e9
            ceiling = min(peak, fp64_gbs)
            out["sell_spmv_kernel<%s>" % ("OpCgA" if which == 4 else "OpCgAt")] = {
                "product": name, "ms_per_launch": ms, "pass_ms_with_combine": pass_ms, "bytes_per_launch": nbytes,
                "achieved_gbs": achieved, "frac_of_hbm": achieved / peak,
                "fp64_fma_ceiling_gbs": fp64_gbs, "frac_of_fp64_fma_ceiling": achieved / fp64_gbs,
                "frac_of_min_ceiling": achieved / ceiling,
                "bound_by": "hbm" if peak <= fp64_gbs else "fp64 fma"}
    return out


def run_reference(args, wl, prob):
    """--impl reference: the reference's CPU algorithm (oracle) on this
    workload, bounded sample per step, all cores it can use (1: a single
    PDOS solve is sequential)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    iters_hint = wl.get("iters_per_solve")
    t_setups, t_iters = [], []
    sample_iters = args.cpu_iters
    for _ in range(args.warmup + args.steps):
        ts, ti = cpu_sample(prob, sample_iters)
        t_setups.append(ts)
        t_iters.append(ti)
    ts = float(np.median(t_setups[args.warmup:]))
    ti = float(np.median(t_iters[args.warmup:]))
    iters = iters_hint or prob.params["MAX_ITERS"]
    val = cpu_solves_per_s(ts, ti, iters)
    line = {
        "impl": "reference", "metric": single_metric(wl), "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 / val, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": config_of(args, wl, prob),
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": 1, "kind": "port",
                         "sample": f"set-up + {sample_iters} ADMM iterations per step, "
                                   f"extrapolated to {iters} iterations per solve"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_seconds_per_admm_iteration": ti, "cpu_setup_seconds": ts,
    }
    print(json.dumps(line))
    return 0


def single_metric(wl):
    """The single-instance workloads' metric, at the workload's own EPS_ABS."""
    return ("solves/s at EPS_ABS %g (plain GPU ADMM, single instance); SpMV HBM GB/s"
            % wl["params"]["EPS_ABS"])


def config_of(args, wl, prob):
    return {"workload": args.workload, "n_vars": prob.n, "m_rows": prob.m, "nnz": prob.nnz,
            "cones": {"f": prob.f, "l": prob.l, "q_count": int(len(prob.q)),
                      "q_max": int(max(prob.q)) if len(prob.q) else 0},
            "precision": wl["precision"], "params": wl["params"],
            "l2": ("inputs larger than L2: A and A' are %.0f MB resident in HBM, re-read by "
                   "every SpMV (129 MB L2)" % (2 * prob.nnz * (12 if wl["precision"] == "fp64" else 8) / 1e6))
            if 2 * prob.nnz * 8 > 129e6 else "small problem (L2-resident)",
            "parallelism": f"replicas x{args.gpus}"}


# ================================================================ batches
BATCH_METRIC = ("solves/s at EPS_ABS 1e-4: batched + learned warm start (one GPU), "
                "beside plain single-instance GPU ADMM; SpMV HBM GB/s")
MIX_METRIC = ("solves/s at EPS_ABS 1e-4: batched uneven instances, cold start (one GPU), "
              "beside plain single-instance GPU ADMM; SpMV HBM GB/s")


def batch_metric(wl):
    return BATCH_METRIC if wl["kind"] == "family" else MIX_METRIC


def batch_draws(wl, count, rank):
    """The random draws behind this rank's held-out instances (cheap)."""
    from pdos_gb300 import generators as g
    if wl["kind"] == "family":
        fam = g.PortfolioFamily(wl["n"], wl["k"], wl["density"], seed=wl["seed"])
        mus, ds = fam.draw(count, seed=wl["seed"] + 1000 + rank)
        return {"fam": fam, "mus": mus, "ds": ds}
    return {"sizes": g.portfolio_batch_sizes(count, wl["n_lo"], wl["n_hi"], seed=wl["seed"] + rank),
            "seed": (wl["seed"] + rank) * 1_000_003}


def batch_problem(d, wl, i):
    from pdos_gb300 import generators as g
    if "fam" in d:
        return d["fam"].instance(d["mus"][i], d["ds"][i], wl["params"])
    n, k = d["sizes"][i]
    return g.portfolio(n, k, wl["density"], seed=d["seed"] + i, params=wl["params"])


def batch_instances(wl, count, rank, world=1):
    """(family or None, mus, ds, problems) of this rank's held-out instances:
    the shard (pdos_gb300.shard, balanced by nonzeros) of a list of
    count * world instances."""
    from pdos_gb300.shard import shard_instances
    d = batch_draws(wl, count * world, 0)
    if "fam" in d:
        costs = [1] * (count * world)
    else:
        costs = [n * (3 + wl["density"] * k) + 2 * k for n, k in d["sizes"]]
    idx = shard_instances(costs, world, rank)
    probs = [batch_problem(d, wl, i) for i in idx]
    if "fam" in d:
        return d["fam"], d["mus"][idx], d["ds"][idx], probs
    return None, None, None, probs


def product_bytes(probs, infos, sv):
    """Algorithmic bytes of every product a batch solve ran: per instance,
    A passes = prep + CG + post, A' passes = tops (one more when solved) +
    CG; each pass reads values and indices once (the batch layout's indices
    are local to an instance and 16-bit), its pointer array, the gathered
    vector(s) once and writes its result."""
    total = 0.0
    for p, d in zip(probs, infos):
        nnz, m, N = p.nnz, p.m, p.n
        it, cg = d["admm_iters"], d["cg_iters"]
        b_ax = nnz * (sv + 2) + (m + 1) * 4 + N * sv + m * sv
        b_at = nnz * (sv + 2) + (N + 1) * 4 + m * sv + N * sv
        tops = it + (1 if d["solved"] else 0)
        total += (1 + cg + it) * b_ax + (cg + tops) * b_at + tops * m * sv  # top gathers y and u
    return total


def cpu_family_sample(probs, count):
    """Oracle (C restatement of the reference, 1 core) cold solves of the
    first `count` instances: (solves/s, seconds)."""
    from oracle import oracle as O
    O.build_port()
    t0 = time.perf_counter()
    for p in probs[:count]:
        O.port_solve(p)
    dt = time.perf_counter() - t0
    return count / dt, dt


# the FP64 oracle of the benchmark spec: the reference's indirect algorithm (C
# restatement) solved to EPS_ABS 1e-8 with CG tightened to the point where
# it matches the reference's direct LDL solver
TIGHT_ORACLE = dict(EPS_ABS=1e-8, MAX_ITERS=100000, CG_MAX_ITS=200, CG_TOL=1e-12)


def _oracle_objective(prob):
    from oracle import oracle as O
    r = O.port_solve(prob.with_params(**TIGHT_ORACLE))
    return float(prob.c @ r["x"]), r["status"]


class OracleCheck:
    """FP64-oracle objectives of `count` held-out instances spread evenly over
    the batch, solved in a spawn pool on the host cores while the GPU trains
    the network; wait() joins the pool, and is called before any timed
    region so that no oracle process competes with the timed work."""

    def __init__(self, probs, count, workers):
        import multiprocessing as mp
        from oracle import oracle as O
        O.build_port()
        self.idx = np.unique(np.linspace(0, len(probs) - 1, count).round().astype(int))
        self.workers = workers
        self.t0 = time.perf_counter()
        self.pool = mp.get_context("spawn").Pool(workers)
        self.pending = self.pool.map_async(_oracle_objective, [probs[i] for i in self.idx], chunksize=1)
        self.result = None

    def wait(self):
        if self.result is None:
            self.result = self.pending.get()
            self.pool.close()
            self.pool.join()
            self.seconds = time.perf_counter() - self.t0
        return self.result

    def errors(self, probs, xs_stacked):
        """Relative objective errors of stacked solutions against the oracle."""
        res = self.wait()
        starts = np.concatenate([[0], np.cumsum([p.n for p in probs])])
        err = []
        for i, (obj, _) in zip(self.idx, res):
            got = float(probs[i].c @ xs_stacked[starts[i]:starts[i + 1]])
            err.append(abs(got - obj) / max(1.0, abs(obj)))
        return np.array(err)

    def summary(self, probs, xs_stacked):
        err = self.errors(probs, xs_stacked)
        return {"instances": int(len(err)), "max_relative_objective_error": float(err.max()),
                "median_relative_objective_error": float(np.median(err)),
                "within_1e-3": int((err <= 1e-3).sum()),
                "oracle_solved": int(sum(st == "Solved" for _, st in self.result))}


def _cpu_worker(job):
    idx, wl_name, count = job
    wl = BATCH_WORKLOADS[wl_name]
    from oracle import oracle as O
    O.port_solve(batch_problem(batch_draws(wl, count, 0), wl, idx))
    return idx


def profile_batch(args, wl):
    """Profiling case, the kernels of one step: --batch instances (default
    64); for the family workload an untrained network's inference and the
    warm start from it; then one launch of the batch kernel running
    --profile-iters ADMM iterations."""
    import torch
    from pdos_gb300 import build
    build.build()
    from pdos_gb300.solver import Batch
    fam, mus, ds, probs = batch_instances(wl, args.batch or 64, 0)
    with Batch(probs, precision=wl["precision"], iters_per_launch=args.profile_iters,
               share_layouts=not args.own_layouts) as b:
        if args.blocks:  # the CTA size of each class, as the tuner would set it
            b.set_blocks([int(v) for v in args.blocks.split(",")])
        if fam is not None:
            from pdos_gb300.warmstart import FamilyWarmStart
            ws = FamilyWarmStart(fam, hidden=wl["hidden"], max_batch=len(probs), seed=0)
            ws.net.set_kernel(args.network_kernel)
            f = np.concatenate([mus, ds], axis=1)
            ws.in_mean, ws.in_std = f.mean(axis=0), np.maximum(f.std(axis=0), 1e-12)
            ws.out_mean = np.zeros(ws.n_out)
            ws.out_std = np.full(ws.n_out, 1e-3)
            x0, y0, s0 = ws.predict_device(mus, ds)
            b.warm_start(x0.data_ptr(), y0.data_ptr(), s0.data_ptr())
            ws.net.close()
        b.launch(1)
        torch.cuda.synchronize()
        inf = b.infos()
        print(json.dumps({"instances": len(probs), "admm_iterations": max(d["admm_iters"] for d in inf),
                          "cg_iterations": int(sum(d["cg_iters"] for d in inf)),
                          "algorithmic_bytes_of_launch": product_bytes(
                              probs, inf, 8 if wl["precision"] == "fp64" else 4)}))
    return 0


def run_batch_reference(args, wl):
    """--impl reference on a batch workload: the reference's CPU algorithm
    (the oracle, 1 thread per process) on every host core, one held-out
    instance per core per step, cold start as the reference has no other."""
    import multiprocessing as mp
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    if wl["kind"] == "mix_waves":
        return run_uneven_reference(args, wl)
    from oracle import oracle as O
    O.build_port()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    rates = []
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            count = args.batch or wl["batch"]
            jobs = [((step * cores + j) % count, args.workload, count) for j in range(cores)]
            t0 = time.perf_counter()
            pool.map(_cpu_worker, jobs)
            rates.append(cores / (time.perf_counter() - t0))
    val = float(np.median(rates[args.warmup:]))
    line = {
        "impl": "reference", "metric": batch_metric(wl), "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cores / val,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "config": {"workload": args.workload, "instances_per_step": cores,
                                                 "params": wl["params"]},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x 1 held-out instance per step (cold start)"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def decile_samples(sizes):
    """n-decile of every instance and the first instance of each decile."""
    ns = np.array([n for n, _ in sizes])
    edges = np.quantile(ns, np.linspace(0, 1, 11))
    decile = np.clip(np.searchsorted(edges, ns, side="right") - 1, 0, 9)
    samples = {int(np.nonzero(decile == d)[0][0]): d for d in range(10) if (decile == d).any()}
    return ns, decile, samples


def _cpu_gen_iter_sample(job):
    n, k, density, seed, params, iters = job
    from pdos_gb300 import generators as g
    return cpu_sample(g.portfolio(n, k, density, seed=seed, params=params), iters)


def stratified_cpu_estimate(wl, sizes, iters_of, per_decile, cpu_iters, pool, seed=7):
    """The oracle's time for a whole uneven batch, from a seeded stratified
    subsample: up to `per_decile` instances of every n-decile (regenerated
    from their seeds in the pool's processes), each timed for set-up plus
    `cpu_iters` ADMM iterations and extrapolated to `iters_of(i, d)`
    iterations; a decile's mean time counts once per instance of the decile.
    Returns (total seconds, per-decile summary, instances sampled)."""
    ns, decile, _ = decile_samples(sizes)
    rng = np.random.default_rng(seed)
    picks = []
    for d in range(10):
        members = np.nonzero(decile == d)[0]
        if len(members) == 0:
            continue
        take = members if len(members) <= per_decile else np.sort(rng.choice(members, per_decile, replace=False))
        picks += [(int(i), d) for i in take]
    seed0 = wl["seed"] * 1_000_003
    jobs = [(sizes[i][0], sizes[i][1], wl["density"], seed0 + i, wl["params"], cpu_iters) for i, _ in picks]
    res = pool.map(_cpu_gen_iter_sample, jobs, chunksize=1)
    times = {d: [] for d in range(10)}
    steps = {d: [] for d in range(10)}
    for (i, d), (ts, ti) in zip(picks, res):
        it = float(iters_of(i, d))
        times[d].append(ts + ti * it)
        steps[d].append(ti)
    total, per = 0.0, {}
    for d in range(10):
        if not times[d]:
            continue
        members = int((decile == d).sum())
        total += float(np.mean(times[d])) * members
        per[d] = {"instances": members, "sampled": len(times[d]),
                  "n_range": [int(ns[decile == d].min()), int(ns[decile == d].max())],
                  "mean_seconds_per_solve": float(np.mean(times[d])),
                  "mean_s_per_admm_iteration": float(np.mean(steps[d]))}
    return total, per, len(picks)


def run_uneven_reference(args, wl):
    """--impl reference on the full-size uneven batch, where one reference
    solve of the largest instances takes minutes: every step times the
    oracle (1 thread per process, all host cores) on one instance per
    n-decile, set-up plus --cpu-iters ADMM iterations, and extrapolates each
    decile with its measured mean iteration count (iters_by_decile); the
    value is the batch's instances over the summed solve time, spread over
    the cores."""
    import multiprocessing as mp
    from pdos_gb300 import generators as g
    from oracle import oracle as O
    O.build_port()
    count = args.batch or wl["batch"]
    sizes = g.portfolio_batch_sizes(count, wl["n_lo"], wl["n_hi"], seed=wl["seed"])
    cores = os.cpu_count() or 1
    rates = []
    with mp.get_context("spawn").Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            total, _, sampled = stratified_cpu_estimate(
                wl, sizes, lambda i, d: wl["iters_by_decile"][d], args.cpu_per_decile, args.cpu_iters, pool,
                seed=7 + step)
            rates.append(cores * count / total)
    val = float(np.median(rates[args.warmup:]))
    line = {
        "impl": "reference", "metric": batch_metric(wl), "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * count / val,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "config": {"workload": args.workload, "instances_per_step": count,
                                                 "n_range": [wl["n_lo"], wl["n_hi"]], "params": wl["params"]},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"oracle on a stratified subsample of {sampled} instances (up to "
                                   f"{args.cpu_per_decile} per n-decile) per step, set-up + {args.cpu_iters} "
                                   f"ADMM iterations each, extrapolated with each decile's measured mean "
                                   f"iteration count, weighted by its instances, spread over {cores} cores"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _gen_mix_instance(job):
    n, k, density, seed, params = job
    from pdos_gb300 import generators as g
    return g.portfolio(n, k, density, seed=seed, params=params)


def _portfolio_shape(n, k, density):
    """(N, m, nnz) of a portfolio instance (pdos_gb300.generators.portfolio)."""
    per_row = min(max(int(round(density * k)), 0), k)
    return n + k + 1, 2 * n + 2 * k + 2, n * (3 + per_row) + 2 * k + 1


def run_batch_waves(args, wl):
    """The uneven batch at full size (about 1.1e10 nonzeros): instances are
    generated in a spawn pool on the host cores, one wave ahead of the wave
    being appended (pdosgpu_batch_append), so that at most two waves of
    problem data exist on the host; one cold-start solve is timed (a solve
    takes minutes, so the step count is 1).  The CPU baseline and the FP64
    checks run on one sampled instance per n-decile."""
    import multiprocessing as mp
    import torch
    from pdos_gb300 import build, generators as g
    build.build()
    from pdos_gb300.solver import Batch, Workspace
    ws_n, rank, local = dist_env()
    torch.cuda.set_device(local)
    count = args.batch or wl["batch"]
    prec = wl["precision"]
    sv = 8 if prec == "fp64" else 4
    sizes = g.portfolio_batch_sizes(count, wl["n_lo"], wl["n_hi"], seed=wl["seed"])
    seed0 = wl["seed"] * 1_000_003
    jobs = [(n, k, wl["density"], seed0 + i, wl["params"]) for i, (n, k) in enumerate(sizes)]
    shapes = [_portfolio_shape(n, k, wl["density"]) for n, k in sizes]
    ns, decile, samples = decile_samples(sizes)
    kept = {}
    cores = os.cpu_count() or 2
    pool = mp.get_context("spawn").Pool(max(1, cores - 1))
    W = wl["wave"]
    wave_idx = [list(range(w, min(count, w + W))) for w in range(0, count, W)]
    t_gen = [0.0]

    def waves():
        pending = pool.map_async(_gen_mix_instance, [jobs[i] for i in wave_idx[0]], chunksize=1)
        for w, idx in enumerate(wave_idx):
            t0 = time.perf_counter()
            probs = pending.get()
            t_gen[0] += time.perf_counter() - t0
            if w + 1 < len(wave_idx):
                pending = pool.map_async(_gen_mix_instance, [jobs[i] for i in wave_idx[w + 1]], chunksize=1)
            for i, p in zip(idx, probs):
                if i in samples:
                    kept[i] = p
            yield probs
            del probs

    t0 = time.perf_counter()
    batch = Batch.in_waves(waves(), precision=prec, device=local)
    t_setup_wall = time.perf_counter() - t0
    blocks = batch.tune(2)
    stream = torch.cuda.ExternalStream(batch.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    batch.reset()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        batch.solve()
        ev1.record(stream)
        ev1.synchronize()
    solve_ms = ev0.elapsed_time(ev1)
    t0 = time.perf_counter()
    x, s_, y, inf = batch.fetch_all()
    t_fetch = time.perf_counter() - t0
    launches = inf[0]["kernel_launches"]
    value = count / (solve_ms / 1e3)

    class _Shape:
        def __init__(self, N, m, nnz):
            self.n, self.m, self.nnz = N, m, nnz
    shp = [_Shape(*sh) for sh in shapes]
    roof_bytes = product_bytes(shp, inf, sv)
    peak, peak_kind = measured_peaks()
    pm, pb = batch.time_products(1)
    achieved = roof_bytes / (solve_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "batch_admm_kernel / batch_cluster_kernel (whole fused ADMM "
                                          "iteration per CTA; instances too large for one CTA's shared "
                                          "memory on a cluster of 2 to 8 CTAs)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "traffic": batch_traffic(args.workload, roof_bytes, "batch_cluster_kernel"),
                "algorithmic_bytes_of_solve": roof_bytes, "ms_of_solve": solve_ms,
                "spmv_products": {"kernel": "batch_products_kernel (u = A p, t = p + A'u)",
                                  "achieved": pb / (pm / 1e3) / 1e9, "ms": pm, "bytes": pb,
                                  "frac": pb / (pm / 1e3) / 1e9 / peak}}
    cls = batch.classes()
    iters = np.array([d["admm_iters"] for d in inf])
    starts_x = np.concatenate([[0], np.cumsum([sh[0] for sh in shapes])])

    # CPU baseline: the oracle (1 core per process) on a seeded stratified
    # subsample (up to --cpu-per-decile instances per n-decile), set-up plus
    # a few ADMM iterations each, extrapolated with the iteration count the
    # GPU solve needed for that instance and weighted by the instances of
    # its decile
    cpu = None
    if not args.no_cpu:
        t0 = time.perf_counter()
        total, per, sampled = stratified_cpu_estimate(wl, sizes, lambda i, d: iters[i], args.cpu_per_decile,
                                                      args.cpu_iters, pool)
        cpu_secs = time.perf_counter() - t0
        cpu = {"value": count / total, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"oracle (C restatement, 1 core per process): a stratified subsample of {sampled} "
                         f"instances (up to {args.cpu_per_decile} per n-decile), set-up + {args.cpu_iters} "
                         f"ADMM iterations each, extrapolated with that instance's GPU iteration count and "
                         f"weighted by its decile's instances ({cpu_secs:.0f} s of sampling)",
               "deciles": per}
    pool.close()
    pool.join()

    # FP64 checks of the FP32 results on the sampled instances: the
    # single-instance FP64 GPU engine at EPS 1e-7 for every decile, and the
    # CPU oracle at EPS 1e-8 (CG 200, 1e-12) for the smallest sample
    checks = []
    for i in sorted(kept):
        p = kept[i]
        got = float(p.c @ x[starts_x[i]:starts_x[i + 1]])
        with Workspace(p.with_params(EPS_ABS=1e-7, MAX_ITERS=30000, CG_MAX_ITS=40, CG_TOL=1e-10),
                       "fp64", device=local) as w1:
            r = w1.solve().fetch()
        ref = float(p.c @ r["x"])
        checks.append({"n": int(ns[i]), "class": int(cls[i]), "batch_iters": int(iters[i]),
                       "fp64_status": r["status"],
                       "relative_objective_error": abs(got - ref) / max(1.0, abs(ref))})
    small = min(kept, key=lambda i: ns[i])
    if not args.no_cpu:
        from oracle import oracle as O
        hi = O.port_solve(kept[small].with_params(**TIGHT_ORACLE))
        ref = float(kept[small].c @ hi["x"])
        got = float(kept[small].c @ x[starts_x[small]:starts_x[small + 1]])
        oracle_small = {"n": int(ns[small]), "relative_objective_error": abs(got - ref) / max(1.0, abs(ref))}
    else:
        oracle_small = None

    h2d = sum(sh[2] * 16 + (sh[0] + 1) * 8 + (sh[1] + sh[0]) * 8 + 8 for sh in shapes)
    d2h = sum((sh[0] + 2 * sh[1]) * 8 for sh in shapes)
    e2e_s = batch.append_seconds + batch.commit_seconds + solve_ms / 1e3 + t_fetch
    total_nnz = int(sum(sh[2] for sh in shapes))
    line = {
        "metric": MIX_METRIC, "value": value, "unit": "solves/s", "n_gpus": ws_n, "steps": 1, "warmup": 0,
        "ms_per_step": solve_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 reductions)" if sv == 4 else "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "instances_per_step": count, "nnz_per_step": total_nnz,
                   "n_range": [wl["n_lo"], wl["n_hi"]], "precision": prec, "params": wl["params"],
                   "waves_of_instances": W, "cta_sizes_by_class": blocks,
                   "instances_by_class": [int(sum(1 for c in cls if c == k)) for k in range(5)],
                   "l2": "inputs larger than L2: %.0f GB of A and A' resident in HBM" %
                         (total_nnz * 2 * (sv + 2) / 1e9),
                   "parallelism": "one GPU"},
        "solved": int(sum(d["solved"] for d in inf)), "admm_iterations_mean": float(iters.mean()),
        "admm_iterations_max": int(iters.max()),
        "setup": {"append_seconds": batch.append_seconds, "commit_seconds": batch.commit_seconds,
                  "generation_wait_seconds": t_gen[0], "wall_seconds": t_setup_wall},
        "fp64_checks": checks, "oracle_check_smallest": oracle_small,
        "roofline": roofline, "cpu_baseline": cpu,
        "e2e": {"value": count / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "seconds_per_step": e2e_s,
                "path": "pdosgpu_batch_append of every wave from host arrays (generation excluded), commit, "
                        "solve, pdosgpu_batch_fetch"},
        "gpu_launches": int(launches), "clocks": clk.summary(),
    }
    print(json.dumps(line))
    batch.close()
    return 0


def run_batch(args, wl):
    import torch
    ws_n, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws_n > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    from pdos_gb300 import build
    build.build()
    from pdos_gb300.solver import Batch, Workspace
    from pdos_gb300.warmstart import FamilyWarmStart, solve_family

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    B = args.batch or wl["batch"]
    prec = wl["precision"]
    sv = 8 if prec == "fp64" else 4
    fam, mus, ds, probs = batch_instances(wl, B, rank, ws_n)
    B = len(probs)
    info = {"instances_per_rank": B}
    # the FP64 oracle on a spread of held-out instances, on the host cores
    # while the GPU trains (joined before the first timed region)
    check = None
    if rank == 0 and not args.no_cpu and args.oracle_instances > 0:
        check = OracleCheck(probs, args.oracle_instances, max(1, (os.cpu_count() or 2) - 1))

    # ---- learned warm start: training set solved by the GPU batch solver
    wsn = None
    if fam is not None:
        n_train = args.train if args.train is not None else wl["train"]
        tmus, tds = fam.draw(n_train, seed=wl["seed"] + 11)
        t0 = time.perf_counter()
        tparams = dict(wl["params"], EPS_ABS=wl["train_eps"])
        if pg:  # each rank solves its part of the training set; every rank gets all of it
            from pdos_gb300.shard import all_gather_rows, shard_instances
            mine = shard_instances([1] * n_train, ws_n, rank)
            X, Y, S, tinf = solve_family(fam, tmus[mine], tds[mine], tparams, prec, device=local)
            X, Y, S = (all_gather_rows(a, mine, n_train, pg, device="cuda") for a in (X, Y, S))
            ok = torch.tensor([sum(d["solved"] for d in tinf)], device="cuda")
            pg.all_reduce(ok)
            n_solved = int(ok.item())
        else:
            X, Y, S, tinf = solve_family(fam, tmus, tds, tparams, prec, device=local)
            n_solved = int(sum(d["solved"] for d in tinf))
        t_data = time.perf_counter() - t0
        wsn = FamilyWarmStart(fam, hidden=wl["hidden"], max_batch=B, seed=0)
        t0 = time.perf_counter()
        hist = wsn.fit(tmus, tds, X, Y, S, epochs=wl["epochs"], batch=256, lr=1e-3)
        t_fit = time.perf_counter() - t0
        info["training"] = {"instances": n_train, "eps_abs": wl["train_eps"],
                            "solved": n_solved, "data_seconds": t_data,
                            "split": f"training-data solve sharded over {ws_n} rank(s), gathered on every "
                                     "rank; the fit runs on every rank from the same data and seed",
                            "epochs": wl["epochs"], "batch": 256, "fit_seconds": t_fit,
                            "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1],
                            "network": f"{wsn.n_in} -> {wl['hidden']} -> {wl['hidden']} -> {wsn.n_out}, "
                                       "BF16 weights, FP32 accumulation"}
        del X, Y, S

    if check is not None:
        check.wait()  # no oracle process runs during the timed regions
    batch = Batch(probs, precision=prec, device=local, share_layouts=not args.own_layouts)
    layout_groups, layout_members, layout_bytes = batch.layouts()
    blocks = batch.tune(4)
    stream = torch.cuda.ExternalStream(batch.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # ---- batched cold start (one warm-up, one timed solve)
    batch.reset().solve()
    batch.reset()
    barrier()
    ev0.record(stream)
    batch.solve()
    ev1.record(stream)
    ev1.synchronize()
    cold_ms = ev0.elapsed_time(ev1)
    cold_inf = batch.infos()
    roof_bytes = product_bytes(probs, cold_inf, sv)
    cold_check = check.summary(probs, batch.fetch_all()[0]) if check is not None else None

    # ---- the step: inference on resident features, warm start, solve
    if wsn is not None:
        feats = torch.from_numpy(wsn.features(mus, ds)).cuda()
        mean = torch.from_numpy(wsn.out_mean.astype(np.float32)).cuda()
        std = torch.from_numpy(wsn.out_std.astype(np.float32)).cuda()
        N, m = wsn.N, wsn.m
        x0 = torch.empty(B * N, dtype=torch.float64, device="cuda")
        y0 = torch.empty(B * m, dtype=torch.float64, device="cuda")
        s0 = torch.empty(B * m, dtype=torch.float64, device="cuda")

    fallbacks = [0]

    def step():
        if wsn is not None:
            wsn.net.predict_start(feats, mean, std, N, m, x0, y0, s0)
            batch.warm_start(x0.data_ptr(), y0.data_ptr(), s0.data_ptr())
        else:
            batch.reset()
        batch.solve()
        inf = batch.infos()
        bad = [i for i, d in enumerate(inf) if not d["solved"]]
        if bad and wsn is not None:  # cold-start fallback
            fallbacks[0] += len(bad)
            with Batch([probs[i] for i in bad], precision=prec, device=local) as fb:
                fb.solve()
        return inf

    for _ in range(args.warmup):
        step()
    launches0 = batch.infos()[0]["kernel_launches"]
    fallbacks[0] = 0
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            warm_inf = step()
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    dev_ms = ev0.elapsed_time(ev1)
    launches = batch.infos()[0]["kernel_launches"] - launches0
    if wsn is not None:
        launches += args.steps * 6  # conversion, 3 products, scatter, warm-start scaling
    if pg:
        t = torch.tensor([dev_ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        dev_ms = float(t.item())
    value = ws_n * B * args.steps / (dev_ms / 1e3)

    # ---- roofline: the fused batch kernel over the cold solve; products alone
    peak, peak_kind = measured_peaks()
    achieved = roof_bytes / (cold_ms / 1e3) / 1e9
    pm, pb = batch.time_products(4)
    roofline = {"bound": "hbm", "kernel": "batch_pair_kernel / batch_admm_kernel (whole fused ADMM "
                                          "iteration per CTA; family instances two per CTA where their "
                                          "vectors fit twice in shared memory)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind,
                "traffic": batch_traffic(args.workload, roof_bytes, "batch_pair_kernel")
                or batch_traffic(args.workload, roof_bytes),
                "algorithmic_bytes_per_solve_of_batch": roof_bytes, "ms_per_solve_of_batch": cold_ms,
                "spmv_products": {"kernel": "batch_products_kernel (u = A p, t = p + A'u)",
                                  "achieved": pb / (pm / 1e3) / 1e9, "ms": pm, "bytes": pb,
                                  "frac": pb / (pm / 1e3) / 1e9 / peak},
                "layouts": {"family_groups": layout_groups, "instances_on_shared_layouts": layout_members,
                            "layout_bytes": layout_bytes,
                            "note": "instances of one family share one matrix layout (values that differ "
                                    "per instance kept apart); algorithmic bytes still count every "
                                    "instance's matrix once per product, as the survey's B_Ax/B_Aty "
                                    "do, so a shared, L2-resident matrix can put `achieved` near or "
                                    "above the copy rate -- `traffic` is the DRAM side"}}
    if wsn is not None:
        fms, ffl = wsn.net.time_forward(B, 10)
        tf_peak = None
        path = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(path):
            with open(path) as fh:
                tf_peak = json.load(fh).get("bf16_tflops")
        roofline["network_forward"] = {"bound": "tensor", "achieved": ffl / (fms / 1e3) / 1e12,
                                       "unit": "TFLOP/s", "peak": tf_peak, "ms": fms,
                                       "kernel": "gemm_nt_tma_kernel (TMA 128-byte swizzled tiles, "
                                                 "tcgen05.mma 128x256x16, TMEM accumulators)"}
        wsn.net.set_kernel(0)  # the mma.sync kernel beside it (same results)
        tms, tfl = wsn.net.time_forward(B, 10)
        wsn.net.set_kernel(2)
        roofline["network_forward_mma_sync"] = {"bound": "tensor", "achieved": tfl / (tms / 1e3) / 1e12,
                                                "unit": "TFLOP/s", "peak": tf_peak, "ms": tms,
                                                "kernel": "gemm_nt_kernel (mma.sync m16n8k16 BF16)"}

    # ---- the single-instance engine's SpMV (the reference's CSR/CSC product
    # pair in FP64) on the n = 200,000 portfolio, beside its two ceilings
    spmv = None
    if rank == 0 and not args.no_spmv:
        spmv = single_instance_spmv(local)

    # ---- the same instances in the reference's arithmetic: an FP64 batch
    # (FP64 storage, products and reductions) from the cold start, its CG
    # products alone beside it, its results against the FP64 oracle
    batched_fp64 = None
    if not args.no_fp64 and sv == 4:
        with Batch(probs, precision="fp64", device=local, share_layouts=not args.own_layouts) as b64:
            blocks64 = b64.tune(2)
            b64.reset()
            s64 = torch.cuda.ExternalStream(b64.stream)
            barrier()
            ev0.record(s64)
            b64.solve()
            ev1.record(s64)
            ev1.synchronize()
            ms64 = ev0.elapsed_time(ev1)
            inf64 = b64.infos()
            pm64, pb64 = b64.time_products(2)
            batched_fp64 = {
                "value": ws_n * B / (ms64 / 1e3), "unit": "solves/s", "precision": "fp64",
                "cta_sizes_by_class": blocks64,
                "admm_iterations_mean": float(np.mean([d["admm_iters"] for d in inf64])),
                "solved": int(sum(d["solved"] for d in inf64)),
                "spmv_products": {"achieved": pb64 / (pm64 / 1e3) / 1e9, "unit": "GB/s", "ms": pm64,
                                  "bytes": pb64},
                "objective_error_vs_fp64_oracle": check.summary(probs, b64.fetch_all()[0])
                if check is not None else None}

    # ---- plain single-instance GPU ADMM on a few of the same instances,
    # cold start, problem resident: the engine pdos() picks for one instance
    # of this size (one 8-CTA cluster running the whole ADMM loop in one
    # launch), and the grid engine beside it
    plain_n = min(args.plain, B)
    plain_s, plain_iters, grid_s = 0.0, [], 0.0
    for p in probs[:plain_n]:
        with Batch([p], precision=prec, device=local, clusters=True) as b1:
            b1.set_blocks([256] * 5)
            b1.solve()  # warm-up
            b1.reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b1.solve()
            torch.cuda.synchronize()
            plain_s += time.perf_counter() - t0
            plain_iters.append(b1.infos()[0]["admm_iters"])
        with Workspace(p, prec, device=local) as w1:
            w1.solve()  # warm-up
            w1.reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w1.solve().fetch()
            torch.cuda.synchronize()
            grid_s += time.perf_counter() - t0
    plain = plain_n / plain_s if plain_s > 0 else None
    plain_grid = plain_n / grid_s if grid_s > 0 else None

    # ---- pdos() latency through the C ABI (set-up, solve, fetch) beside the
    # oracle on one core, on the small portfolio (n = 100) and one instance of
    # the family
    latency = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        from pdos_gb300.generators import portfolio
        from pdos_gb300.solver import pdos_call
        latency = {}
        small = portfolio(100, 10, 0.5, seed=0, params=dict(wl["params"], EPS_ABS=5e-3))
        for name, pr in (("portfolio_n100_eps5e-3", small), ("family_instance", probs[0])):
            pdos_call(pr, prec, device=local)  # warm-up
            t0 = time.perf_counter()
            out = pdos_call(pr, prec, device=local)
            t_gpu = time.perf_counter() - t0
            t0 = time.perf_counter()
            O.port_solve(pr)
            t_cpu = time.perf_counter() - t0
            latency[name] = {"pdos_seconds": t_gpu, "oracle_1_core_seconds": t_cpu, "admm_iterations": out["iters"],
                             "setup_ms": out["info"]["setup_ms"], "solve_ms": out["info"]["solve_ms"],
                             "nnz": pr.nnz, "precision": prec}

    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        h2d = sum(p.nnz * 16 + (p.n + 1) * 8 + (p.m + p.n) * 8 + len(p.q) * 8 for p in probs)
        d2h = sum((p.n + 2 * p.m) * 8 for p in probs)
        if wsn is not None:
            h2d += B * wsn.n_in * 4
        e2e_steps = max(1, min(args.steps, 2))
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            with Batch(probs, precision=prec, device=local, share_layouts=not args.own_layouts) as eb:
                eb.set_blocks(blocks)
                if wsn is not None:  # fetches every result once
                    wsn.solve(eb, mus, ds, fallback_params=wl["params"], precision=prec, device=local)
                else:
                    eb.solve().fetch_all()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": ws_n * B / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s,
               "path": "pdosgpu_batch_setup from host arrays, features H2D, inference, "
                       "pdosgpu_batch_warm_start, pdosgpu_batch_solve, pdosgpu_batch_fetch"}

    # error of the step's results (the last warm-started solve) and of the
    # cold-start solve against the FP64 oracle
    oracle_err = None
    if check is not None:
        oracle_err = check.summary(probs, batch.fetch_all()[0])
        oracle_err.update({
            "cold_start": cold_check, "seconds": check.seconds, "workers": check.workers,
            "spread": f"{len(check.idx)} instances evenly spaced over the {B} of the step",
            "oracle": "oracle (C restatement of the reference's indirect solver, FP64) at "
                      "EPS_ABS 1e-8, CG_MAX_ITS 200, CG_TOL 1e-12"})
    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, secs = cpu_family_sample(probs, args.cpu_instances)
        cpu = {"value": rate, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"oracle (C restatement, 1 core): {args.cpu_instances} held-out instances "
                         f"solved from the cold start in {secs:.1f} s"}
    if rank == 0:
        warm_iters = [d["admm_iters"] for d in warm_inf]
        cold_iters = [d["admm_iters"] for d in cold_inf]
        cfg = {"workload": args.workload, "instances_per_step": ws_n * B,
               "nnz_per_step": int(ws_n * sum(p.nnz for p in probs)), "precision": prec,
               "params": wl["params"], "cta_sizes_by_class": blocks,
               "l2": "inputs larger than L2: the batch's A and A' (%.0f MB) stream from HBM every "
                     "iteration (129 MB L2)" % (sum(p.nnz for p in probs) * 2 * (sv + 2) / 1e6),
               "parallelism": f"instances sharded over {ws_n} GPU(s), no collective"}
        if fam is not None:
            cfg.update({"family": {"n": wl["n"], "k": wl["k"], "density": wl["density"]}})
        line = {
            "metric": batch_metric(wl), "value": value, "unit": "solves/s", "n_gpus": ws_n,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 reductions)" if sv == 4 else "f64", "data": "synthetic (seeded)",
            "config": cfg,
            "plain_gpu_admm": {"value": plain, "unit": "solves/s", "instances": plain_n,
                               "engine": "one instance on an 8-CTA cluster (what pdos() picks at this size)",
                               "grid_engine_value": plain_grid,
                               "admm_iterations_mean": float(np.mean(plain_iters)) if plain_iters else None},
            "pdos_latency": latency,
            "batched_cold": {"value": ws_n * B / (cold_ms / 1e3), "unit": "solves/s",
                             "admm_iterations_mean": float(np.mean(cold_iters)),
                             "admm_iterations_max": int(max(cold_iters))},
            "batched_cold_fp64": batched_fp64,
            "speedup_vs_plain_gpu_admm": (value / plain) if plain else None,
            "admm_iterations_mean": float(np.mean(warm_iters)),
            "admm_iterations_max": int(max(warm_iters)),
            "solved": int(sum(d["solved"] for d in warm_inf)), "cold_start_fallbacks": fallbacks[0],
            "objective_error_vs_fp64_oracle": oracle_err,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "single_instance_spmv": spmv,
            "gpu_launches": int(launches), "clocks": clk.summary(),
        }
        line.update(info)
        print(json.dumps(line))
    if wsn is not None:
        wsn.net.close()
    batch.close()
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    ap.add_argument("--batch", type=int, default=0, help="instances per GPU per step (batch workloads)")
    ap.add_argument("--train", type=int, default=None, help="training instances (family workload)")
    ap.add_argument("--plain", type=int, default=8, help="instances solved one at a time for the comparison")
    ap.add_argument("--cpu-instances", type=int, default=4)
    ap.add_argument("--network-kernel", type=int, default=2, choices=[0, 1, 2],
                    help="profiling case: the network's product kernel "
                         "(0 mma.sync, 1 tcgen05 fed by cp.async, 2 tcgen05 fed by TMA)")
    ap.add_argument("--oracle-instances", type=int, default=64,
                    help="held-out instances checked against the FP64 oracle at EPS_ABS 1e-8 "
                         "(batch workloads)")
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--cpu-per-decile", type=int, default=64,
                    help="full-size uneven batch: instances per n-decile in the CPU baseline's subsample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--own-layouts", action="store_true",
                    help="batch workloads: every instance keeps its own matrix layout (no family sharing)")
    ap.add_argument("--no-spmv", action="store_true",
                    help="skip the single-instance SpMV block of the batch workloads")
    ap.add_argument("--blocks", default="",
                    help="profiling case: CTA size of each of the five size classes, comma-separated")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the FP64 batch of the family workload")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="profiling case: set up the workload, run this many ADMM "
                         "iterations, print nothing else (for ncu)")
    args = ap.parse_args()
    if args.workload in BATCH_WORKLOADS:
        wl = BATCH_WORKLOADS[args.workload]
        if args.impl == "reference":
            return run_batch_reference(args, wl)
        if args.profile_iters:  # a small batch of the workload's instances (all on the host at once)
            return profile_batch(args, wl)
        if wl["kind"] == "mix_waves":
            return run_batch_waves(args, wl)
        return run_batch(args, wl)
    wl = WORKLOADS[args.workload]
    prob = make_problem(wl)
    if args.impl == "reference":
        return run_reference(args, wl, prob)
    if args.profile_iters:
        from pdos_gb300.solver import Workspace
        with Workspace(prob, wl["precision"]) as ws:
            ws.iterate(args.profile_iters)
            print("iterations", ws.fetch()["iters"])
        return 0

    import torch
    ws_n, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws_n > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    from pdos_gb300 import build
    build.build()
    from pdos_gb300.solver import Workspace, pdos_call

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    sv = 8 if wl["precision"] == "fp64" else 4
    wsp = Workspace(prob, wl["precision"], device=local)
    stream = torch.cuda.ExternalStream(wsp.stream)
    for _ in range(args.warmup):
        wsp.reset().solve()
    first = wsp.fetch()
    launches0 = first["info"]["kernel_launches"]
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters_seen = []
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            wsp.reset().solve()
            r = wsp.fetch()
            iters_seen.append(r["iters"])
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    dev_ms = ev0.elapsed_time(ev1)
    res = wsp.fetch()
    launches = res["info"]["kernel_launches"] - launches0
    if pg:
        t = torch.tensor([dev_ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        dev_ms = float(t.item())
    ms_per_step = dev_ms / args.steps
    value = ws_n * args.steps / (dev_ms / 1e3)
    iters = int(np.median(iters_seen))
    cg_per_iter = res["cg_iters"] / max(res["iters"], 1)

    # roofline of the dominant kernel: the SpMV of the CG A pass (launched
    # k times per iteration, the largest share); the CG A' SpMV beside it
    ms_a = wsp.time_kernel(4, 20)
    ms_t = wsp.time_kernel(5, 20)
    ms_pass_a = wsp.time_kernel(0, 20)
    ms_pass_t = wsp.time_kernel(1, 20)
    wsp.reset()
    peak, peak_kind = measured_peaks()
    alg = spmv_bytes(prob, 0, sv)
    achieved = alg / (ms_a / 1e3) / 1e9
    traffic = committed_traffic(args.workload, "sell_spmv_kernel<OpCgA>")
    roofline = {"bound": "hbm", "kernel": "sell_spmv_kernel<OpCgA> (u = A p)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "traffic": traffic, "bytes_per_launch": alg,
                "ms_per_launch": ms_a,
                "cg_A_pass_ms_with_combine": ms_pass_a,
                "other_cg_kernel": {"kernel": "sell_spmv_kernel<OpCgAt> (t = p + A'u)",
                                    "ms_per_launch": ms_t,
                                    "achieved_GBs": spmv_bytes(prob, 1, sv) / (ms_t / 1e3) / 1e9,
                                    "pass_ms_with_combine": ms_pass_t}}
    # end to end through pdos() with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = {}
        for name in ("Ax", "Ai", "Ap", "b", "c"):
            a = getattr(prob, name)
            t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int64,
                            pin_memory=True)
            t.numpy()[:] = a
            pin[name] = t
        p2 = prob.with_params()
        for name, t in pin.items():
            setattr(p2, name, t.numpy())
        pdos_call(p2, wl["precision"], device=local)  # warm-up
        barrier()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 3))
        for _ in range(e2e_steps):
            pdos_call(p2, wl["precision"], device=local)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        h2d = prob.nnz * 16 + (prob.n + 1) * 8 + prob.m * 8 + prob.n * 8
        d2h = (prob.n + 2 * prob.m) * 8
        e2e = {"value": ws_n / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s,
               "path": "pdos_ex() C ABI, pinned host buffers"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        ts, ti = cpu_sample(prob, args.cpu_iters)
        cpu = {"value": cpu_solves_per_s(ts, ti, iters), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"oracle (C restatement, 1 core): set-up {ts:.2f} s + {args.cpu_iters} ADMM "
                         f"iterations at {ti:.3f} s each, extrapolated to {iters} iterations per solve",
               "admm_iterations_per_s": 1.0 / ti}
    opt_err = None
    if prob.optimum is not None:  # the FP64 optimum the generator built the problem around
        oo = float(prob.c @ prob.optimum["x"])
        opt_err = {"relative_objective_error": abs(float(prob.c @ res["x"]) - oo) / max(1.0, abs(oo)),
                   "optimal_objective": oo,
                   "relative_x_error": float(np.linalg.norm(res["x"] - prob.optimum["x"]) /
                                             max(1.0, np.linalg.norm(prob.optimum["x"])))}
    if rank == 0:
        line = {
            "metric": single_metric(wl), "value": value, "unit": "solves/s", "n_gpus": ws_n,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if sv == 8 else "f32 (f64 reductions)", "data": "synthetic (seeded)",
            "config": config_of(args, wl, prob),
            "admm_iterations_per_solve": iters, "cg_iterations_per_admm": cg_per_iter,
            "admm_iterations_per_s": ws_n * iters * args.steps / (dev_ms / 1e3),
            "status": res["status"], "error_vs_fp64_optimum": opt_err,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk.summary(),
        }
        print(json.dumps(line))
    wsp.close()
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
