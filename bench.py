#!/usr/bin/env python
"""Benchmark of the GB300 PDOS indirect solver.

Default workload (single GPU): the factor-model portfolio SOCP with
n = 200,000 assets, k = 2,000 factors, F at 5 % density (N = 202,001
variables, m = 404,002 rows, nnz = 20,604,001), FP64, EPS_ABS = 1e-4,
seeded synthetic data.  One step = one complete solve (reset to the cold
start, ADMM until the DIMACS test passes).

JSON line (rank 0):
  value    solves/s with the problem resident in HBM (device time, CUDA events
           on the solver's stream), whole job over all ranks
  e2e      solves/s through the drop-in pdos() with pinned host buffers: H2D
           of A, b, c, device set-up (transpose, equilibration), solve, D2H of
           x, s, y -- all inside the timed region
  roofline the SELL SpMV kernel of the CG A pass (u = A p, the kernel with the
           largest share of the solve), algorithmic bytes per launch / mean
           launch time (CUDA events on the solver's stream), against the
           measured HBM copy peak; traffic from the committed ncu capture
  cpu_baseline  the oracle (C restatement of the reference, 1 core) on a
           bounded sample: set-up plus a few ADMM iterations, extrapolated
           to a full solve with the GPU's iteration count
--impl reference runs that CPU solver instead, on this workload.
Multi-GPU (torchrun): replicas only -- every rank solves its own copy; no
collective is involved in the solve.
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
    # the small CPU-runnable case
    "portfolio_n100_fp64": dict(gen="portfolio", n=100, k=10, density=0.5, seed=0, precision="fp64",
                                params=dict(EPS_ABS=5e-3, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                            MAX_ITERS=2000, NORMALIZE=0)),
    # mixed precision random feasible SOCP
    "random_socp_m600k_fp32": dict(gen="random", m=600_000, n=200_000, nnz_per_col=20, seed=2,
                                   precision="fp32",
                                   params=dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4,
                                               MAX_ITERS=2000, NORMALIZE=1)),
}
DEFAULT_WORKLOAD = "portfolio_n200k_fp64"


def make_problem(wl):
    from pdos_gb300.generators import portfolio, random_feasible
    if wl["gen"] == "portfolio":
        return portfolio(wl["n"], wl["k"], wl["density"], seed=wl["seed"], params=wl["params"])
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
        "impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s",
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


METRIC = "solves/s at EPS_ABS 1e-4 (plain GPU ADMM, single instance); SpMV HBM GB/s"


def config_of(args, wl, prob):
    return {"workload": args.workload, "n_vars": prob.n, "m_rows": prob.m, "nnz": prob.nnz,
            "cones": {"f": prob.f, "l": prob.l, "q_count": int(len(prob.q)),
                      "q_max": int(max(prob.q)) if len(prob.q) else 0},
            "precision": wl["precision"], "params": wl["params"],
            "l2": ("inputs larger than L2: A and A' are %.0f MB resident in HBM, re-read by "
                   "every SpMV (129 MB L2)" % (2 * prob.nnz * (12 if wl["precision"] == "fp64" else 8) / 1e6))
            if 2 * prob.nnz * 8 > 129e6 else "small problem (L2-resident)",
            "parallelism": f"replicas x{args.gpus}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="profiling case: set up the workload, run this many ADMM "
                         "iterations, print nothing else (for ncu)")
    args = ap.parse_args()
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
        pdos_call(p2, wl["precision"])  # warm-up
        barrier()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 3))
        for _ in range(e2e_steps):
            pdos_call(p2, wl["precision"])
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
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws_n,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if sv == 8 else "f32 (f64 reductions)", "data": "synthetic (seeded)",
            "config": config_of(args, wl, prob),
            "admm_iterations_per_solve": iters, "cg_iterations_per_admm": cg_per_iter,
            "admm_iterations_per_s": ws_n * iters * args.steps / (dev_ms / 1e3),
            "status": res["status"],
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
