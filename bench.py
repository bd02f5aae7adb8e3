"""Benchmark: per-RHS time to rtol 1e-8 on R-MAT scale 20 (graph-Laplacian
multigrid solve, K-cycle with low-degree elimination).

Our arm (default): FP32 hierarchy / FP64 outer FCG, k = 32 right-hand sides
solved as one n x k row-major block through the C ABI
(ligmg_solve_batched_device, inputs resident in HBM).  A step = one batched
solve of k RHS to rtol 1e-8.  `e2e` repeats the measurement through the host
entry point ligmg_solve_batched (pinned host buffers; H2D of B and D2H of X
inside the timed region).  The plain FP64 single-RHS GPU solve is measured
next to it (the per-RHS comparison of the FP32 batched solve against plain
FP64) and the CPU oracle (the restated reference algorithm, all host cores)
gives cpu_baseline.

--impl reference: the reference (CombBLAS/PETSc/MPI) cannot be built on this
image, so this arm times the CPU restatement of its algorithm (oracle/),
FP64, one RHS per step, with all host threads.

Multi-GPU: replicas (each rank builds its own hierarchy and solves its own
RHS blocks; no collective on the data path); `value` aggregates all ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import faulthandler

import numpy as np

faulthandler.enable()

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "per-RHS time to rtol 1e-8: FP32/batched vs plain FP64 GPU; SpMV GB/s vs HBM"
SCALE = 20
EDGE_FACTOR = 16
GRAPH_SEED = 0


def log(*a):
    print("[bench]", *a, file=sys.stderr, flush=True)


def nvtx_push(name):
    try:
        import torch
        torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def nvtx_pop():
    try:
        import torch
        torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--k", type=int, default=32)
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", default="rmat20",
                    choices=["rmat20", "grid2d", "grid3d-ksweep", "rgg-batch", "adjoint"],
                    help="rmat20: the headline line (default); grid2d: 256^2 5-point grid, FP64 "
                         "V-cycle with Chebyshev(2,2) in FCG; grid3d-ksweep: 128^3 7-point grid, "
                         "lognormal weights, k in 1,8,32,64; rgg-batch: 256 uneven random "
                         "geometric graphs solved in one launch; adjoint: R-MAT 18 gradients "
                         "against central differences and oracle-built gradients")
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--tail-rows", type=int, default=None,
                    help="levels with at most this many rows (from the first such level "
                         "down) run as one persistent kernel; 0 disables (library default)")
    ap.add_argument("--graphs", type=int, default=256)
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# DRAM bytes per matrix entry of the k = 32 FP32 SpMM with the fused
# Chebyshev epilogue, from an ncu capture of a smaller case of the same kernel
# (the row-stream k_spmm_rs, R-MAT 19 level 1, the ChebZ launch: 157.8 MB read
# and 22.7 MB written over 15,448,585 entries); roofline.traffic scales it by
# the dominant launch's entries.  Levels whose vectors stay in L2 move less,
# so this is an upper estimate there.
SPMM_K32_DRAM_BYTES_PER_NNZ = 180.56e6 / 15448585
SPMM_K32_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_spmm_rs<float, 32, "
                           "ChebZ> on R-MAT 19 level 1 (15,448,585 entries, 157.8 + 22.7 MB, 11.7 "
                           "bytes per entry), scaled by the launch's entries")


def level_nnz_of(S, level):
    try:
        return S.level_info(level)["nnz"]
    except Exception:
        return None


# DRAM bytes per matrix entry of the FP64 single right-hand-side SpMV
# (k_spmv_tile, y = A x), from an ncu capture of a smaller case of the same
# kernel (see SPMV_TRAFFIC_SOURCE); scaled to a launch by its entries.
SPMV_DRAM_BYTES_PER_NNZ = 213.96e6 / 15448585
SPMV_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_spmv_tile<double, "
                       "Store> on R-MAT 19 level 1 (15,448,585 entries): 193.2 MB read + 20.7 MB "
                       "written per launch, 13.9 bytes per entry, scaled by this launch's entries")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def workload_graph(scale):
    from ligmg_gb300 import graphs as G
    return G.rmat(scale, edge_factor=EDGE_FACTOR, seed=GRAPH_SEED)


TAIL_ROWS = None


def solver_kw(prec):
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg")
    if TAIL_ROWS is not None:
        kw["tail_rows"] = TAIL_ROWS
    return kw


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline_oracle(L, b, threads):
    """The oracle (CPU restatement of the reference algorithm), FP64 K-cycle,
    one RHS; returns (ms per RHS, setup seconds, iterations, oracle solver,
    its solution)."""
    from oracle import oracle as O
    O.set_threads(threads)
    t = time.perf_counter()
    S = O.OracleSolver(L, kcycle=1, outer_ksp_type="fcg")
    setup = time.perf_counter() - t
    t = time.perf_counter()
    x, info = S.solve(b)
    return (time.perf_counter() - t) * 1e3, setup, info["iters"], S, x


def _proj(x):
    return x - x.mean()


def hierarchy_parity(S, S64, R, b, x_oracle):
    """The GPU hierarchy of the headline workload against the oracle's, on the
    same graph: every level's type, sizes, CSR arrays and value bits and its
    ids must be identical; one FP64 cycle from the first cycled level
    (after the top elimination) must match to 1e-12 relative after
    projecting out the constant; the FP64 GPU solve of b must match the
    oracle's solution to 1e-6 relative."""
    nl = R.num_levels
    out = {"levels_gpu": S.num_levels, "levels_oracle": nl, "levels_equal": 0,
           "first_mismatch": None}
    for l in range(min(nl, S.num_levels)):
        gi, ri = S.level_info(l), R.level_info(l)
        eq = gi == ri
        if eq:
            grp, gci, gv = S.level_matrix(l)
            rrp, rci, rv = R.level_matrix(l)
            eq = (np.array_equal(grp, rrp) and np.array_equal(gci, rci)
                  and np.array_equal(gv.view(np.int64), rv.view(np.int64)))
            del grp, gci, gv, rrp, rci, rv
        if eq and ri["type"] != "coarse":
            eq = np.array_equal(S.level_ids(l), R.level_ids(l))
        if eq:
            out["levels_equal"] += 1
        elif out["first_mismatch"] is None:
            out["first_mismatch"] = l
    base = 1 if R.level_info(0)["type"] == "elim" else 0
    bb = _proj(np.random.default_rng(42).standard_normal(R.level_info(base)["n"]))
    xg, xr = S64.cycle(base, bb), R.cycle(base, bb)
    out["cycle_level"] = base
    out["cycle_fp64_relerr"] = float(np.linalg.norm(_proj(xg) - _proj(xr)) /
                                     np.linalg.norm(_proj(xr)))
    xs = S64.solve(b).solution
    out["solution_fp64_relerr_vs_oracle"] = float(np.linalg.norm(_proj(xs) - _proj(x_oracle)) /
                                                  np.linalg.norm(_proj(x_oracle)))
    out["bars"] = "levels bit-equal; cycle <= 1e-12; solution <= 1e-6"
    out["ok"] = bool(out["levels_equal"] == nl == S.num_levels and out["cycle_fp64_relerr"] <= 1e-12
                     and out["solution_fp64_relerr_vs_oracle"] <= 1e-6)
    return out


def spmv_roofline(S64, stream, peak, peak_kind, reps=20):
    """The plain FP64 single right-hand-side SpMV y = A x (the reference's
    SpMV_inplace, util.hpp:451-476) on the level with the most entries below
    the top elimination, through the device-pointer entry point: CUDA events
    on the handle's stream around `reps` launches; x (8n bytes) lies in L2,
    the matrix (12 bytes per entry plus row pointers) does not."""
    import ctypes as C
    import torch
    from ligmg_gb300._lib import check, lib
    lv = max(range(1, S64.num_levels - 1), key=lambda l: S64.level_info(l)["nnz"])
    inf = S64.level_info(lv)
    n, nnz = inf["n"], inf["nnz"]
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.randn(n, dtype=torch.float64, device=dev)
    y = torch.empty(n, dtype=torch.float64, device=dev)

    def run():
        check(lib().ligmg_spmv_device_noalloc(S64._h, lv, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(y.data_ptr())), "spmv")
    for _ in range(3):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nvtx_push("spmv_roofline")
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    byt = 8.0 * (n + 1) + 12.0 * nnz + 16.0 * n
    traffic = SPMV_DRAM_BYTES_PER_NNZ * nnz if SPMV_DRAM_BYTES_PER_NNZ else None
    return {"bound": "hbm", "achieved": byt / sec / 1e9, "peak": peak, "unit": "GB/s",
            "frac": byt / sec / 1e9 / peak, "peak_source": peak_kind,
            "traffic": traffic, "traffic_source": SPMV_TRAFFIC_SOURCE if traffic else None,
            "kernel": f"FP64 k=1 SpMV y = A x (layout picked by the setup autotuner), "
                      f"level {lv} n={n} nnz={nnz}",
            "bytes_per_launch": byt, "us_per_launch": sec * 1e6, "launches_timed": reps,
            "gather": gather_roof(n, 8, nnz, sec)}


def gather_roof(n, width, nnz, sec):
    """The same launch against the gather ceiling measured on this GPU: one
    random `width`-byte row of x per entry, from a table of the level's n rows
    (ligmg_measure_gather_peak), entries per second over that ceiling."""
    from ligmg_gb300 import Solver
    try:
        peak = Solver.gather_peak(n, width, nnz)
    except Exception as e:  # measurement only
        return {"error": str(e)}
    ach = nnz / sec
    return {"bound": "l2-gather", "achieved": ach, "peak": peak, "unit": "rows/s",
            "frac": ach / peak, "row_bytes": width, "table_rows": n,
            "peak_source": "measured in this run (ligmg_measure_gather_peak)"}


def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return
    from ligmg_gb300 import graphs as G
    threads = os.cpu_count() or 1
    L = workload_graph(args.scale)
    from oracle import oracle as O
    O.set_threads(threads)
    t = time.perf_counter()
    S = O.OracleSolver(L, kcycle=1, outer_ksp_type="fcg")
    setup = time.perf_counter() - t
    B = G.rhs(L.n, k=args.warmup + args.steps, seed=1000)
    for w in range(args.warmup):
        S.solve(B[:, w].copy())
    times, iters = [], []
    for s in range(args.steps):
        b = B[:, args.warmup + s].copy()
        t = time.perf_counter()
        _, info = S.solve(b)
        times.append(time.perf_counter() - t)
        iters.append(info["iters"])
    ms_per_rhs = 1e3 * sum(times) / len(times)
    out = {
        "impl": "reference", "metric": METRIC, "value": ms_per_rhs, "unit": "ms/RHS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_rhs, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": {"workload": f"rmat{args.scale} (a,b,c,d=.57,.19,.19,.05; ef {EDGE_FACTOR}; LCC; "
                               f"w~U(0.5,2)) n={L.n} nnz={L.nnz}; K-cycle + elimination; FCG "
                               f"rtol 1e-8; 1 RHS per step",
                   "note": "reference (CombBLAS+PETSc+MPI) unbuildable here; CPU restatement "
                           "of its algorithm (oracle/) timed instead",
                   "setup_s": setup, "iters": iters, "threads": threads},
        "cpu_baseline": {"value": ms_per_rhs, "unit": "ms/RHS", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} single-RHS FP64 solves to rtol 1e-8 on the "
                                   f"full rmat{args.scale} graph; setup ({setup:.1f}s) untimed"},
        "e2e": {"value": ms_per_rhs, "unit": "ms/RHS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from ligmg_gb300 import Solver
    from ligmg_gb300 import build as B
    from ligmg_gb300 import graphs as G
    B.build()
    k = args.k
    L = workload_graph(args.scale)
    n = L.n
    log(f"graph n={n} nnz={L.nnz}")
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- FP32-hierarchy batched solver -----------------------------------------
    t0 = time.perf_counter()
    S = Solver(L, **solver_kw("fp32"), device=local)
    setup_s = time.perf_counter() - t0
    log(f"fp32 setup {setup_s:.2f}s levels={S.num_levels}")
    S.set_stream(stream.cuda_stream)
    nblk = 4
    rng_seed = 100 + 1000 * rank
    Bd = [torch.from_numpy(G.rhs(n, k=k, seed=rng_seed + i)).to(dev) for i in range(nblk)]
    Xd = torch.empty((n, k), dtype=torch.float64, device=dev)
    infos = []
    first_s = None
    for w in range(args.warmup):
        t0 = time.perf_counter()
        infos.append(S.solve_batched_device(Bd[w % nblk].data_ptr(), k, Xd.data_ptr()))
        torch.cuda.synchronize()
        if first_s is None:
            first_s = time.perf_counter() - t0  # includes launch-shape autotuning
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = Solver.launch_count()
    nvtx_push("timed_region")
    ev0.record(stream)
    timed_infos = []
    for s in range(args.steps):
        timed_infos.append(S.solve_batched_device(Bd[s % nblk].data_ptr(), k, Xd.data_ptr()))
    ev1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop()
    launches = Solver.launch_count() - l0
    barrier()
    clocks = sampler.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    log(f"timed {elapsed_ms:.2f} ms for {args.steps} steps")
    # ---- profiled repeat of the timed steps (per-kernel CUDA events) -------------
    # Every library kernel is bracketed by events on the solver's stream; the
    # events cost time of their own, so `value` comes from the unprofiled region
    # above and the roofline from this identical repeat.
    S.profile(True)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for s in range(args.steps):
        S.solve_batched_device(Bd[s % nblk].data_ptr(), k, Xd.data_ptr())
    p1.record(stream)
    torch.cuda.synchronize()
    profiled_ms = p0.elapsed_time(p1)
    stats = S.kernel_stats()
    S.profile(False)
    log(f"profiled repeat {profiled_ms:.2f} ms")
    iters = [i.iters() for i in timed_infos]
    true_res = max(float(np.max(i.col_true_rel_residual)) for i in timed_infos)
    converged = all(i.converged for i in timed_infos)
    # ---- e2e through the host entry point (pinned host buffers) ------------------
    Bh = torch.empty((n, k), dtype=torch.float64, pin_memory=True)
    Bh.copy_(Bd[0].cpu())
    Bh_np = Bh.numpy()
    Xh = torch.empty((n, k), dtype=torch.float64, pin_memory=True)
    import ctypes as C
    from ligmg_gb300._lib import check, lib
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    info_e, keep_hist, keep_ci, keep_ct = S._info(k)  # arrays must outlive the calls
    e0.record(stream)
    for s in range(args.steps):
        check(lib().ligmg_solve_batched(S._h, C.c_void_p(Bh.data_ptr()), k,
                                        C.c_void_p(Xh.data_ptr()), C.byref(info_e)))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    log(f"e2e {e2e_ms:.2f} ms")
    # ---- FP32-hierarchy single-RHS solve on the same handle (one zero-mean RHS,
    # the unbatched form of the same solve) -------------------------------------------
    fp32s = {}
    if not args.no_fp64:
        b1 = torch.from_numpy(G.rhs(n, k=1, seed=rng_seed)).to(dev).reshape(n, 1).contiguous()
        x1 = torch.empty((n, 1), dtype=torch.float64, device=dev)
        for _ in range(max(args.warmup, 1)):  # the first k = 1 solve also tunes its plans
            S.solve_batched_device(b1.data_ptr(), 1, x1.data_ptr())
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        nrep = 3
        it32 = []
        for _ in range(nrep):
            inf = S.solve_batched_device(b1.data_ptr(), 1, x1.data_ptr())
            it32.append(inf.iters())
        f1.record(stream)
        torch.cuda.synchronize()
        fp32s = {"ms_per_rhs": f0.elapsed_time(f1) / nrep, "iters": it32,
                 "true_rel_residual": inf.true_rel_residual}
        log(f"fp32 single {fp32s['ms_per_rhs']:.2f} ms/RHS")
    # ---- plain FP64 single-RHS GPU solve (per-RHS comparison) ----------------------
    fp64 = {}
    S64 = None
    if not args.no_fp64:
        t0 = time.perf_counter()
        S64 = Solver(L, **solver_kw("fp64"), device=local)
        fp64["setup_s"] = time.perf_counter() - t0
        S64.set_stream(stream.cuda_stream)
        b1 = torch.from_numpy(G.rhs(n, k=1, seed=rng_seed)).to(dev).reshape(n, 1).contiguous()
        x1 = torch.empty((n, 1), dtype=torch.float64, device=dev)
        for _ in range(max(args.warmup, 1)):
            S64.solve_batched_device(b1.data_ptr(), 1, x1.data_ptr())
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        nrep = 3
        it64 = []
        for _ in range(nrep):
            inf = S64.solve_batched_device(b1.data_ptr(), 1, x1.data_ptr())
            it64.append(inf.iters())
        f1.record(stream)
        torch.cuda.synchronize()
        fp64["ms_per_rhs"] = f0.elapsed_time(f1) / nrep
        fp64["iters"] = it64
        fp64["true_rel_residual"] = inf.true_rel_residual
        # per-kernel figures from one more, profiled solve (events cost time)
        S64.profile(True)
        S64.solve_batched_device(b1.data_ptr(), 1, x1.data_ptr())
        st64 = S64.kernel_stats()
        S64.profile(False)
        fp64["profile_ms_by_level"] = by_key(st64, "level", 1)
        log(f"fp64 single {fp64['ms_per_rhs']:.2f} ms/RHS")
    # ---- aggregate over ranks ----------------------------------------------------
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([elapsed_ms, e2e_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms, e2e_ms = float(t[0]), float(t[1])
    total_rhs = args.steps * k * ws
    value = elapsed_ms / total_rhs
    if rank != 0:
        return
    peak, peak_kind = peaks()
    # the dominant bandwidth-bound kernel (krylov / vector / outer entries group
    # several kernels; the persistent coarse-tail kernel is issue-bound, one SM
    # per column slice, and is reported on its own in config.tail)
    single = [r for r in stats if r["kind"] not in ("krylov", "vector", "outer", "tail")]
    tails = [r for r in stats if r["kind"] == "tail"]
    top = max(single, key=lambda r: r["seconds"]) if single else None
    roof = None
    if top:
        per_launch_bytes = top["bytes"] / top["launches"]
        per_launch_s = top["seconds"] / top["launches"]
        ach = per_launch_bytes / per_launch_s / 1e9
        traffic, traffic_src = None, None
        if not top["fp64"] and top["kind"] in ("cheb_b", "spmv"):
            # DRAM bytes per entry of the k = 32 FP32 Chebyshev SpMM measured on a
            # smaller case (SPMM_K32_TRAFFIC_SOURCE), scaled by entries
            nnz_top = level_nnz_of(S, top["level"])
            traffic = SPMM_K32_DRAM_BYTES_PER_NNZ * nnz_top if nnz_top else None
            traffic_src = SPMM_K32_TRAFFIC_SOURCE
        gath = None
        if top["kind"] in ("cheb_a", "cheb_b", "spmv", "resid"):
            # one gathered X row (k values) per entry of the level's A
            lv_top = S.level_info(top["level"])
            gath = gather_roof(lv_top["n"], top["k"] * (8 if top["fp64"] else 4), lv_top["nnz"],
                               per_launch_s) if top["k"] * (8 if top["fp64"] else 4) in (4, 8, 128) \
                else None
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "gather": gath,
                "traffic": traffic, "traffic_source": traffic_src, "peak_source": peak_kind,
                "kernel": f"spmm_{top['kind']} level {top['level']} k={top['k']} "
                          f"{'fp64' if top['fp64'] else 'fp32'}",
                "bytes_per_launch": per_launch_bytes, "us_per_launch": per_launch_s * 1e6,
                "share_of_profiled": top["seconds"] / (profiled_ms / 1e3),
                "measured_over": f"profiled repeat of the {args.steps} timed steps "
                                 f"({profiled_ms / args.steps:.2f} ms/step with events)"}
    cpu = None
    cpu1 = None
    parity = None
    if not args.no_cpu_baseline and ws == 1:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        b0 = Bd[0][:, 0].cpu().numpy().copy()
        ms, osetup, oit, R, xo = cpu_baseline_oracle(L, b0, threads)
        cpu = {"value": ms, "unit": "ms/RHS", "cores": threads, "kind": "port",
               "sample": f"1 RHS (column 0 of the first block), FP64 K-cycle solve to rtol 1e-8 on "
                         f"the full graph, {oit} iterations; oracle setup {osetup:.1f}s untimed"}
        O.set_threads(1)
        t0 = time.perf_counter()
        R.solve(b0)
        cpu1 = {"value": (time.perf_counter() - t0) * 1e3, "unit": "ms/RHS", "cores": 1,
                "kind": "port", "sample": "the same single-RHS solve on one core"}
        O.set_threads(threads)
        log(f"oracle {ms:.1f} ms/RHS on {threads} threads, {cpu1['value']:.1f} on one")
        if S64 is not None:
            t0 = time.perf_counter()
            parity = hierarchy_parity(S, S64, R, b0, xo)
            parity["seconds"] = time.perf_counter() - t0
            log(f"parity {parity}")
        del R
    spmv_roof = spmv_roofline(S64, stream, *peaks()) if S64 is not None else None
    if S64 is not None:
        S64.close()
    levels = [S.level_info(l) for l in range(S.num_levels)]
    out = {
        "metric": METRIC, "value": value, "unit": "ms/RHS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 cycle / fp64 outer",
        "data": "synthetic",
        "config": {
            "workload": f"rmat{args.scale} (a,b,c,d=.57,.19,.19,.05; edge factor {EDGE_FACTOR}; "
                        f"symmetrised, LCC; w~U(0.5,2)) n={n} nnz={L.nnz}; K-cycle + elimination; "
                        f"FP32 hierarchy in FP64 FCG; rtol 1e-8; k={k} RHS per step",
            "k": k, "rhs_per_s": 1e3 / value, "setup_s": setup_s,
            "setup_phases_s": S.setup_times(),
            "first_solve_s": first_s, "autotune": True,
            "iters": iters, "converged": converged, "max_true_rel_residual": true_res,
            "levels": len(levels), "level_n": [l["n"] for l in levels],
            "level_nnz": [l["nnz"] for l in levels],
            "l2": "hierarchy (>= 300 MB FP32+FP64 matrices) larger than the 129 MB L2",
            "fp64_single_rhs": fp64,
            "parity": parity,
            "cpu_baseline_1thread": cpu1,
            "speedup_vs_fp64_single": (fp64.get("ms_per_rhs", 0) / value) if fp64 else None,
            "fp32_single_rhs": fp32s,
            "speedup_fp32_single_vs_fp64_single": (fp64["ms_per_rhs"] / fp32s["ms_per_rhs"])
            if (fp64 and fp32s) else None,
            "top_kernels": [{**r, "gbs": r["bytes"] / r["seconds"] / 1e9}
                            for r in sorted(stats, key=lambda r: -r["seconds"])[:8]],
            "profile_ms_per_step_by_level": by_key(stats, "level", args.steps),
            "profile_ms_per_step_by_kind": by_key(stats, "kind", args.steps),
            "profiled_ms_per_step": profiled_ms / args.steps,
            "tail": ({"level": tails[0]["level"], "launches_per_step": tails[0]["launches"] / args.steps,
                      "us_per_launch": 1e6 * tails[0]["seconds"] / tails[0]["launches"],
                      "share_of_profiled": tails[0]["seconds"] / (profiled_ms / 1e3),
                      "note": "coarse levels from `level` down as one persistent kernel in "
                              "shared memory (kept by the autotuner)"} if tails else None),
            "gathers_by_level": [
                {"level": r["level"], "kind": r["kind"],
                 "rows_per_s": S.level_info(r["level"])["nnz"] * r["launches"] / r["seconds"],
                 "l2_to_sm_tbs": S.level_info(r["level"])["nnz"] * r["launches"] / r["seconds"]
                 * r["k"] * (8 if r["fp64"] else 4) / 1e12}
                for r in sorted(stats, key=lambda r: (r["level"], r["kind"]))
                if r["kind"] in ("cheb_a", "cheb_b", "spmv") and 1 <= r["level"] <= 4],
            "profile_table": [[r["level"], r["kind"], round(r["launches"] / args.steps, 1),
                               round(r["seconds"] * 1e3 / args.steps, 3)]
                              for r in sorted(stats, key=lambda r: -r["seconds"])],
        },
        "roofline": roof,
        "roofline_spmv": spmv_roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_ms / total_rhs, "unit": "ms/RHS",
                "h2d_bytes_per_step": n * k * 8, "d2h_bytes_per_step": n * k * 8},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(out), flush=True)


def by_key(stats, key, steps):
    """Summed event time (ms per step) and launches per step of the profiled
    repeat, grouped by level or by kernel kind."""
    out = {}
    for r in stats:
        d = out.setdefault(str(r[key]), {"ms": 0.0, "launches": 0})
        d["ms"] += r["seconds"] * 1e3 / steps
        d["launches"] += r["launches"] / steps
    return {k: {"ms": round(v["ms"], 3), "launches": round(v["launches"], 1)}
            for k, v in sorted(out.items(), key=lambda kv: -kv[1]["ms"])}


def _timed_solves(S, stream, Bd, k, steps, warmup):
    import torch
    n = Bd[0].shape[0]
    Xd = torch.empty((n, k), dtype=torch.float64, device=Bd[0].device)
    for w in range(warmup):
        S.solve_batched_device(Bd[w % len(Bd)].data_ptr(), k, Xd.data_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    infos = [S.solve_batched_device(Bd[t % len(Bd)].data_ptr(), k, Xd.data_ptr())
             for t in range(steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), infos


def run_grid3d(args):
    """3-D grid Laplacian: k right-hand sides as an n x k block, k in {1, 8, 32, 64}."""
    import torch
    from ligmg_gb300 import Solver
    from ligmg_gb300 import build as Bld
    from ligmg_gb300 import graphs as G
    Bld.build()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    L = G.grid3d(args.grid, weights="lognormal", seed=1)
    log(f"grid3d n={L.n} nnz={L.nnz}")
    S = Solver(L, **solver_kw("fp32"))
    S.set_stream(stream.cuda_stream)
    per_k = {}
    for k in (1, 8, 32, 64):
        Bd = [torch.from_numpy(G.rhs(L.n, k=k, seed=7 + i)).to(dev).reshape(L.n, k).contiguous()
              for i in range(2)]
        ms, infos = _timed_solves(S, stream, Bd, k, args.steps, args.warmup)
        per_k[k] = {"ms_per_rhs": ms / (args.steps * k), "iters": [i.iters() for i in infos],
                    "max_true_rel_residual": max(float(np.max(i.col_true_rel_residual)) for i in infos)}
        log(f"k={k} {per_k[k]['ms_per_rhs']:.3f} ms/RHS")
        del Bd
    S64 = Solver(L, **solver_kw("fp64"))
    S64.set_stream(stream.cuda_stream)
    b1 = [torch.from_numpy(G.rhs(L.n, seed=3)).to(dev).reshape(L.n, 1).contiguous()]
    ms64, inf64 = _timed_solves(S64, stream, b1, 1, 3, 1)
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        ms_c, osetup, oit, _, _ = cpu_baseline_oracle(L, G.rhs(L.n, seed=3), threads)
        cpu = {"value": ms_c, "unit": "ms/RHS", "cores": threads, "kind": "port",
               "sample": f"1 RHS, FP64 K-cycle FCG to rtol 1e-8 by the oracle, {oit} "
                         f"iterations; oracle setup {osetup:.1f}s untimed"}
    out = {"metric": METRIC, "value": per_k[32]["ms_per_rhs"], "unit": "ms/RHS", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_k[32]["ms_per_rhs"] * 32,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32 cycle / fp64 outer", "data": "synthetic",
           "config": {"workload": f"grid3d {args.grid}^3 7-point, lognormal(0,1) weights, n={L.n} "
                                  f"nnz={L.nnz}; FP32 hierarchy, K-cycle, FCG rtol 1e-8",
                      "per_k": per_k, "fp64_single_ms_per_rhs": ms64 / 3},
           "cpu_baseline": cpu}
    print(json.dumps(out), flush=True)


def run_rgg_batch(args):
    """Batch of 256 random geometric graphs (n log-uniform in [1e4, 2e5],
    mean degree ~12, w = clip(1/d, 0.1, 10), largest component each), one
    zero-mean RHS per graph, FP32 cycle inside FP64 outer FCG to rtol 1e-8,
    through the host entry point ligmg_batch_solve (H2D of b and D2H of x
    inside the timed region).  Two arms on the same batch: the persistent
    work-queue launch (batch_queue = 1, one launch per 16 outer iterations,
    each graph advancing on its own) and the level kernels over the union
    replayed from a CUDA graph (batch_queue = 0).  Three graphs (smallest,
    median, largest) are checked against the oracle's single-graph solves."""
    from ligmg_gb300 import BatchSolver
    from ligmg_gb300 import build as Bld
    from ligmg_gb300 import graphs as G
    from oracle import oracle as O
    Bld.build()
    t0 = time.perf_counter()
    gs = G.rgg_batch(args.graphs, seed=0)
    gen_s = time.perf_counter() - t0
    log(f"{len(gs)} graphs, {sum(g.n for g in gs)} vertices, {sum(g.nnz for g in gs)} nnz "
        f"generated in {gen_s:.1f}s")
    bs = [G.rhs(g.n, seed=100 + i) for i, g in enumerate(gs)]
    arms = {}
    xs_q = None
    for name, q in (("queue", 1), ("union_graph", 0)):
        t0 = time.perf_counter()
        B = BatchSolver(gs, precision="fp32", kcycle=1, batch_queue=q)
        setup = time.perf_counter() - t0
        for _ in range(args.warmup):
            B.solve(bs)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            xs, info = B.solve(bs)
        secs = (time.perf_counter() - t0) / args.steps
        arms[name] = {"ms_per_step": 1e3 * secs, "ms_per_rhs": 1e3 * secs / len(gs),
                      "setup_s": setup, "max_iters": int(np.max(info.col_iters)),
                      "mean_iters": float(np.mean(info.col_iters)),
                      "converged": bool(info.converged),
                      "max_true_rel_residual": float(np.max(info.col_true_rel_residual)),
                      "levels": B.num_levels}
        log(f"{name}: {arms[name]['ms_per_step']:.1f} ms per batch")
        if q == 1:
            xs_q = xs
        B.close()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    cpu = None
    if not args.no_cpu_baseline:
        pick = np.random.default_rng(1).choice(len(gs), 8, replace=False)
        t_cpu = 0.0
        for g in pick:
            R = O.OracleSolver(gs[g], kcycle=1, outer_ksp_type="fcg")
            t0 = time.perf_counter()
            R.solve(bs[g])
            t_cpu += time.perf_counter() - t0
        cpu = {"value": 1e3 * t_cpu / len(pick), "unit": "ms/RHS", "cores": threads,
               "kind": "port", "sample": "8 random graphs of the batch, each one FP64 K-cycle FCG "
                                         "solve to rtol 1e-8 by the oracle (setup untimed), "
                                         "ms per graph"}
    order = np.argsort([g.n for g in gs])
    sample = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
    parity = {}
    for g in sample:
        xr, _ = O.OracleSolver(gs[g], kcycle=1, outer_ksp_type="fcg").solve(bs[g])
        a, b = xs_q[g] - xs_q[g].mean(), xr - xr.mean()
        parity[str(g)] = {"n": gs[g].n, "relerr_vs_oracle": float(np.linalg.norm(a - b) /
                                                                 np.linalg.norm(b))}
    value = arms["queue"]["ms_per_rhs"]
    out = {"metric": METRIC, "value": value, "unit": "ms/RHS", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": arms["queue"]["ms_per_step"],
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32 cycle / fp64 outer", "data": "synthetic",
           "config": {"workload": f"{len(gs)} random geometric graphs, n log-uniform in "
                                  f"[1e4, 2e5], mean degree ~12, w = clip(1/d, .1, 10), LCC; "
                                  f"one RHS each; host-timed ligmg_batch_solve incl. H2D/D2H",
                      "vertices": int(sum(g.n for g in gs)), "nnz": int(sum(g.nnz for g in gs)),
                      "generation_s": gen_s, "arms": arms, "parity_vs_oracle": parity},
           "cpu_baseline": cpu,
           "e2e": {"value": value, "unit": "ms/RHS",
                   "h2d_bytes_per_step": 8 * int(sum(g.n for g in gs)),
                   "d2h_bytes_per_step": 8 * int(sum(g.n for g in gs))}}
    print(json.dumps(out), flush=True)


def run_grid2d(args):
    """2-D 5-point grid Laplacian 256 x 256, unit weights, one zero-mean RHS:
    FP64 V-cycle with Chebyshev(2,2) smoothing preconditioning FCG to rtol
    1e-8 (plain method), timed per RHS with device-resident b; the oracle
    timed on one and on all host cores; the GPU hierarchy, one FP64 cycle and
    the solution checked against the oracle's."""
    import torch
    from ligmg_gb300 import Solver
    from ligmg_gb300 import build as Bld
    from ligmg_gb300 import graphs as G
    from oracle import oracle as O
    Bld.build()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    L = G.grid2d(args.grid)
    kw = dict(kcycle=0, outer_ksp_type="fcg", pre_smooth=2, post_smooth=2)
    t0 = time.perf_counter()
    S = Solver(L, **kw)
    setup = time.perf_counter() - t0
    S.set_stream(stream.cuda_stream)
    b = G.rhs(L.n, seed=7)
    Bd = [torch.from_numpy(b).to(dev).reshape(L.n, 1).contiguous()]
    clk = ClockSampler(0)
    clk.start()
    ms, infos = _timed_solves(S, stream, Bd, 1, args.steps, args.warmup)
    clocks = clk.stop()
    # the same solve with the FP32 hierarchy (single and 32 RHS)
    S32 = Solver(L, precision="fp32", **kw)
    S32.set_stream(stream.cuda_stream)
    ms32, inf32 = _timed_solves(S32, stream, Bd, 1, args.steps, args.warmup)
    B32 = [torch.from_numpy(G.rhs(L.n, k=32, seed=8)).to(dev)]
    ms32k, inf32k = _timed_solves(S32, stream, B32, 32, args.steps, args.warmup)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    t0 = time.perf_counter()
    R = O.OracleSolver(L, **kw)
    osetup = time.perf_counter() - t0
    t0 = time.perf_counter()
    xo, io = R.solve(b)
    cpu_all = (time.perf_counter() - t0) * 1e3
    O.set_threads(1)
    t0 = time.perf_counter()
    R.solve(b)
    cpu_one = (time.perf_counter() - t0) * 1e3
    O.set_threads(threads)
    parity = hierarchy_parity(S, S, R, b, xo)
    value = ms / args.steps
    peak, peak_kind = peaks()
    out = {"metric": METRIC, "value": value, "unit": "ms/RHS", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {"workload": f"grid2d {args.grid}x{args.grid} 5-point, unit weights, "
                                  f"n={L.n} nnz={L.nnz}; FP64 V-cycle, Chebyshev(2,2), FCG "
                                  f"rtol 1e-8; 1 RHS per step",
                      "setup_s": setup, "iters": [i.iters() for i in infos],
                      "max_true_rel_residual": max(i.true_rel_residual for i in infos),
                      "levels": S.num_levels, "parity": parity,
                      "fp32_hierarchy_single_ms_per_rhs": ms32 / args.steps,
                      "fp32_hierarchy_k32_ms_per_rhs": ms32k / (32 * args.steps),
                      "fp32_iters": [i.iters() for i in inf32],
                      "oracle_setup_s": osetup, "oracle_iters": io["iters"],
                      "cpu_1thread_ms_per_rhs": cpu_one,
                      "l2": "the hierarchy (< 20 MB) fits in L2: a latency-bound workload"},
           "roofline": spmv_roofline(S, stream, peak, peak_kind),
           "cpu_baseline": {"value": cpu_all, "unit": "ms/RHS", "cores": threads, "kind": "port",
                            "sample": "the same FP64 solve (1 RHS) by the oracle, all host cores; "
                                      f"one core: {cpu_one:.1f} ms"},
           "clocks": clocks}
    print(json.dumps(out), flush=True)


def run_adjoint(args):
    """Differentiation through the solve on R-MAT 18: loss = 0.5 ||x - x_t||^2
    with x = L(w)^+ b.  Gradients with respect to every edge weight and to b
    from ligmg_forward / ligmg_backward (FP64, rtol 1e-12), checked on 64
    random edges and 64 random entries of b against central differences
    (relative step 1e-6, every perturbed system solved from a fresh setup to
    rtol 1e-12) and on all edges against the gradient built from two oracle
    solves (x and the adjoint lambda).  value: ms per forward + backward."""
    import torch
    from ligmg_gb300 import Solver
    from ligmg_gb300 import build as Bld
    from ligmg_gb300 import graphs as G
    from oracle import oracle as O
    Bld.build()
    scale = 18 if args.scale == SCALE else args.scale
    L0 = G.rmat(scale, edge_factor=EDGE_FACTOR, seed=GRAPH_SEED)
    A = L0.to_scipy().tocoo()
    m = A.row < A.col
    u, v, w = A.row[m], A.col[m], -A.data[m]
    n = L0.n
    rng = np.random.default_rng(5)
    b = G.rhs(n, seed=9)
    xt = rng.standard_normal(n)
    xt -= xt.mean()
    kw = dict(kcycle=1, outer_ksp_type="fcg", tol=1e-12)
    L = G.laplacian_from_edges(n, u, v, w)
    S = Solver(L, **kw)
    pos = np.empty(len(u), dtype=np.int64)  # CSR position of (u, v)
    for e in range(len(u)):
        lo = L.rowptr[u[e]]
        pos[e] = lo + np.searchsorted(L.col[lo:L.rowptr[u[e] + 1]], v[e])

    def fwd_bwd():
        info = S.forward(b)
        x = info.solution - info.solution.mean()
        dw, db = S.backward(x - xt)
        return x, dw[pos], db, info
    for _ in range(args.warmup):
        fwd_bwd()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        x, gw, gb, info = fwd_bwd()
    value = (time.perf_counter() - t0) * 1e3 / args.steps

    # Central differences of the loss, each perturbed system solved to rtol
    # 1e-12.  The perturbed solution is written x + d, d solving the perturbed
    # system's residual equation L' d = b' - L' x from a fresh setup on L', and
    # loss(+) - loss(-) = (x - x_t).(d+ - d-) + (|d+|^2 - |d-|^2) / 2, which
    # keeps the O(h) change of the loss free of the cancellation between two
    # losses of size ~n.
    def dloss(dp, dm):
        return float(np.dot(x - xt, dp - dm) + 0.5 * (np.dot(dp, dp) - np.dot(dm, dm)))

    def corr_w(wv):
        Lp = G.laplacian_from_edges(n, u, v, wv)
        Sx = Solver(Lp, **kw)
        d = Sx.solve(b - Lp.to_scipy() @ x).solution
        Sx.close()
        return d - d.mean()

    def corr_b(bv):
        d = S.solve(bv - L.to_scipy() @ x).solution
        return d - d.mean()
    t0 = time.perf_counter()
    ew = rng.choice(len(w), 64, replace=False)
    fd_w = []
    for e in ew:
        h = 1e-6 * w[e]
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd_w.append(dloss(corr_w(wp), corr_w(wm)) / (2 * h))
    ib = rng.choice(n, 64, replace=False)
    fd_b = []
    for i in ib:
        bp, bm = b.copy(), b.copy()
        bp[i] += 1e-6
        bm[i] -= 1e-6
        fd_b.append(dloss(corr_b(bp), corr_b(bm)) / 2e-6)
    fd_s = time.perf_counter() - t0
    fd_w, fd_b = np.array(fd_w), np.array(fd_b)

    def rel(fd, g):
        return np.abs(fd - g) / np.maximum(np.abs(fd), 1e-300)
    # the oracle's own solves: x, then lambda = L^+ (x - x_t)
    O.set_threads(os.cpu_count() or 1)
    R = O.OracleSolver(L, **kw)
    t0 = time.perf_counter()
    xo, _ = R.solve(b)
    xo -= xo.mean()
    lam, _ = R.solve(xo - xt)
    lam -= lam.mean()
    cpu_ms = (time.perf_counter() - t0) * 1e3
    gw_o = -(xo[u] - xo[v]) * (lam[u] - lam[v])
    rw, rb = rel(fd_w, gw[ew]), rel(fd_b, gb[ib])
    out = {"metric": "gradient of 0.5||x - x_t||^2 through the solve: ms per forward+backward",
           "value": value, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": value, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {"workload": f"rmat{scale} (ef {EDGE_FACTOR}, w~U(0.5,2), LCC) n={n} "
                                  f"edges={len(u)}; FP64 K-cycle FCG rtol 1e-12; "
                                  "central differences with relative step 1e-6",
                      "forward_iters": info.iters(),
                      "edge_fd_rel_err_max": float(rw.max()),
                      "edge_fd_rel_err_median": float(np.median(rw)),
                      "edges_within_1e-5": int((rw <= 1e-5).sum()),
                      "b_fd_rel_err_max": float(rb.max()),
                      "b_within_1e-5": int((rb <= 1e-5).sum()),
                      "checked": "64 random edges, 64 random entries of b",
                      "vs_oracle_gradient_rel_err": float(np.linalg.norm(gw - gw_o) /
                                                          np.linalg.norm(gw_o)),
                      "vs_oracle_db_rel_err": float(np.linalg.norm(gb - lam) / np.linalg.norm(lam)),
                      "fd_seconds": fd_s},
           "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": os.cpu_count() or 1,
                            "kind": "port", "sample": "the forward and adjoint solves by the "
                                                      "oracle (FP64, rtol 1e-12), setup untimed"}}
    print(json.dumps(out), flush=True)


def main():
    global TAIL_ROWS
    args = parse()
    TAIL_ROWS = args.tail_rows
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "grid3d-ksweep":
        run_grid3d(args)
    elif args.workload == "rgg-batch":
        run_rgg_batch(args)
    elif args.workload == "grid2d":
        if args.grid == 128:
            args.grid = 256
        run_grid2d(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
