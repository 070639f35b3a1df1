#!/usr/bin/env python
"""Benchmark of the RBF-FD hot path on GB300.

Workload (one GPU): N = 1024 x 1024 = 1,048,576 jittered nodes on [0,1]^2 (h = 2^-10,
jitter +-0.3h, seed 1), PHS r^3, polynomial degree 3 (m = 10), k = 30 (s = 40); operators
Dx, Dy and Lap = Dxx + Dyy.  One step = the hot path over that node set: grid build, kNN
stencils, mixed-precision weight solves (FP32 LU, FP64 residual refinement, FP64 fallback)
writing CSR, then one SpMV of each operator on a random N(0,1) field.  Inputs are resident
in HBM when a step starts; L2 is flushed (256 MB write) before every step.

value = weight solves per second (rows of all operators' local systems solved per second,
whole job); the weights are verified against the FP64 GPU path over all rows and against
the CPU oracle on a sample (<= 1e-9 max row-relative error).

--impl reference: the reference algorithm's CPU path (the oracle port of the Julia code;
Julia is not installed) timed on all host cores on a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1024, help="grid side per GPU (N = nx^2 rows per GPU)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-phases", action="store_true", help="reference arm: skip the full-size CPU phase times")
    ap.add_argument("--workload", default="collocated", choices=["collocated", "uneven", "rk4"],
                    help="collocated: the headline line; uneven: mixed stencil sizes with boundary and ghost "
                         "classes (2,097,152 nodes); rk4: advection-diffusion-hyperviscosity RK4 on 2048^2 nodes")
    ap.add_argument("--total", type=int, default=2_097_152, help="uneven: number of nodes")
    ap.add_argument("--rk-nx", type=int, default=2048, help="rk4: grid side")
    ap.add_argument("--rk-steps", type=int, default=1000, help="rk4: time steps per precision")
    ap.add_argument("--no-uneven", action="store_true", help="headline line without the uneven-batch block")
    ap.add_argument("--no-rk4", action="store_true", help="headline line without the time-stepping block")
    ap.add_argument("--rk-fields", type=int, default=64, help="rk4: fields advanced together")
    return ap.parse_args()


WORKLOAD = dict(p=3, n=30, deg=3, ops=("Dx", "Dy", "Lap"))
METRIC = "weight solves/s at <=1e-9 rel err (FP32+refine vs FP64); stencil-apply HBM GB/s"


def workload_name(nx):
    """The headline workload as named in both arms' `config.workload`."""
    return (f"{nx}x{nx} jittered nodes per GPU (h=1/{nx}, +-0.3h), PHS r^3, deg 3 (m=10), "
            f"k=30 (s=40), ops Dx,Dy,Lap; step = grid+kNN+mixed solves+CSR + 1 SpMV per op")

# DRAM traffic per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum):
# the mixed solve on 512x512 nodes (262,144 systems; traffic is the gathered stencils and the
# CSR output, so it scales with the systems) and the SELL SpMV on 1024x1024 nodes (31.46 M nnz).
NCU_TRAFFIC = {"solve_bytes_per_system": (46.59e6 + 174.67e6) / 262144,
               "spmv_bytes_per_nnz": (385.90e6 + 4.11e6) / 31457280}


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth of MEASURED_PEAKS.json, else the fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm = json.load(open(path)).get("hbm_gbs") if os.path.exists(path) else None
    if hbm:
        return float(hbm), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6800 GB/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def shard_rows(rank, world, rows_per_rank):
    """Evaluation rows of one rank (weak scaling: every rank owns rows_per_rank rows)."""
    return rank * rows_per_rank, (rank + 1) * rows_per_rank


def max_over_ranks(value, dist=None):
    """Max of a per-rank float over all ranks (the job is as slow as its slowest rank)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def node_set(nx, ws):
    """Global node set: nx columns x (nx * ws) rows; rank r owns rows [r*nx^2, (r+1)*nx^2)."""
    import __graft_entry__

    pkg = __graft_entry__.load_package()
    X, h, _ = pkg.nodesets.jittered_grid(nx, nx * ws, 0.3, 1, box=((0.0, 1.0), (0.0, float(ws))))
    return X, h


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


def cpu_sample_rate(X, target_s, nthreads=0, seed=0):
    """Oracle (CPU restatement of the reference) weight solves per second on a random sample
    of rows of the workload; the sample size is grown until it takes about target_s."""
    from oracle import oracle as orc

    rng = np.random.default_rng(seed)
    p, n, deg, ops = WORKLOAD["p"], WORKLOAD["n"], WORKLOAD["deg"], WORKLOAD["ops"]
    size = 2000
    while True:
        rows = np.sort(rng.choice(len(X), size, replace=False))
        t0 = time.perf_counter()
        orc.generate(X, X[rows], p, n, deg, ops, nthreads=nthreads)
        dt = time.perf_counter() - t0
        if dt >= target_s * 0.5 or size >= len(X):
            return size / dt, size, dt
        size = min(len(X), int(size * max(2.0, target_s / max(dt, 1e-3))))


def cpu_description():
    """CPU model, logical core count and the oracle's compiler flags (oracle/Makefile)."""
    model = None
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
            for line in out.splitlines():
                if line.startswith("Model name:"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    flags = None
    for line in open(os.path.join(ROOT, "oracle", "Makefile")):
        if line.startswith("CFLAGS"):
            flags = line.split("=", 1)[1].strip()
    return {"cpu_model": model, "host_cores": os.cpu_count(), "compiler": "gcc", "compiler_flags": flags}


def cpu_phases(X, solve_rate, seed=11):
    """Per-phase CPU times of the oracle at the full node count: kNN of every node (all
    threads), the weight solves (extrapolated from the sampled rate), sparse(I, J, V) of one
    operator, and one SpMV both as single-threaded CSC (Julia's `*`) and as threaded row form."""
    from oracle import oracle as orc

    N, n = len(X), WORKLOAD["n"]
    t0 = time.perf_counter()
    cols, _ = orc.knn(X, X, n)
    knn_ms = 1e3 * (time.perf_counter() - t0)
    W = np.random.default_rng(seed).standard_normal((N, n))
    t0 = time.perf_counter()
    colptr, rowval, nzval = orc.to_csc(N, N, cols, W)
    csc_ms = 1e3 * (time.perf_counter() - t0)
    x = np.random.default_rng(seed + 1).standard_normal(N)
    t0 = time.perf_counter()
    y_csc = orc.spmv_csc(N, colptr, rowval, nzval, x)
    spmv_csc_ms = 1e3 * (time.perf_counter() - t0)
    orc.spmv_rows(cols, W, x)
    t0 = time.perf_counter()
    y_rows = orc.spmv_rows(cols, W, x)
    spmv_rows_ms = 1e3 * (time.perf_counter() - t0)
    if not np.allclose(y_csc, y_rows, rtol=1e-12, atol=1e-12):
        raise RuntimeError("CPU SpMV forms disagree")
    return {
        "knn_all_nodes": knn_ms,
        "solves_all_nodes_extrapolated": 1e3 * N / solve_rate,
        "csc_build_per_op": csc_ms,
        "spmv_csc_1_thread": spmv_csc_ms,
        "spmv_rows_all_threads": spmv_rows_ms,
    }


def run_reference(args):
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    from oracle import oracle as orc

    X, _ = node_set(args.nx, 1)
    cores = orc.max_threads()
    rate0, size, dt = cpu_sample_rate(X, max(2.0, args.cpu_seconds / max(1, args.steps + args.warmup)))
    rng = np.random.default_rng(7)
    p, n, deg, ops = WORKLOAD["p"], WORKLOAD["n"], WORKLOAD["deg"], WORKLOAD["ops"]
    times = []
    for it in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(len(X), size, replace=False))
        t0 = time.perf_counter()
        orc.generate(X, X[rows], p, n, deg, ops)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    value = size / (ms * 1e-3)
    rate1, size1, dt1 = cpu_sample_rate(X, max(2.0, args.cpu_seconds / 2), nthreads=1, seed=1)
    phases = cpu_phases(X, value) if not args.no_cpu_phases else None
    sample = (f"{size} random rows of the {len(X)}-node workload per step (stencils, explicit "
              f"inverse of the 40x40 system, weights of Dx/Dy/Lap), C oracle port, {cores} threads")
    print(json.dumps({
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded jittered grid)",
        "config": {"workload": workload_name(args.nx), "rows_per_step": size,
                   "parallelism": f"host cores x{cores}"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample,
                         "value_1_thread": rate1, "sample_1_thread": f"{size1} random rows, 1 thread, {dt1:.1f} s",
                         "phases_ms_full_size": phases, **cpu_description()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def manufactured_errors(pkg, h):
    """The 64x64 manufactured-solution case (p=3, deg 2, k=15): f = sin(2 pi x) cos(3 pi y)
    applied through the device operators of both precisions (SELL SpMV); max error on the
    interior nodes (|x - 1/2|, |y - 1/2| < 0.35) relative to the exact derivative's max."""
    import torch

    X, _, _ = pkg.nodesets.jittered_grid(64, seed=1)
    f, fx, fy, lap = pkg.nodesets.manufactured(X)
    inner = (np.abs(X - 0.5) < 0.35).all(1)
    exact = {"Dx": fx, "Dy": fy, "Lap": lap}
    out = {}
    for prec in ("fp64", "mixed"):
        with pkg.OperatorSet(X, None, 3, 15, 2, ops=("Dx", "Dy", "Lap"), precision=prec, handle=h) as s:
            fd = torch.tensor(f, device="cuda")
            yd = torch.empty_like(fd)
            for o, ex in exact.items():
                y = s.spmv(o, fd, yd).cpu().numpy()
                out[f"{prec}_{o}"] = float(np.abs(y - ex)[inner].max() / np.abs(ex).max())
    return out


def row_rel_err(a, b, n):
    """max over rows of ||a_i - b_i||_inf / ||b_i||_inf for row-major (rows, n) torch tensors."""
    import torch

    a = a.view(-1, n)
    b = b.view(-1, n)
    num = (a - b).abs().amax(1)
    den = b.abs().amax(1)
    return float((num / den).max().item()), float((num / den).median().item())


def run_ours(args):
    import torch

    import __graft_entry__

    pkg = __graft_entry__.load_package()
    nat = pkg._native
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = nat.load()
    h = pkg.Handle(device=local)
    st_ptr = h.stream
    stream = torch.cuda.ExternalStream(st_ptr)
    p, n, deg, ops = WORKLOAD["p"], WORKLOAD["n"], WORKLOAD["deg"], WORKLOAD["ops"]
    X_host, hgrid = node_set(args.nx, ws)
    N = len(X_host)
    rows_per = args.nx * args.nx
    rb, re = shard_rows(rank, ws, rows_per)
    fp64_peak, fp32_peak = ctypes.c_double(), ctypes.c_double()
    L.rbffd_measure_fma_peaks(local, ctypes.byref(fp64_peak), ctypes.byref(fp32_peak))

    with torch.cuda.stream(stream):
        Xd = torch.tensor(X_host, device="cuda")
        gen = torch.Generator(device="cuda")
        gen.manual_seed(1234)
        xfield = torch.randn(N, dtype=torch.float64, device="cuda", generator=gen)
        ys = [torch.empty(rows_per, dtype=torch.float64, device="cuda") for _ in ops]
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream.synchronize()

    def opset(precision):
        return pkg.OperatorSet(Xd, None, p, n, deg, ops=ops, precision=precision, row_range=(rb, re), handle=h,
                               device=True)

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def step(precision, collect):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = ev(), ev()
        e0.record(stream)
        s = opset(precision)
        for q, o in enumerate(ops):
            s.spmv_ptr(o, xfield.data_ptr(), ys[q].data_ptr())
        e1.record(stream)
        e1.synchronize()
        collect.append((e0.elapsed_time(e1), s.stats.as_dict()))
        s.close()

    # ---- verification (untimed): mixed vs FP64 GPU over all rows, both vs the oracle on a sample
    s64 = opset("fp64")
    smx = opset("mixed")
    err_all = {}
    for q, o in enumerate(ops):
        with torch.cuda.stream(stream):
            err_all[o] = row_rel_err(smx.device_values(o), s64.device_values(o), n)
    mixed_stats = smx.stats.as_dict()
    from oracle import oracle as orc

    rng = np.random.default_rng(3)
    sample = np.sort(rng.choice(np.arange(rb, re), 2000, replace=False))
    ref = orc.generate(X_host, X_host[sample], p, n, deg, ops)
    err_oracle = {}
    for q, o in enumerate(ops):
        for name, s in (("fp64", s64), ("mixed", smx)):
            _, _, val = s.csr_arrays(o)
            W = val.reshape(-1, n)[sample - rb]
            e = np.abs(W - ref["W"][q]).max(1) / np.abs(ref["W"][q]).max(1)
            err_oracle[f"{name}_{o}"] = float(e.max())
    s64.close()
    smx.close()

    # ---- timed steps (mixed = the metric), then the FP64 form for the ratio
    for _ in range(args.warmup):
        step("mixed", [])
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    t_wall = time.perf_counter()
    timed = []
    for _ in range(args.steps):
        step("mixed", timed)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - t_wall
    clocks = clk.stop()
    ms_step = max_over_ranks(float(np.mean([t for t, _ in timed])), dist)
    total_rows = rows_per * ws
    value = total_rows / (ms_step * 1e-3)

    fp64_steps = []
    for _ in range(1):
        step("fp64", [])
    for _ in range(max(2, args.steps // 2)):
        step("fp64", fp64_steps)
    ms_fp64 = float(np.mean([t for t, _ in fp64_steps]))

    # ---- kernel-level numbers: solve kernel (from the library's events) and SpMV
    st_mixed = [s for _, s in timed]
    solve_ms = float(np.mean([s["ms_solve"] for s in st_mixed]))
    knn_ms = float(np.mean([s["ms_knn"] for s in st_mixed]))
    solve_ms_fp64 = float(np.mean([s["ms_solve"] for _, s in fp64_steps]))
    s = opset("mixed")
    spmv_times = []
    for it in range(12):
        e0, e1 = ev(), ev()
        e0.record(stream)
        s.spmv_ptr("Lap", xfield.data_ptr(), ys[2].data_ptr())
        e1.record(stream)
        e1.synchronize()
        if it >= 2:
            spmv_times.append(e0.elapsed_time(e1))
    spmv_ms = float(np.mean(spmv_times))
    nnz = s.nnz
    # algorithmic bytes: weights + int32 columns, row pointers (int32 count), x read once, y written once
    spmv_bytes = nnz * (8 + 4) + (rows_per + 1) * 4 + N * 8 + rows_per * 8
    spmv_gbs = spmv_bytes / (spmv_ms * 1e-3) / 1e9
    s.close()

    # ---- e2e: the drop-in C-ABI call with host buffers (H2D of X, D2H of the CSC operators)
    e2e = None
    if not args.no_e2e and ws == 1:
        mask = sum(1 << nat.OP_CODES[o] for o in ops)
        pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True)  # noqa: E731
        Xp = pin((N, 2), torch.float64)
        Xp.copy_(torch.from_numpy(X_host))
        outs = (nat.CSC * len(ops))()
        keep = []
        for q in range(len(ops)):
            cp, rv, nz = pin(N + 1, torch.int64), pin(N * n, torch.int64), pin(N * n, torch.float64)
            keep += [cp, rv, nz]
            outs[q].colptr, outs[q].rowval, outs[q].nzval = cp.data_ptr(), rv.data_ptr(), nz.data_ptr()
        est = nat.Stats()
        e2e_t = []
        for it in range(1 + max(3, args.steps // 2)):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            stream.synchronize()
            t0 = time.perf_counter()
            rc = L.rbffd_generate_operator(h.ptr, ctypes.c_void_p(Xp.data_ptr()), N, ctypes.c_void_p(Xp.data_ptr()),
                                           N, p, n, deg, None, mask, nat.PREC["mixed"], outs, ctypes.byref(est))
            dt = time.perf_counter() - t0
            nat.check(h.ptr, rc)
            if it >= 1:
                e2e_t.append(dt)
        ms_e2e = 1e3 * float(np.median(e2e_t))  # host copies vary with the pinned pages' placement
        e2e = {
            "value": N / (ms_e2e * 1e-3),
            "unit": "solves/s",
            "ms_per_call": ms_e2e,
            "h2d_bytes_per_step": N * 16,
            "d2h_bytes_per_step": len(ops) * (N * n * 16 + (N + 1) * 8),
            "call": "rbffd_generate_operator (host X in, caller-allocated pinned CSC out, Dx/Dy/Lap, mixed)",
        }

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- CPU baseline (oracle port, host cores, bounded sample)
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as orc

        rate, size, dt = cpu_sample_rate(X_host[: rows_per] if ws == 1 else X_host, args.cpu_seconds)
        rate1, size1, dt1 = cpu_sample_rate(X_host[: rows_per] if ws == 1 else X_host, args.cpu_seconds / 2,
                                            nthreads=1, seed=1)
        cpu = {"value": rate, "unit": "solves/s", "cores": orc.max_threads(), "kind": "port",
               "sample": f"{size} random rows of the {rows_per}-node workload (kNN, explicit inverse, Dx/Dy/Lap "
                         f"weights), C oracle port, {dt:.1f} s",
               "value_1_thread": rate1,
               "sample_1_thread": f"{size1} random rows, 1 thread, {dt1:.1f} s",
               **cpu_description()}

    manu = manufactured_errors(pkg, h)
    m = 10
    s_ = n + m
    # FP64 work of the mixed solve per system: the monomials of P (7 products per node at
    # degree 3), the closed-form right-hand sides of Dx/Dy/Lap for r^3 (29 flops per node: r^2,
    # r and 1/r by Newton steps, 3r, the three values), the first refinement residual
    # 2 (s^2 - m^2) r and the output (hi + lo, and the scale of Dx/Dy: 5 per node).  The
    # pairwise Phi = r^3 is exact fixed-point integer work, and the later residuals and the
    # solution updates are double-float FP32: none of them is FP64 work or counted.
    fp64_flops_sys = 7 * n + 29 * n + 2 * (s_ * s_ - m * m) * 3 + 5 * n
    hist = mixed_stats["refine_hist"]
    solve_ach = rows_per * fp64_flops_sys / (solve_ms * 1e-3) / 1e12
    hbm, hbm_src = hbm_peak()
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded jittered grid, splitmix64)",
        "config": {
            "workload": workload_name(args.nx),
            "rows_per_gpu": rows_per,
            "l2": "flushed (256 MB write) before every step",
            "parallelism": f"row shards x{ws}" if ws > 1 else "single GPU",
        },
        "e2e": e2e,
        "gpu_launches": int(np.mean([s["kernel_launches"] for s in st_mixed])) + len(ops),
        "clocks": clocks,
        "wall_s_timed_region": wall,
        "accuracy": {
            "max_row_rel_err_mixed_vs_fp64_gpu_all_rows": {o: v[0] for o, v in err_all.items()},
            "median_row_rel_err_mixed_vs_fp64_gpu": {o: v[1] for o, v in err_all.items()},
            "max_row_rel_err_vs_oracle_2000_rows": err_oracle,
            "fallback_fraction": mixed_stats["n_fallback"] / max(1, mixed_stats["n_systems"]),
            "refine_hist": hist,
            "manufactured_64x64_k15_deg2_rel_err": manu,
        },
        "fp64_form": {"value": rows_per * ws / (ms_fp64 * 1e-3), "ms_per_step": ms_fp64,
                      "solve_kernel_ms": solve_ms_fp64},
        "mixed_over_fp64": ms_fp64 / ms_step,
        "mixed_over_fp64_solve_kernel": solve_ms_fp64 / solve_ms,
        "phases_ms": {"knn": knn_ms, "solve_mixed": solve_ms, "spmv_per_op": spmv_ms,
                      "grid": float(np.mean([s["ms_grid"] for s in st_mixed]))},
        "measured_fma_peaks_tflops": {"fp64": fp64_peak.value, "fp32": fp32_peak.value},
        "solve_autotune": h.autotune_report(),
        "roofline": {
            "kernel": "solve_mixed_schur_kernel",
            "bound": "fp64",
            "achieved": solve_ach,
            "peak": fp64_peak.value,
            "unit": "TFLOP/s",
            "frac": solve_ach / fp64_peak.value if fp64_peak.value else None,
            "traffic": NCU_TRAFFIC["solve_bytes_per_system"] * rows_per,
            "traffic_note": "bytes per launch, ncu on 512x512 scaled by systems (stencil gathers + CSR output)",
            "note": "FP64 work of the mixed solve (P monomials, closed-form right-hand sides, first residual, "
                    "output; Phi = r^3 is exact fixed-point integer work, the later residuals and the updates "
                    "double-float FP32) over the kernel's "
                    "event-timed duration, against the measured FP64 FMA peak (rbffd_measure_fma_peaks); the kernel "
                    "is latency/issue-bound with the FP64 pipe one of several busy units (profiles/)",
        },
        "roofline_apply": {
            "kernel": "spmv_f64_sell",
            "bound": "hbm",
            "achieved": spmv_gbs,
            "peak": hbm,
            "unit": "GB/s",
            "frac": spmv_gbs / hbm,
            "traffic": NCU_TRAFFIC["spmv_bytes_per_nnz"] * nnz,
            "algorithmic_bytes": spmv_bytes,
            "peak_source": hbm_src,
        },
        "cpu_baseline": cpu,
    }
    # the uneven-batch and time-stepping workloads, measured after the headline (one GPU)
    if ws == 1 and not args.no_uneven:
        out["uneven"] = uneven_block(uneven_results(args, 2, 1))
    if ws == 1 and not args.no_rk4:
        out["rk4"] = rk4_block(rk4_results(args))
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def uneven_results(args, steps, warmup):
    """Mixed stencil sizes, boundary and ghost classes: rectangle [0,2]x[0,1] with 4 boundaries
    and one ghost layer, per-node (k, deg) in {(20,2), (30,3), (45,4), (60,5)} (85% (30,3)),
    boundary-class-masked kNN, Dx/Dy/Lap with PHS r^3 and Dxk/Dyk (K=4) with PHS r^5; mixed
    against plain FP64."""
    import torch

    import __graft_entry__

    pkg = __graft_entry__.load_package()
    d = pkg.nodesets.rectangle_with_ghosts(total=args.total, seed=4)
    X, cls, nn, dd = d["X"], d["node_class"], d["n"], d["deg"]
    h = pkg.Handle()
    Xd = torch.tensor(X, device="cuda")
    cd = torch.tensor(cls, dtype=torch.int32, device="cuda")
    nd = torch.tensor(nn, dtype=torch.int32, device="cuda")
    ddev = torch.tensor(dd, dtype=torch.int32, device="cuda")
    sets = {"ops": (3, ("Dx", "Dy", "Lap"), 0), "hyperviscosity": (5, ("Dxk", "Dyk"), 4)}
    res = {}
    vals = {}
    for name, (p, ops, kd) in sets.items():
        for prec in ("mixed", "fp64"):
            ts, st = [], None
            for it in range(warmup + steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s = pkg.OperatorSet(Xd, None, p, 0, 0, ops=ops, precision=prec, node_class=cd, n_per_node=nd,
                                    deg_per_node=ddev, k_deriv=kd, handle=h, device=True)
                torch.cuda.synchronize()
                if it >= warmup:
                    ts.append(time.perf_counter() - t0)
                st = s.stats.as_dict()
                if it == warmup + steps - 1:
                    rp = s.device_csr(ops[0])[0]
                    rpt = torch.as_tensor(pkg.operators._DeviceArray(rp, s.rows + 1, "<i8"), device="cuda").clone()
                    vals[(name, prec)] = ([s.device_values(o).clone() for o in ops], rpt)
                s.close()
            ms = 1e3 * float(np.mean(ts))
            res[f"{name}_{prec}"] = {"solves_per_s": len(X) / (ms * 1e-3), "ms_per_build": ms,
                                     "ms_knn": st["ms_knn"], "ms_solve": st["ms_solve"],
                                     "ms_fallback": st["ms_fallback"], "fallback": st["n_fallback"],
                                     "refine_hist": st["refine_hist"], "kernel_launches": st["kernel_launches"]}
        errs = {}
        rpt = vals[(name, "fp64")][1]
        lengths = rpt[1:] - rpt[:-1]
        rid = torch.repeat_interleave(torch.arange(len(lengths), device="cuda"), lengths)
        for q, o in enumerate(sets[name][1]):
            a, b = vals[(name, "mixed")][0][q], vals[(name, "fp64")][0][q]
            num = torch.zeros(len(lengths), dtype=torch.float64, device="cuda").scatter_reduce_(
                0, rid, (a - b).abs(), "amax")
            den = torch.zeros_like(num).scatter_reduce_(0, rid, b.abs(), "amax")
            e = num / den
            errs[o] = {"max": float(e.max().item()), "median": float(e.median().item())}
        res[f"{name}_row_rel_err_mixed_vs_fp64"] = errs
        res[f"{name}_mixed_over_fp64"] = res[f"{name}_fp64"]["ms_solve"] / res[f"{name}_mixed"]["ms_solve"]
    out = {"workload": "uneven: rectangle [0,2]x[0,1], 4 boundaries + ghosts, per-node (k,deg) "
                       "{(20,2),(30,3),(45,4),(60,5)}, boundary-masked kNN",
           "nodes": int(len(X)), "counts": d["counts"],
           "steps": steps, "warmup": warmup, "timing": "wall clock of the whole device build, "
           "inputs resident in HBM", "solve_autotune": h.autotune_report(), **res}
    h.close()
    return out


def uneven_block(u):
    """The uneven workload's figures for the headline line."""
    blk = {"workload": u["workload"], "nodes": u["nodes"], "per_class": u["counts"]["per_class"],
           "boundary_nodes": u["counts"]["boundary"], "ghost_nodes": u["counts"]["ghost"]}
    for name, label in (("ops", "Dx,Dy,Lap (r^3)"), ("hyperviscosity", "Dxk,Dyk (r^5, K=4)")):
        mx, f64 = u[f"{name}_mixed"], u[f"{name}_fp64"]
        blk[name] = {
            "operators": label,
            "solves_per_s_mixed": mx["solves_per_s"], "solves_per_s_fp64": f64["solves_per_s"],
            "ms_build_mixed": mx["ms_per_build"], "ms_build_fp64": f64["ms_per_build"],
            "ms_solve_mixed": mx["ms_solve"] + mx["ms_fallback"], "ms_solve_fp64": f64["ms_solve"],
            "mixed_over_fp64_solves": f64["ms_solve"] / (mx["ms_solve"] + mx["ms_fallback"]),
            "mixed_over_fp64_build": f64["ms_per_build"] / mx["ms_per_build"],
            "row_rel_err_mixed_vs_fp64": u[f"{name}_row_rel_err_mixed_vs_fp64"],
            "fallback_fraction": mx["fallback"] / u["nodes"], "refine_hist": mx["refine_hist"],
        }
    blk["solve_autotune"] = u["solve_autotune"]
    return blk


def run_uneven(args):
    print(json.dumps(uneven_results(args, args.steps, args.warmup)))


def rk4_results(args):
    """du/dt = L u, L = -a.grad + nu Lap - gamma (Dxk + Dyk), a = (1, 0.5), nu = 1e-3,
    gamma = 100 h^4 (examples/adv_diff_test.jl:152), Dxk/Dyk with K = 4 and PHS r^5; RK4 with
    dt = 0.2 h (reduced to the largest stable step when rho(L) dt exceeds RK4's real-axis
    limit), rows within one spacing of the boundary held fixed, F fields of 8 seeded Gaussians;
    FP64 and FP32 weights and fields, drift ||u32 - u64|| / ||u64||."""
    import torch

    import __graft_entry__

    pkg = __graft_entry__.load_package()
    nx = args.rk_nx
    X, hh, _ = pkg.nodesets.jittered_grid(nx, seed=5)
    N = len(X)
    h = pkg.Handle()
    Xd = torch.tensor(X, device="cuda")
    t0 = time.perf_counter()
    s3 = pkg.OperatorSet(Xd, None, 3, 30, 3, ops=("Dx", "Dy", "Lap"), precision="mixed", handle=h, device=True)
    s5 = pkg.OperatorSet(Xd, None, 5, 30, 3, ops=("Dxk", "Dyk"), precision="mixed", k_deriv=4, handle=h,
                         device=True)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    nu, gamma = 1e-3, 100.0 * hh ** 4
    coef = [-1.0, -0.5, nu, -gamma, -gamma]
    fixed = ((X[:, 0] < hh) | (X[:, 0] > 1 - hh) | (X[:, 1] < hh) | (X[:, 1] > 1 - hh)).astype(np.uint8)
    F = args.rk_fields
    rng = np.random.default_rng(11)
    cx, cy = rng.uniform(0, 1, (F, 8)), rng.uniform(0, 1, (F, 8))
    sg, am = rng.uniform(0.05, 0.15, (F, 8)), rng.uniform(-1, 1, (F, 8))
    Xt = torch.tensor(X, device="cuda")
    u0 = torch.zeros(N, F, dtype=torch.float64, device="cuda")
    for f in range(F):
        for g in range(8):
            r2 = (Xt[:, 0] - cx[f, g]) ** 2 + (Xt[:, 1] - cy[f, g]) ** 2
            u0[:, f] += am[f, g] * torch.exp(-r2 / (2 * sg[f, g] ** 2))
    out = {"workload": f"rk4: {nx}x{nx} jittered nodes, k=30, deg 3, L = -a.grad + nu Lap - gamma (Dxk + Dyk)",
           "nodes": N, "fields": F, "nnz_per_operator": s3.nnz, "build_s": t_build,
           "fixed_rows": int(fixed.sum())}
    rk = {}
    for dt_name in ("f64", "f32"):
        rk[dt_name] = pkg.RK4Stepper([s3, s5], coef, F, dtype=dt_name, fixed_rows=fixed, handle=h)
    # rho(L) by power iteration on one field (FP64)
    one = pkg.RK4Stepper([s3, s5], coef, 1, dtype="f64", fixed_rows=fixed, handle=h)
    v = torch.randn(N, 1, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    held = torch.tensor(fixed, device="cuda").bool()
    v[held] = 0
    w = torch.empty_like(v)
    lam = 0.0
    for _ in range(100):  # the operator of the dynamics: rows held fixed have du = 0
        v /= v.norm()
        one.apply(v, w)
        w[held] = 0
        lam = float(w.norm().item())
        v, w = w, v
    one.close()
    dt = 0.2 * hh
    limit = 2.78
    stable = lam * dt <= limit
    dt_used = dt if stable else 0.9 * limit / lam
    out.update({"rho_L": lam, "dt_nominal": dt, "rho_dt_nominal": lam * dt, "rk4_limit": limit,
                "stable_at_nominal_dt": bool(stable), "dt_used": dt_used})
    res = {}
    stream = torch.cuda.ExternalStream(h.stream)
    hbm = hbm_peak()[0]
    for dt_name, tdt in (("f64", torch.float64), ("f32", torch.float32)):
        u = u0.to(tdt).contiguous().clone()
        rk[dt_name].run(u, dt_used, 2)  # warm-up (graph capture)
        u = u0.to(tdt).contiguous().clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rk[dt_name].run(u, dt_used, args.rk_steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        res[dt_name] = (u, ms)
        sz = 8 if dt_name == "f64" else 4
        nnz = s3.nnz
        # one Horner stage out = u + c L v: the weights and column ids once, the stage input v
        # and the state u read once each and the result written once; the first stage of a
        # step has v = u (one array read), so a step moves 4 nnz (sz + 4) + 11 N F sz bytes
        step_bytes = 4 * nnz * (sz + 4) + (2 + 3 * 3) * N * F * sz
        stage_bytes = step_bytes / 4
        gbps = args.rk_steps * step_bytes / (ms * 1e-3) / 1e9
        out[f"{dt_name}"] = {"ms_per_step": ms / args.rk_steps, "steps": args.rk_steps,
                             "stage_algorithmic_bytes": stage_bytes,
                             "stage_bytes_note": "mean over the 4 Horner stages: weights + column ids, v and u "
                                                 "read once (v = u in stage 1), out written once",
                             "stage_GBps_without_u": args.rk_steps * (4 * nnz * (sz + 4) + 8 * N * F * sz)
                                                     / (ms * 1e-3) / 1e9,
                             "stage_algorithmic_GBps": gbps, "stage_frac_of_hbm": gbps / hbm,
                             "stage_fma_TFLOPs": 4 * args.rk_steps * 2.0 * nnz * F / (ms * 1e-3) / 1e12,
                             "finite": bool(torch.isfinite(u).all().item())}
    u64, u32 = res["f64"][0], res["f32"][0].double()
    out["drift_f32_vs_f64"] = float(((u32 - u64).norm() / u64.norm()).item())
    out["hbm_peak_GBps"] = hbm
    for r in rk.values():
        r.close()
    s3.close()
    s5.close()
    h.close()
    return out


def rk4_block(r):
    """The time-stepping workload's figures for the headline line."""
    keys = ("workload", "nodes", "fields", "nnz_per_operator", "fixed_rows", "rho_L", "dt_nominal",
            "rho_dt_nominal", "stable_at_nominal_dt", "dt_used", "drift_f32_vs_f64", "hbm_peak_GBps")
    blk = {k: r[k] for k in keys}
    for p in ("f64", "f32"):
        blk[p] = {k: r[p][k] for k in ("ms_per_step", "steps", "stage_algorithmic_bytes", "stage_algorithmic_GBps",
                                       "stage_frac_of_hbm", "stage_GBps_without_u", "stage_bytes_note",
                                       "stage_fma_TFLOPs", "finite")}
    return blk


def run_rk4(args):
    print(json.dumps(rk4_results(args)))


def main():
    args = parse()
    if args.workload == "uneven":
        run_uneven(args)
        return
    if args.workload == "rk4":
        run_rk4(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
