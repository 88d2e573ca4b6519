"""Benchmark of the nalgebra dense-solve hot path on GB300.

Default workload (the headline): ragged batched Cholesky -- 20000 SPD systems
with n uniform in [8, 256], A = B B^T + n I, B ~ N(0,1) f64, 4 right-hand sides
~ N(0,1) each -- factor + solve + log-determinant of every system in ONE
persistent launch (nacu_dposv_ragged), against one plain FP64 launch per
matrix (nacu_dposv) and nalgebra's CPU path (the oracle restatement) on the
host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload ragged_cholesky|lu_batched]

Prints ONE JSON line.  A "step" is one pass of the hot path over the whole
batch.  The factorization is in place, so each step first restores the input
from a pristine device copy; that restore is outside the timed events (CUDA
events bracket each kernel launch on its stream).  Inputs (3.4 GB) are larger
than the 129 MB L2, so no extra flush is needed.
"""
from __future__ import annotations

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

EPS64 = 2.220446049250313e-16
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")


# ----------------------------------------------------------------------------- util

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def read_peaks():
    try:
        with open(PEAKS_PATH) as f:
            return json.load(f)
    except Exception:
        return {}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def combine_over_ranks(res, units, world, device="cuda"):
    """Whole-job figures of `world` independent replicas that each process
    `units` per step: the slowest rank's time per step (MAX over ranks), for
    the device-timed figure and for the end-to-end one, and units * world over
    that time.  Every rank must call it (a collective)."""
    if world <= 1:
        return res
    import torch

    e2e = res.get("e2e") or {}
    t = torch.tensor([float(res["ms_per_step"]), float(e2e.get("ms_per_step", 0.0))], dtype=torch.float64,
                     device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    res["ms_per_step"] = float(t[0])
    res["value"] = units * world / (res["ms_per_step"] * 1e-3)
    if e2e.get("ms_per_step"):
        e2e["ms_per_step"] = float(t[1])
        e2e["value"] = units * world / (e2e["ms_per_step"] * 1e-3)
    return res


# ----------------------------------------------------------------------------- ragged Cholesky

RAGGED = dict(count=20000, n_lo=8, n_hi=256, nrhs=4, seed=0)


def active_buckets(n_max):
    """Size buckets of the ragged launch that can hold an order <= n_max (bucket b
    holds orders above the previous bound; bucket 0 is always launched)."""
    bounds = (32, 64, 96, 128, 192, 256, 384, 512)
    return 1 + sum(1 for b in range(1, len(bounds)) if bounds[b - 1] < n_max)


def ragged_flops(ns, nrhs):
    ns = ns.astype(np.float64)
    return float(np.sum(ns ** 3 / 3.0 + nrhs * 2.0 * ns ** 2))


def ragged_bytes(ns, nrhs):
    # read A (lower), write L (lower), read B, write X, 8 bytes each
    ns = ns.astype(np.float64)
    return float(np.sum(8.0 * ns * (ns + 1) + 2 * 8.0 * nrhs * ns))


def batch_accuracy(ns, aoff, a_host, boff, b_host, x_host, nrhs, x_ref=None):
    """Accuracy of every system of the batch (host, outside the timed events):
    the normwise backward error with the residual by Dot2 (the oracle's
    compensated dot), in units of n * eps64, and -- given the oracle's FP64
    solutions x_ref -- the forward error ||x - x_ref||_inf / ||x_ref||_inf per
    right-hand side."""
    import oracle as O

    berr = O.ragged_backward_errors(ns, aoff, a_host, boff, b_host, x_host, nrhs)
    units = berr / (ns.astype(np.float64) * EPS64)
    out = {"backward_error_max_over_batch_in_n_eps": float(np.max(units)),
           "systems_above_n_eps": int(np.sum(~(units <= 1.0))), "systems_checked": int(ns.size)}
    if x_ref is not None:
        # one segment per (system, right-hand side): rows boff[s] + c*n ... + n
        ns64 = ns.astype(np.int64)
        packed = bool(np.all(np.diff(boff) == ns64[:-1] * nrhs)) and int(boff[-1] + ns64[-1] * nrhs) == x_host.size
        starts = (boff[:, None] + np.arange(nrhs)[None, :] * ns64[:, None]).ravel()[np.repeat(ns, nrhs) > 0]
        if packed and starts.size:
            d = np.maximum.reduceat(np.abs(x_host - x_ref), starts)
            r = np.maximum.reduceat(np.abs(x_ref), starts)
        else:
            lens = np.repeat(ns64, nrhs)[np.repeat(ns, nrhs) > 0]
            d = np.array([np.max(np.abs(x_host[a:a + k] - x_ref[a:a + k])) for a, k in zip(starts, lens)])
            r = np.array([np.max(np.abs(x_ref[a:a + k])) for a, k in zip(starts, lens)])
        out["forward_error_max_vs_fp64_oracle_over_batch"] = float(np.max(d / np.where(r > 0, r, 1.0))) if d.size else 0.0
    return out


def oracle_solutions(ns, aoff, a_host, boff, b_host, nrhs):
    """The oracle's FP64 solutions of the whole batch (nalgebra's
    Cholesky::solve restated), all host threads."""
    import oracle as O

    return O.posv_ragged(ns, aoff, a_host, boff, b_host, nrhs)[1]


def bench_ragged_ours(args, rank, world):
    import torch

    from nalgebra_gb300 import DeviceBatch, _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = dict(RAGGED)
    if args.count:
        cfg["count"] = args.count
    w = W.ragged_spd_torch(cfg["count"], cfg["n_lo"], cfg["n_hi"], cfg["nrhs"], seed=cfg["seed"] + rank, device=dev)
    ns, aoff, boff, nrhs = w["ns"], w["a_offsets"], w["b_offsets"], cfg["nrhs"]
    count = ns.size
    a0, b0 = w["a_flat"], w["b_flat"]
    A = a0.clone()
    B = b0.clone()
    batch = DeviceBatch(A, ns, ns, aoff)
    rhs = DeviceBatch(B, ns, np.full(count, nrhs), boff)
    chol = batch.cholesky()
    info_t = torch.as_tensor(chol.info, device=dev)  # torch views of the mirror's buffers
    logdet_t = torch.as_tensor(chol.logdet, device=dev)
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    n_max = int(ns.max())
    from nalgebra_gb300 import tuning

    tune_res = tuning.autotune(per_bucket=2500, save=False) if args.autotune else None
    tiles_table = tuning.current(L)

    def launch():  # the stream is read at call time: inside a capture it is the capture stream
        _lib.call("nacu_dposv_ragged", count, n_max, batch._d_rows.data_ptr(), batch._d_off.data_ptr(),
                  A.data_ptr(), nrhs, rhs._d_off.data_ptr(), B.data_ptr(), chol.info.data_ptr(),
                  chol.logdet.data_ptr(), chol._order.data_ptr() if args.single_launch else None,
                  chol._ws.data_ptr(), chol._ws.numel(), 0.0, 0, int(torch.cuda.current_stream().cuda_stream))

    def restore():
        A.copy_(a0)
        B.copy_(b0)

    for _ in range(args.warmup):
        restore()
        launch()
    torch.cuda.synchronize()
    # the batching form runs as a captured CUDA graph (memset + persistent launch)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        launch()
    stream = torch.cuda.current_stream()
    restore()
    info_t.fill_(-7)
    graph.replay()
    torch.cuda.synchronize()
    if int((info_t != 0).sum().item()) != 0:
        raise RuntimeError("graph replay did not run the factorization")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            restore()
            ev[i][0].record(stream)
            graph.replay()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    times = [e0.elapsed_time(e1) for e0, e1 in ev]
    kern_ms = float(np.mean(times))
    if args.profile:
        out = {"workload": "ragged_cholesky", "count": count, "ms_per_step": kern_ms}
        if args.profile_mixed:
            out["mixed"] = bench_ragged_mixed(args, L, ns, aoff, boff, a0, b0, nrhs, stream, a0.cpu().numpy(),
                                              b0.cpu().numpy())
            out["mixed"].pop("_objects")
        return out, None
    info = info_t.cpu().numpy()
    if np.any(info != 0):
        raise RuntimeError(f"{int(np.sum(info != 0))} systems failed to factor")
    # accuracy of the last step's solutions, every system of the batch
    rng = np.random.default_rng(1)
    a_host = a0.cpu().numpy()
    b_host = b0.cpu().numpy()
    x_host = B.cpu().numpy()
    x_ref = oracle_solutions(ns, aoff, a_host, boff, b_host, nrhs)
    acc64 = batch_accuracy(ns, aoff, a_host, boff, b_host, x_host, nrhs, x_ref)

    # precision form: FP32 factor + FP64 refinement, same inputs, one launch
    mixed = bench_ragged_mixed(args, L, ns, aoff, boff, a0, b0, nrhs, stream, a_host, b_host, x_ref)
    mchol, mrhs, mout = mixed.pop("_objects")
    use_mixed = mixed["systems_above_n_eps"] == 0 and mixed["ms_per_step"] < kern_ms

    # e2e through the public API from pinned host buffers (H2D of A and B in,
    # D2H of X, info and the per-matrix status out), inside the timed region.
    a_pin = torch.empty(a0.numel(), dtype=torch.float64, pin_memory=True)
    b_pin = torch.empty(b0.numel(), dtype=torch.float64, pin_memory=True)
    x_pin = torch.empty(b0.numel(), dtype=torch.float64, pin_memory=True)
    i_pin = torch.empty(count, dtype=torch.int32, pin_memory=True)
    l_pin = torch.empty(count, dtype=torch.float64, pin_memory=True)
    a_pin.copy_(a0)
    b_pin.copy_(b0)
    e2e_steps = max(1, min(args.steps, 5))
    # the mixed form from host memory: nacu_dposv_ragged_mixed_host pipelines
    # the copies in, the solves and the copies out over chunks of the batch
    it_pin = torch.empty(count, dtype=torch.int32, pin_memory=True)
    ns_pin = torch.from_numpy(ns.astype(np.int32)).pin_memory()
    aoff_pin = torch.from_numpy(aoff.astype(np.int64)).pin_memory()
    boff_pin = torch.from_numpy(boff.astype(np.int64)).pin_memory()
    n_max_all = int(ns.max())
    host_ws = None
    if use_mixed:
        nbytes = L.nacu_mixed_host_workspace_bytes(count, n_max_all, ns_pin.data_ptr(), aoff_pin.data_ptr(),
                                                   boff_pin.data_ptr(), nrhs, args.e2e_chunks)
        host_ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")

    def e2e_step():
        if use_mixed:  # host arrays in, host solutions out (A and B read-only)
            _lib.call("nacu_dposv_ragged_mixed_host", count, n_max_all, ns_pin.data_ptr(), aoff_pin.data_ptr(),
                      a_pin.data_ptr(), nrhs, boff_pin.data_ptr(), b_pin.data_ptr(), x_pin.data_ptr(),
                      i_pin.data_ptr(), it_pin.data_ptr(), args.e2e_chunks, host_ws.data_ptr(), host_ws.numel(),
                      0.0, 0, 0.0, 0, int(stream.cuda_stream))
        else:
            A.copy_(a_pin, non_blocking=True)
            B.copy_(b_pin, non_blocking=True)
            chol.factored = False
            chol.solve_mut(rhs)
            x_pin.copy_(B, non_blocking=True)
            i_pin.copy_(info_t, non_blocking=True)
            l_pin.copy_(logdet_t, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    t1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / e2e_steps
    h2d = (a0.numel() + b0.numel()) * 8 + (count * 20 if use_mixed else 0)
    d2h = b0.numel() * 8 + count * (8 if use_mixed else 12)

    # one plain FP64 launch per matrix (nacu_dposv), on a sample, one stream
    plain_sample = rng.choice(count, size=min(1000, count), replace=False)
    restore()
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for s in plain_sample:
        n = int(ns[s])
        _lib.call("nacu_dposv", n, A.data_ptr() + int(aoff[s]) * 8, nrhs, B.data_ptr() + int(boff[s]) * 8,
                  chol.info.data_ptr() + int(s) * 4, chol.logdet.data_ptr() + int(s) * 8, 0.0, 0, sp)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    plain_solves_per_s = plain_sample.size / (plain_ms * 1e-3)
    plain_flops = ragged_flops(ns[plain_sample], nrhs) / (plain_ms * 1e-3)

    peak = ctypes_probe(L)
    flops = ragged_flops(ns, nrhs)
    achieved = flops / (kern_ms * 1e-3)
    fp64_form = {"solves_per_s": count / (kern_ms * 1e-3), "gflops": achieved / 1e9, "ms_per_step": kern_ms,
                 "frac_of_fp64_peak": achieved / peak, **acc64}
    mixed["frac_of_fp64_peak_executed"] = mixed["fp64_flops_executed_per_launch"] / (mixed["ms_per_step"] * 1e-3) / peak
    head_ms = mixed["ms_per_step"] if use_mixed else kern_ms
    value = count * world / (head_ms * 1e-3)
    if use_mixed:
        roof_achieved = mixed["fp64_flops_executed_per_launch"] / (head_ms * 1e-3)
        roof_note = ("dominant kernel chol_mixed_kernel: FP64 residual work executed per launch / launch time; "
                     "the FP32 factor and solves run on the FMA pipe and are latency-bound")
    else:
        roof_achieved = achieved
        roof_note = "dominant kernel chol_ragged_kernel<false>: n^3/3 + 2 nrhs n^2 per system"
    acc_head = {k: (mixed if use_mixed else acc64)[k] for k in acc64}
    res = {
        "metric": "solves/s at backward err <= n*eps64 (ragged batched SPD solve, chosen forms vs plain FP64)",
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head_ms,  # the time of the form `value` reports
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded; A = B B^T + n I, B ~ N(0,1); 4 RHS ~ N(0,1))",
        "config": {"workload": "ragged_cholesky", "count": count, "n_range": [cfg["n_lo"], cfg["n_hi"]],
                   "nrhs": nrhs,
                   "form": ("batched persistent mixed precision (FP32 factor, FP64 refinement), CUDA graph"
                            if use_mixed else "batched persistent FP64, CUDA graph"),
                   "fp64_launch": ("one launch, host largest-first order, default tile" if args.single_launch else
                                   "size-bucketed persistent launches, autotuned tile per bucket"),
                   "tile_table": tiles_table, "autotuned_now": tune_res,
                   "l2": "inputs (3.4 GB) larger than L2; input restore outside the timed events",
                   "parallelism": "replicas" if world > 1 else "single"},
        "gflops": flops / (head_ms * 1e-3) / 1e9,
        **acc_head,
        "forms": {
            "batched_persistent_fp64": fp64_form,
            "plain_fp64_launch_per_matrix": {"solves_per_s": plain_solves_per_s, "gflops": plain_flops / 1e9,
                                             "sample": int(plain_sample.size)},
            "batched_mixed_fp32_factor_fp64_refined": mixed,
            "speedup_mixed_vs_fp64_batched": kern_ms / mixed["ms_per_step"],
        },
        "roofline": {"bound": "fp64", "achieved": roof_achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": roof_achieved / peak, "traffic": None, "note": roof_note,
                     "peak_source": fp64_peak_source(),
                     "algorithmic_bytes_per_launch": ragged_bytes(ns, nrhs),
                     "hbm_frac_of_measured": (ragged_bytes(ns, nrhs) / (head_ms * 1e-3)) / (read_peaks().get("hbm_gbs", 6794.8) * 1e9)},
        "e2e": {"value": count / (e2e_ms * 1e-3), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        # per step: the mixed form launches chol_mixed_kernel + chol_mixed_fallback_kernel; the FP64
        # form three sort kernels and one persistent launch per size bucket that can hold this batch
        "gpu_launches": args.steps * (2 if use_mixed else (1 if args.single_launch else 3 + active_buckets(n_max))),
        "clocks": clk.summary(),
    }
    traffic = PROFILED_TRAFFIC.get("chol_mixed_kernel" if use_mixed else "chol_ragged_kernel")
    if traffic is not None and count == RAGGED["count"]:
        res["roofline"]["traffic"] = traffic[0]
        res["roofline"]["traffic_source"] = traffic[1]
    return res, dict(ns=ns, aoff=aoff, boff=boff, a_host=a_host, b_host=b_host, nrhs=nrhs)


def bench_ragged_mixed(args, L, ns, aoff, boff, a0, b0, nrhs, stream, a_host, b_host, x_ref=None):
    """The precision form on the same inputs (A and B read-only, X out), one
    graph-replayed launch per step."""
    import torch

    from nalgebra_gb300 import DeviceBatch, Graph

    count = ns.size
    batch = DeviceBatch(a0, ns, ns, aoff)
    rhs = DeviceBatch(b0, ns, np.full(count, nrhs), boff)
    out = DeviceBatch(torch.zeros_like(b0), ns, np.full(count, nrhs), boff)
    chol = batch.cholesky()
    for _ in range(args.warmup):
        chol.solve_refined_into(rhs, out)
    torch.cuda.synchronize()
    graph = Graph()  # the mirror's own capture (nacu_graph_*), replayed on the default stream
    with graph.capture():
        chol.solve_refined_into(rhs, out)
    out.data.zero_()
    graph.replay()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(stream)
        graph.replay()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    it = chol._iters.to_numpy()[:count]
    if np.any(chol.info.to_numpy()[:count] != 0):
        raise RuntimeError("mixed form: systems reported not SPD")
    x_host = out.data.to_numpy()
    acc = batch_accuracy(ns, aoff, a_host, boff, b_host, x_host, nrhs, x_ref)
    n = ns.astype(np.float64)
    fp64_flops = float(np.sum(np.abs(it) * 2.0 * nrhs * n * n))  # FP64 residual work actually executed
    return {"solves_per_s": count / (ms * 1e-3), "ms_per_step": ms,
            "gflops_fp64_equivalent": ragged_flops(ns, nrhs) / (ms * 1e-3) / 1e9,
            "fp64_flops_executed_per_launch": fp64_flops,
            "residuals_per_system_mean": float(np.mean(np.abs(it))), "fp64_fallbacks": int(np.sum(it < 0)),
            **acc, "_objects": (chol, rhs, out)}


_FP64_PEAK = {}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# dominant kernel, from one ncu capture of a smaller case of the same workload,
# scaled to a full launch by the systems processed (traffic grows with them).
PROFILED_TRAFFIC = {
    # 1.269 GB read + 0.277 GB written for a 2000-system slice of the same size
    # distribution (profiles/chol_mixed_kernel__ragged_spd_2000.md), x 10 systems
    "chol_mixed_kernel": (15.46e9, "ncu capture of 2000 systems, scaled x10 by systems processed "
                                   "(profiles/chol_mixed_kernel__ragged_spd_2000.md)"),
}


def ctypes_probe(L):
    """FP64 roofline denominator: the best of a cuBLAS DGEMM (torch.matmul on
    float64, 8192^3, best of 2 -- the FP64 counterpart of the cuBLAS BF16 figure
    in MEASURED_PEAKS.json), this library's own DGEMM (nacu_dgemm, 8192^3, best
    of 2) and its DFMA probe, all measured in this run.  Cached per process."""
    if "value" in _FP64_PEAK:
        return _FP64_PEAK["value"]
    import ctypes

    import torch

    v = ctypes.c_double(0.0)
    rc = L.nacu_probe_fp64_peak(ctypes.byref(v))
    if rc != 0:
        raise RuntimeError("FP64 probe failed")
    n = 8192
    a = torch.randn((n, n), dtype=torch.float64, device="cuda")
    b = torch.randn((n, n), dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3))
    # the library's own DGEMM on the same operands (column-major views of a, b)
    c = torch.empty((n, n), dtype=torch.float64, device="cuda")
    sp = int(torch.cuda.current_stream().cuda_stream)
    own = 0.0
    for i in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = L.nacu_dgemm(n, n, n, ctypes.c_double(1.0), ctypes.c_void_p(a.data_ptr()), n,
                          ctypes.c_void_p(b.data_ptr()), n, ctypes.c_double(0.0), ctypes.c_void_p(c.data_ptr()), n,
                          ctypes.c_void_p(sp))
        e1.record()
        torch.cuda.synchronize()
        if rc != 0:
            raise RuntimeError("nacu_dgemm failed in the FP64 peak probe")
        if i:
            own = max(own, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3))
    del a, b, c
    _FP64_PEAK.update(value=max(best, own, v.value), cublas_dgemm=best, own_dgemm=own, dfma_probe=v.value)
    return _FP64_PEAK["value"]


def fp64_peak_source():
    return ("FP64: max of cuBLAS DGEMM 8192^3 (%.3f TFLOP/s), this library's nacu_dgemm 8192^3 (%.3f TFLOP/s) and "
            "the DFMA probe (%.3f TFLOP/s), measured in this run; MEASURED_PEAKS.json has no FP64 figure"
            % (_FP64_PEAK.get("cublas_dgemm", 0) / 1e12, _FP64_PEAK.get("own_dgemm", 0) / 1e12,
               _FP64_PEAK.get("dfma_probe", 0) / 1e12))


def cpu_baseline_ragged(data, max_seconds=20.0):
    """The oracle (C++ restatement of nalgebra's Cholesky + solve + ln_det) on
    the host cores, on a bounded sample of the same workload."""
    import oracle as O

    ns, aoff, boff, a_host, b_host, nrhs = (data[k] for k in ("ns", "aoff", "boff", "a_host", "b_host", "nrhs"))
    threads = O.max_threads()
    count = ns.size
    # sample: the first k systems (same distribution), sized to ~max_seconds
    k = min(count, 2000)
    while True:
        sl = slice(0, k)
        a_s = a_host[: int(aoff[k - 1] + ns[k - 1] ** 2)] if k < count else a_host
        b_s = b_host[: int(boff[k - 1] + ns[k - 1] * nrhs)] if k < count else b_host
        t0 = time.perf_counter()
        O.posv_ragged(ns[sl], aoff[sl], a_s, boff[sl], b_s, nrhs, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt > 2.0 or k == count:
            break
        k = min(count, int(k * max(2.0, 5.0 / max(dt, 1e-3))))
    return {"value": k / dt, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"first {k} of {count} systems of the same workload, {dt:.2f} s",
            "gflops": ragged_flops(ns[:k], nrhs) / dt / 1e9}


def bench_ragged_reference(args, rank, world):
    """--impl reference: nalgebra's CPU path (the oracle restatement, all host
    threads), same config/metric; each step a bounded sample."""
    import oracle as O
    from nalgebra_gb300 import workloads as W

    cfg = dict(RAGGED)
    k = 2000
    w = W.ragged_spd(k, cfg["n_lo"], cfg["n_hi"], cfg["nrhs"], seed=cfg["seed"])
    threads = O.max_threads()
    for _ in range(args.warmup):
        O.posv_ragged(w["ns"], w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], cfg["nrhs"], nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.posv_ragged(w["ns"], w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], cfg["nrhs"], nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    value = k / dt
    return {
        "impl": "reference",
        "metric": "solves/s at backward err <= n*eps64 (ragged batched SPD solve, chosen forms vs plain FP64)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded; A = B B^T + n I, B ~ N(0,1); 4 RHS ~ N(0,1))",
        "config": {"workload": "ragged_cholesky", "count": RAGGED["count"], "n_range": [cfg["n_lo"], cfg["n_hi"]],
                   "nrhs": cfg["nrhs"], "form": "nalgebra CPU path (C++ restatement), OpenMP across systems"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{k} systems of the same distribution per step"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ----------------------------------------------------------------------------- LU batched

def bench_lu_ours(args, rank, world):
    import torch

    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count, n = 4096, 64
    a, b = W.dense_lu(count, n, 1, seed=rank)
    a0 = torch.from_numpy(a).cuda().reshape(-1)
    b0 = torch.from_numpy(b).cuda().reshape(-1)
    A, B = a0.clone(), b0.clone()
    ipiv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0

    def launch():
        _lib.call("nacu_dgesv_batched", n, 1, A.data_ptr(), n * n, ipiv.data_ptr(), B.data_ptr(), n,
                  info.data_ptr(), count, flags, sp)

    for _ in range(args.warmup):
        A.copy_(a0); B.copy_(b0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); B.copy_(b0); flush.zero_()
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    flops = count * (2.0 / 3 * n ** 3 + 2.0 * n ** 2)
    peak = ctypes_probe(L)
    # every system against the oracle (nalgebra's LU::new + solve restated):
    # identical pivot sequences, backward error <= 10 n eps64 (residual by Dot2)
    import oracle as O

    _, piv_ref, _, _ = O.gesv_batched(a, b, n)
    piv = ipiv.cpu().numpy().reshape(count, n)
    x = B.cpu().numpy()
    ns = np.full(count, n, dtype=np.int32)
    be = O.ragged_backward_errors(ns, np.arange(count, dtype=np.int64) * n * n, a.reshape(-1),
                                  np.arange(count, dtype=np.int64) * n, b.reshape(-1), x, 1, symmetric=False)
    accuracy = {"systems_checked": count, "pivot_sequences_identical": int(np.sum(np.all(piv == piv_ref, axis=1))),
                "backward_error_max_over_batch_in_n_eps": float(np.max(be) / (n * EPS64)),
                "systems_above_10_n_eps": int(np.sum(~(be / (n * EPS64) <= 10.0))),
                "info_nonzero": int(np.sum(info.cpu().numpy() != 0))}
    return {"metric": "solves/s (batched LU factor+solve, 4096 x 64x64 f64)", "value": count / (ms * 1e-3),
            "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "lu_batched", "count": count, "n": n, "exact": bool(args.exact),
                                            "l2": "256 MB flush between steps"},
            "gflops": flops / (ms * 1e-3) / 1e9,
            "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                         "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / peak, "traffic": None,
                         "peak_source": fp64_peak_source()},
            "accuracy": accuracy, "gpu_launches": args.steps, "clocks": clk.summary()}


def bench_lu_inverse_ours(args, rank, world):
    """Batched `m.try_inverse()` for n > 4 (src/linalg/inverse.rs:135-137 ->
    lu.rs:266-297): nacu_dgetrf_batched then nacu_dgetri_batched on 4096
    64x64 f64 systems per step; work counted as nalgebra's 2/3 n^3 (factor)
    + 2 n^3 (n solves with the identity) flops per inverse."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count, n = 4096, 64
    a, _ = W.dense_lu(count, n, 1, seed=rank)
    a0 = torch.from_numpy(a).cuda().reshape(-1)
    A = a0.clone()
    inv = torch.empty(count * n * n, dtype=torch.float64, device="cuda")
    ipiv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0

    def launch():
        _lib.call("nacu_dgetrf_batched", n, A.data_ptr(), n * n, ipiv.data_ptr(), info.data_ptr(), count, flags, sp)
        _lib.call("nacu_dgetri_batched", n, A.data_ptr(), n * n, ipiv.data_ptr(), inv.data_ptr(), n * n,
                  info.data_ptr(), count, flags, sp)

    for _ in range(args.warmup):
        A.copy_(a0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); flush.zero_()
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    assert int((info != 0).sum().item()) == 0
    # accuracy on a sample: A * inv(A) - I
    worst = 0.0
    for s in range(0, count, 512):
        m = a[s].reshape(n, n).T
        x = inv[s * n * n:(s + 1) * n * n].cpu().numpy().reshape(n, n).T
        worst = max(worst, float(np.abs(m @ x - np.eye(n)).max()))
    flops = count * (2.0 / 3 * n ** 3 + 2.0 * n ** 3)
    peak = ctypes_probe(L)
    res = {"metric": "inverses/s (batched LU factor + try_inverse, 4096 x 64x64 f64)", "value": count / (ms * 1e-3),
           "unit": "inverses/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "lu_inverse", "count": count, "n": n, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "gflops": flops / (ms * 1e-3) / 1e9, "max_abs_A_Ainv_minus_I_sample": worst,
           "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source()},
           "gpu_launches": args.steps * (2 + (n + 15) // 16), "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 256
        t0 = time.perf_counter()
        for s in range(sample):
            lu_, piv, _ = O.lu(a[s].reshape(n, n).T)
            O.lu_try_inverse(lu_, piv)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "inverses/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} systems, oracle LU::new + try_inverse, one thread"}
    return res


def bench_trsv_ours(args, rank, world):
    """Batched triangular solves at the reference's solve benchmark shape
    (benches/linalg/solve.rs: 100x100, one vector): 4096 systems per step for
    solve_lower_triangular (the headline form), solve_upper_triangular and
    tr_solve_lower_triangular (nacu_dtrsv_batched).  Entries U[0, 1) as
    DMatrix::new_random, plus n on the diagonal so the solutions stay finite.
    HBM roofline: the triangle (n(n+1)/2 doubles) read, b read and written."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib

    count, n = 4096, 100
    rng = np.random.default_rng(rank)
    t = rng.random((count, n, n)) + n * np.eye(n)
    b = rng.random((count, n))
    T = torch.from_numpy(np.ascontiguousarray(np.transpose(t, (0, 2, 1))).reshape(count, n * n)).cuda()
    b0 = torch.from_numpy(b).cuda()
    B = b0.clone()
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0
    forms = {}
    for name, upper, trans in (("solve_lower_triangular", 0, 0), ("solve_upper_triangular", 1, 0),
                               ("tr_solve_lower_triangular", 0, 1)):
        def launch():
            _lib.call("nacu_dtrsv_batched", n, 1, upper, trans, 0, 0.0, T.data_ptr(), n * n, B.data_ptr(), n,
                      info.data_ptr(), count, flags, sp)
        for _ in range(args.warmup):
            B.copy_(b0); launch()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            for i in range(args.steps):
                B.copy_(b0); flush.zero_()
                ev[i][0].record(stream)
                launch()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
        ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
        x = B.cpu().numpy()
        errs = []
        for s in range(0, count, 512):
            tri = np.triu(t[s]) if upper else np.tril(t[s])
            m = tri.T if trans else tri
            errs.append(float(np.abs(m @ x[s] - b[s]).max() / np.abs(b[s]).max()))
        forms[name] = {"ms": ms, "solves_per_s": count / (ms * 1e-3), "max_rel_residual_sample": max(errs),
                       "clocks": clk.summary()}
    head = forms["solve_lower_triangular"]
    bytes_per = (n * (n + 1) / 2 + 2 * n) * 8
    flops_per = float(n * n)  # n(n-1)/2 multiply-adds and n divisions
    peaks = read_peaks()
    hbm = float(peaks.get("hbm_gbs", 6794.8)) if peaks else 6794.8
    L = _lib.load()
    fp64 = ctypes_probe(L)
    achieved = count * flops_per / (head["ms"] * 1e-3)
    res = {"metric": "solves/s (batched solve_lower_triangular, 4096 x 100x100 f64, one vector)",
           "value": head["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (U[0,1) entries, n added on the diagonal)",
           "config": {"workload": "trsv_batched", "count": count, "n": n, "nrhs": 1, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "forms": forms,
           "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64 / 1e12, "unit": "TFLOP/s",
                        "frac": achieved / fp64, "traffic": None, "peak_source": fp64_peak_source(),
                        "note": ("n^2 flops per solve; at 2 flops per 8 bytes the FP64 pipe binds before HBM "
                                 "(%.2f of the measured HBM rate)" % (count * bytes_per / (head["ms"] * 1e-3)
                                                                       / (hbm * 1e9)))},
           "gpu_launches": 3 * args.steps, "clocks": head["clocks"]}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 1000
        t0 = time.perf_counter()
        for s in range(sample):
            O.triangular_solve(t[s], b[s])
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} systems, oracle solve_lower_triangular, one thread "
                                         "(includes the ctypes call per system)"}
    return res


def bench_chol_update_ours(args, rank, world):
    """Batched Cholesky::rank_one_update (cholesky.rs:277-285, 410-449) on 4096
    factors of order 128 per step (sigma = 1), with remove_column and
    insert_column (j = 64) timed beside it.  Work: 2 n^2 flops per update (two
    multiply-adds on each of the n^2/2 entries below the diagonal); FP64
    roofline."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib

    L_ = _lib.load()
    count, n, j = 4096, 128, 64
    rng = np.random.default_rng(rank)
    b = rng.standard_normal((16, n, n))
    base = []
    for k in range(16):
        l, _ = O.cholesky(b[k] @ b[k].T + n * np.eye(n))
        base.append(np.asfortranarray(l).ravel(order="F"))
    facs = np.stack([base[k % 16] for k in range(count)])
    L0 = torch.from_numpy(facs).cuda()
    Lw = L0.clone()
    X = torch.from_numpy(rng.standard_normal((count, n))).cuda()
    S = torch.ones(count, dtype=torch.float64, device="cuda")
    # insert_column puts an n-th row and column back into the order n-1 factors
    # that remove_column writes; A's eigenvalues are >= n, so col[j] above
    # |col|^2 + n keeps the new diagonal positive.
    cols = rng.standard_normal((count, n))
    cols[:, j] = (cols * cols).sum(axis=1) + n + 1.0
    C = torch.from_numpy(cols).cuda()
    out_rm = torch.empty((count, (n - 1) ** 2), dtype=torch.float64, device="cuda")
    out_in = torch.empty((count, n * n), dtype=torch.float64, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0
    calls = {
        "rank_one_update": lambda: _lib.call("nacu_dchol_rank1_update_batched", n, Lw.data_ptr(), n * n, X.data_ptr(), n,
                                             S.data_ptr(), count, flags, sp),
        "remove_column": lambda: _lib.call("nacu_dchol_remove_column_batched", n, L0.data_ptr(), n * n, j,
                                           out_rm.data_ptr(), (n - 1) ** 2, count, flags, sp),
        "insert_column": lambda: _lib.call("nacu_dchol_insert_column_batched", n - 1, out_rm.data_ptr(), (n - 1) ** 2,
                                           j, C.data_ptr(), n, out_in.data_ptr(), n * n, info.data_ptr(),
                                           count, flags, sp),
    }
    calls["remove_column"]()  # the inputs of insert_column
    torch.cuda.synchronize()
    forms = {}
    for name, fn in calls.items():
        for _ in range(args.warmup):
            Lw.copy_(L0); fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            for i in range(args.steps):
                Lw.copy_(L0); flush.zero_()
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
        ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
        forms[name] = {"ms": ms, "updates_per_s": count / (ms * 1e-3), "clocks": clk.summary()}
    # accuracy on a sample of the rank-one updates
    Lw.copy_(L0); calls["rank_one_update"](); torch.cuda.synchronize()
    g = Lw.cpu().numpy()
    worst = 0.0
    for s in range(0, count, 1024):
        lo = np.tril(g[s].reshape(n, n).T)
        x = X[s].cpu().numpy()
        a = base[s % 16].reshape(n, n).T
        a = np.tril(a) @ np.tril(a).T + np.outer(x, x)
        worst = max(worst, float(np.abs(lo @ lo.T - a).max() / np.abs(a).max()))
    head = forms["rank_one_update"]
    flops = count * 4.0 * n * n / 2
    peak = ctypes_probe(L_)
    res = {"metric": "updates/s (batched Cholesky::rank_one_update, 4096 factors of order 128, f64)",
           "value": head["updates_per_s"], "unit": "updates/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (factors of B B^T + n I, x ~ N(0,1), sigma = 1)",
           "config": {"workload": "chol_update", "count": count, "n": n, "j": j, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "forms": forms, "max_rel_error_sample": worst,
           "roofline": {"bound": "fp64", "achieved": flops / (head["ms"] * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (head["ms"] * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source(),
                        "note": "2 n^2 flops per update (two multiply-adds per entry below the diagonal, three FP64 "
                                "instructions); the per-column scalar chain (a square root and a reciprocal after the "
                                "diagonal's reciprocals are formed in bulk) runs in one lane of each 8-lane group and "
                                "costs a full warp instruction per step"},
           "gpu_launches": 3 * args.steps, "clocks": head["clocks"]}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 200
        t0 = time.perf_counter()
        for s in range(sample):
            O.cholesky_rank_one_update(facs[s].reshape(n, n).T, X[s].cpu().numpy(), 1.0)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "updates/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} factors, oracle rank_one_update, one thread"}
    return res


def bench_full_piv_lu_ours(args, rank, world):
    """Batched FullPivLU::new + solve (src/linalg/full_piv_lu.rs:56-91,
    185-211) on the plain-LU workload: 4096 dense 64x64 systems, one RHS
    (nacu_dfullpivlu_batched).  Work: 2/3 n^3 + 2 n^2 flops per system, as
    the partial-pivot LU (the full pivot search compares integer images of |a|
    and costs no flops); FP64 roofline."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count, n = 4096, 64
    a, b = W.dense_lu(count, n, 1, seed=rank)
    a0 = torch.from_numpy(a).cuda().reshape(-1)
    b0 = torch.from_numpy(b).cuda().reshape(-1)
    A, B = a0.clone(), b0.clone()
    ipiv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    jpiv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0

    def launch():
        _lib.call("nacu_dfullpivlu_batched", n, 1, A.data_ptr(), n * n, ipiv.data_ptr(), jpiv.data_ptr(),
                  B.data_ptr(), n, info.data_ptr(), count, flags, sp)

    for _ in range(args.warmup):
        A.copy_(a0); B.copy_(b0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); B.copy_(b0); flush.zero_()
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    x = B.cpu().numpy().reshape(count, n)
    am = a.reshape(count, n, n)
    bm = b.reshape(count, n)
    berr = 0.0
    for s in range(0, count, 256):
        m = am[s].T  # column-major storage
        berr = max(berr, float(np.abs(m @ x[s] - bm[s]).max() / (np.abs(m).max() * np.abs(x[s]).max() * n)))
    flops = count * (2.0 / 3 * n ** 3 + 2.0 * n ** 2)
    peak = ctypes_probe(L)
    res = {"metric": "solves/s (batched FullPivLU factor+solve, 4096 x 64x64 f64)", "value": count / (ms * 1e-3),
           "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (the plain-LU workload: N(0,1) entries plus 64 on the diagonal)",
           "config": {"workload": "full_piv_lu", "count": count, "n": n, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "gflops": flops / (ms * 1e-3) / 1e9, "backward_error_sample_in_eps": berr / np.finfo(float).eps,
           "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source()},
           "gpu_launches": args.steps, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 400
        t0 = time.perf_counter()
        for s in range(sample):
            lu, ip, jp, _ = O.full_piv_lu(am[s].T)
            O.full_piv_lu_solve(lu, ip, jp, bm[s])
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} systems, oracle FullPivLU new + solve, one thread"}
    return res


def bench_col_piv_qr_ours(args, rank, world):
    """Batched ColPivQR::new + solve (src/linalg/col_piv_qr.rs:59-92,
    227-247) on the plain-LU workload: 4096 dense 64x64 systems, one RHS
    (nacu_dcolpivqr_batched).  Work: 4/3 n^3 (Householder QR of a square
    matrix) + 3 n^2 (Q^T b and the upper solve) flops per system; FP64
    roofline."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count, n = 4096, 64
    a, b = W.dense_lu(count, n, 1, seed=rank)
    a0 = torch.from_numpy(a).cuda().reshape(-1)
    b0 = torch.from_numpy(b).cuda().reshape(-1)
    A, B = a0.clone(), b0.clone()
    diag = torch.zeros(count * n, dtype=torch.float64, device="cuda")
    jpiv = torch.zeros(count * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0

    def launch():
        _lib.call("nacu_dcolpivqr_batched", n, 1, A.data_ptr(), n * n, diag.data_ptr(), jpiv.data_ptr(),
                  B.data_ptr(), n, info.data_ptr(), count, flags, sp)

    for _ in range(args.warmup):
        A.copy_(a0); B.copy_(b0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); B.copy_(b0); flush.zero_()
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    x = B.cpu().numpy().reshape(count, n)
    am = a.reshape(count, n, n)
    bm = b.reshape(count, n)
    berr = 0.0
    for s in range(0, count, 256):
        m = am[s].T  # column-major storage
        berr = max(berr, float(np.abs(m @ x[s] - bm[s]).max() / (np.abs(m).max() * np.abs(x[s]).max() * n)))
    flops = count * (4.0 / 3 * n ** 3 + 3.0 * n ** 2)
    peak = ctypes_probe(L)
    res = {"metric": "solves/s (batched ColPivQR factor+solve, 4096 x 64x64 f64)", "value": count / (ms * 1e-3),
           "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (the plain-LU workload: N(0,1) entries plus 64 on the diagonal)",
           "config": {"workload": "col_piv_qr", "count": count, "n": n, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "gflops": flops / (ms * 1e-3) / 1e9, "backward_error_sample_in_eps": berr / np.finfo(float).eps,
           "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source()},
           "gpu_launches": args.steps, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 400
        t0 = time.perf_counter()
        for s in range(sample):
            qr, d, jp = O.col_piv_qr(am[s].T)
            O.col_piv_qr_solve(qr, d, jp, bm[s])
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} systems, oracle ColPivQR new + solve, one thread"}
    return res


def bench_trsv_large_ours(args, rank, world):
    """Triangular solves of one large matrix (nacu_dtrsv) at the reference's
    solve benchmark shape (benches/linalg/solve.rs: 1000x1000, one vector;
    entries U[0, 1) as DMatrix::new_random, plus n on the diagonal so the
    solutions stay finite) for the four variants, and solve_lower_triangular at
    n = 8192 (a 256 MiB triangle, larger than L2).  One solve per launch; the
    1000x1000 triangle (4 MB) stays in L2 between launches, as the reference's
    CPU bench keeps it in cache.  HBM roofline at n = 8192: the triangle read
    once, b read and x written."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib

    L = _lib.load()
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    rng = np.random.default_rng(rank)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    out, cpu = {}, {}
    for n in (1000, 8192):
        t = rng.random((n, n)) + n * np.eye(n)
        b = rng.random(n)
        T = torch.from_numpy(np.asfortranarray(t).ravel(order="F")).cuda()
        b0 = torch.from_numpy(b).cuda()
        B = b0.clone()
        ws = torch.empty(L.nacu_trsv_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        variants = (("solve_lower_triangular", 0, 0), ("solve_upper_triangular", 1, 0),
                    ("tr_solve_lower_triangular", 0, 1), ("tr_solve_upper_triangular", 1, 1))
        if n > 1000:
            variants = variants[:1]
        reps = 20 if n <= 1000 else 4
        for name, upper, trans in variants:
            def launch():
                _lib.call("nacu_dtrsv", n, 1, upper, trans, 0, 0.0, T.data_ptr(), n, B.data_ptr(), n,
                          info.data_ptr(), ws.data_ptr(), ws.numel(), 0, sp)
            for _ in range(args.warmup):
                B.copy_(b0); launch()
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
            with ClockSampler(torch.cuda.current_device()) as clk:
                for i in range(args.steps):
                    ev[i][0].record(stream)
                    for _ in range(reps):
                        launch()  # re-solving in place: same work, same data movement
                    ev[i][1].record(stream)
                torch.cuda.synchronize()
            ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev])) / reps
            B.copy_(b0); launch(); torch.cuda.synchronize()
            x = B.cpu().numpy()
            tri = np.triu(t) if upper else np.tril(t)
            m = tri.T if trans else tri
            rel = float(np.abs(m @ x - b).max() / np.abs(b).max())
            key = f"{name}_{n}"
            out[key] = {"ms": ms, "solves_per_s": 1e3 / ms, "rel_residual": rel, "info": int(info.item()),
                        "clocks": clk.summary()}
            if rank == 0 and not args.no_cpu_baseline and name == "solve_lower_triangular":
                k = 5 if n <= 1000 else 1
                t0 = time.perf_counter()
                for _ in range(k):
                    O.triangular_solve(tri, b)
                cpu[key] = (time.perf_counter() - t0) / k * 1e3
        del T
        torch.cuda.empty_cache()
    head = out["solve_lower_triangular_1000"]
    big = out["solve_lower_triangular_8192"]
    n = 8192
    bytes_big = (n * (n + 1) / 2 + 2 * n) * 8
    peaks = read_peaks()
    hbm = float(peaks.get("hbm_gbs", 6794.8)) if peaks else 6794.8
    achieved = bytes_big / (big["ms"] * 1e-3) / 1e9
    res = {"metric": "solves/s (solve_lower_triangular, one 1000x1000 f64 matrix, one vector)",
           "value": head["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (U[0,1) entries, n added on the diagonal)",
           "config": {"workload": "trsv_large", "n": [1000, 8192], "nrhs": 1,
                      "l2": "1000x1000 L2-resident (4 MB), 8192x8192 triangle 256 MiB > L2"},
           "forms": out,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "traffic": None, "workload": "solve_lower_triangular at n = 8192",
                        "note": "the 64-row blocks form a dependency chain; n(n+1)/2 doubles + 2n per solve"},
           "gpu_launches": args.steps * 20, "clocks": head["clocks"]}
    if cpu:
        res["cpu_baseline"] = {"value": 1e3 / cpu["solve_lower_triangular_1000"], "unit": "solves/s", "cores": 1,
                               "kind": "port", "ms_at_8192": cpu.get("solve_lower_triangular_8192"),
                               "sample": "oracle solve_lower_triangular (nalgebra's column axpy loop), one thread, "
                                         "5 solves at n = 1000, 1 at n = 8192"}
    return res


def bench_qr_square_ours(args, rank, world):
    """Batched square QR::new + QR::solve (src/linalg/qr.rs:55-76, 204-256) at
    the reference's QR solve benchmark shape (benches/linalg/qr.rs: 100x100,
    one vector; entries U[0, 1) as DMatrix::new_random): 4096 systems per step
    (nacu_dqr_batched, the solve fused).  Work: 4/3 n^3 + 3 n^2 flops per
    system; FP64 roofline."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib

    L = _lib.load()
    count, n = 4096, 100
    rng = np.random.default_rng(rank)
    a = rng.random((count, n, n))
    b = rng.random((count, n))
    a0 = torch.from_numpy(np.ascontiguousarray(np.transpose(a, (0, 2, 1))).reshape(count, n * n)).cuda()
    b0 = torch.from_numpy(b).cuda()
    A, B = a0.clone(), b0.clone()
    diag = torch.zeros(count * n, dtype=torch.float64, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flags = 1 if args.exact else 0

    def launch():
        _lib.call("nacu_dqr_batched", n, 1, A.data_ptr(), n * n, diag.data_ptr(), B.data_ptr(), n, info.data_ptr(),
                  count, flags, sp)

    for _ in range(args.warmup):
        A.copy_(a0); B.copy_(b0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); B.copy_(b0); flush.zero_()
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    x = B.cpu().numpy()
    berr = 0.0
    for s in range(0, count, 256):
        berr = max(berr, float(np.abs(a[s] @ x[s] - b[s]).max() / (np.abs(a[s]).max() * np.abs(x[s]).max() * n)))
    flops = count * (4.0 / 3 * n ** 3 + 3.0 * n ** 2)
    peak = ctypes_probe(L)
    res = {"metric": "solves/s (batched QR factor+solve, 4096 x 100x100 f64)", "value": count / (ms * 1e-3),
           "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (U[0,1) entries, as DMatrix::new_random)",
           "config": {"workload": "qr_square", "count": count, "n": n, "exact": bool(args.exact),
                      "l2": "256 MB flush between steps"},
           "gflops": flops / (ms * 1e-3) / 1e9, "backward_error_sample_in_eps": berr / np.finfo(float).eps,
           "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source()},
           "gpu_launches": args.steps, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        sample = 200
        t0 = time.perf_counter()
        for s in range(sample):
            qr, d = O.qr(a[s])
            O.qr_solve(qr, d, b[s])
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"{sample} of the {count} systems, oracle QR::new + QR::solve, one thread"}
    return res


def bench_qr_large_ours(args, rank, world):
    """QR::new + QR::solve of one large matrix (nacu_dqr, then nacu_dqr_solve:
    src/linalg/qr.rs:55-76, 204-256): n = 4096 square, one vector, entries
    U[0, 1) as DMatrix::new_random plus n on the diagonal; also n = 1000 and
    the reference's wide qr_decompose_100x500 shape (factor only).  The
    factorization is in place: each step restores A from a pristine device
    copy outside the timed events (the 134 MB matrix is about the size of L2).
    Work: 4/3 n^3 flops for the factor, 5 n^2 for Q^T b and the upper solve;
    FP64 roofline."""
    import time

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib

    L = _lib.load()
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    rng = np.random.default_rng(rank)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    forms, cpu = {}, {}
    if args.profile:  # one untimed factor + solve of the 4096 case, for profiler captures
        n = 4096
        a = rng.random((n, n)) + n * np.eye(n)
        A = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
        B = torch.from_numpy(rng.random(n)).cuda()
        diag = torch.zeros(n, dtype=torch.float64, device="cuda")
        ws = torch.empty(L.nacu_qr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        _lib.call("nacu_dqr", n, n, A.data_ptr(), n, diag.data_ptr(), 0, sp)
        _lib.call("nacu_dqr_solve", n, n, 1, A.data_ptr(), n, diag.data_ptr(), B.data_ptr(), n, info.data_ptr(),
                  ws.data_ptr(), ws.numel(), 0, sp)
        torch.cuda.synchronize()
        return {"workload": "qr_large", "profile": True, "n": n, "info": int(info.item())}
    for (m, n, solve) in ((4096, 4096, True), (1000, 1000, True), (100, 500, False)):
        a = rng.random((m, n)) + (n * np.eye(m, n) if m == n else 0.0)
        b = rng.random(m)
        a0 = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
        b0 = torch.from_numpy(b).cuda()
        A, B = a0.clone(), b0.clone()
        diag = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
        ws = torch.empty(max(L.nacu_qr_solve_workspace_bytes(n), 1), dtype=torch.uint8, device="cuda")

        def launch():
            _lib.call("nacu_dqr", m, n, A.data_ptr(), m, diag.data_ptr(), 0, sp)
            if solve:
                _lib.call("nacu_dqr_solve", m, n, 1, A.data_ptr(), m, diag.data_ptr(), B.data_ptr(), m,
                          info.data_ptr(), ws.data_ptr(), ws.numel(), 0, sp)

        steps = args.steps if n >= 4096 else max(args.steps, 10)
        for _ in range(args.warmup):
            A.copy_(a0); B.copy_(b0); launch()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            for i in range(steps):
                A.copy_(a0); B.copy_(b0)
                ev[i][0].record(stream)
                launch()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
        ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
        key = f"{m}x{n}" + ("_factor_solve" if solve else "_factor")
        f = {"ms": ms, "per_s": 1e3 / ms, "clocks": clk.summary(), "launches_per_step": min(m, n) + 1 + (4 if solve else 0)}
        if solve:
            x = B.cpu().numpy()[:n]
            f["backward_error_in_eps"] = float(np.abs(a @ x - b).max() / (np.abs(a).max() * np.abs(x).max() * n)
                                               / np.finfo(float).eps)
            f["info"] = int(info.item())
        forms[key] = f
        if rank == 0 and not args.no_cpu_baseline and n <= 1000:
            t0 = time.perf_counter()
            qr, d = O.qr(a)
            if solve:
                O.qr_solve(qr, d, b)
            cpu[key] = (time.perf_counter() - t0) * 1e3
        del A, a0, ws
        torch.cuda.empty_cache()
    head = forms["4096x4096_factor_solve"]
    n = 4096
    flops = 4.0 / 3 * n ** 3 + 5.0 * n ** 2
    peak = ctypes_probe(L)
    res = {"metric": "solves/s (QR::new + QR::solve, one 4096x4096 f64 matrix, one vector)",
           "value": 1e3 / head["ms"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (U[0,1) entries, n added on the diagonal)",
           "config": {"workload": "qr_large", "shapes": ["4096x4096", "1000x1000", "100x500"], "nrhs": 1,
                      "l2": "A restored from a pristine copy before each step (134 MB at n = 4096)"},
           "forms": forms,
           "roofline": {"bound": "fp64", "achieved": flops / (head["ms"] * 1e-3) / 1e12, "peak": peak / 1e12,
                        "unit": "TFLOP/s", "frac": flops / (head["ms"] * 1e-3) / peak, "traffic": None,
                        "peak_source": fp64_peak_source(),
                        "note": "one launch per Householder step; 4/3 n^3 + 5 n^2 flops per solve"},
           "gpu_launches": args.steps * head["launches_per_step"], "clocks": head["clocks"]}
    if cpu:
        res["cpu_baseline"] = {"value": 1e3 / cpu["1000x1000_factor_solve"], "unit": "solves/s at n = 1000",
                               "cores": 1, "kind": "port", "ms": cpu,
                               "sample": "oracle QR::new + QR::solve at 1000x1000, and QR::new at 100x500, "
                                         "one thread, one run each"}
    return res


# ----------------------------------------------------------------------------- QR least squares

def bench_ls_ours(args, rank, world):
    import torch

    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count = args.count or 8192
    n = 64
    w = W.ragged_ls(count, 128, 512, n, seed=rank)
    ms = w["ms"]
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    a0, b0 = d(w["a_flat"]), d(w["b_flat"])
    A, B = a0.clone(), b0.clone()
    dms, daoff, dboff = d(ms), d(w["a_offsets"]), d(w["b_offsets"])
    X = torch.zeros(count * n, dtype=torch.float64, device="cuda")
    diag = torch.zeros(count * n, dtype=torch.float64, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    ws = torch.zeros(L.nacu_qr_workspace_bytes(count), dtype=torch.uint8, device="cuda")
    order = d(np.argsort(-ms, kind="stable").astype(np.int32))
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)

    def launch():
        _lib.call("nacu_dgels_batched", count, n, int(ms.max()), dms.data_ptr(), daoff.data_ptr(), A.data_ptr(),
                  dboff.data_ptr(), B.data_ptr(), X.data_ptr(), diag.data_ptr(), info.data_ptr(),
                  order.data_ptr(), ws.data_ptr(), ws.numel(), 0, sp)

    for _ in range(args.warmup):
        A.copy_(a0); B.copy_(b0); launch()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for i in range(args.steps):
            A.copy_(a0); B.copy_(b0)
            ev[i][0].record(stream)
            launch()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    ms_step = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
    m = ms.astype(np.float64)
    flops = float(np.sum(2 * m * n * n - 2.0 * n ** 3 / 3 + 4 * m * n + n * n))
    peak = ctypes_probe(L)
    if np.any(info.cpu().numpy() != 0):
        raise RuntimeError("rank-deficient problems in the LS workload")
    # every problem against the oracle (QR::new + q_tr_mul + the top-n solve):
    # the relative difference of the solutions, and the normal-equations
    # residual ||A^T (A x - b)|| / (||A||^2 ||x||) of the reference's LS test
    import oracle as O

    _, _, x_ref, _ = O.gels_batched(ms, n, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"])
    xg = X.cpu().numpy().reshape(count, n)
    rel = np.max(np.abs(xg - x_ref), axis=1) / np.max(np.abs(x_ref), axis=1)
    ne = 0.0
    for s_ in range(0, count, 64):  # normal equations on every 64th problem
        m_ = int(ms[s_])
        am = w["a_flat"][w["a_offsets"][s_]:w["a_offsets"][s_] + m_ * n].reshape(n, m_).T
        bm = w["b_flat"][w["b_offsets"][s_]:w["b_offsets"][s_] + m_]
        ne = max(ne, float(np.abs(am.T @ (am @ xg[s_] - bm)).max() / (np.abs(am).sum(axis=0).max() ** 2 *
                                                                      np.abs(xg[s_]).max())))
    accuracy = {"problems_checked": count, "solution_rel_diff_vs_oracle_max": float(np.max(rel)),
                "normal_equations_residual_max_every_64th": ne}
    return {"metric": "solves/s (batched Householder QR least squares, 8192 x m in [128,512] x 64 f64)",
            "value": count / (ms_step * 1e-3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ls_qr", "count": count, "m_range": [128, 512], "n": n},
            "gflops": flops / (ms_step * 1e-3) / 1e9,
            "roofline": {"bound": "fp64", "achieved": flops / (ms_step * 1e-3) / 1e12, "peak": peak / 1e12,
                         "unit": "TFLOP/s", "frac": flops / (ms_step * 1e-3) / peak, "traffic": None,
                         "peak_source": fp64_peak_source()},
            "accuracy": accuracy, "gpu_launches": args.steps, "clocks": clk.summary()}


# ----------------------------------------------------------------------------- adjoint

def bench_adjoint_ours(args, rank, world):
    """2048 SPD systems of order 128 (f64 and f32): forward (factor + solve +
    logdet) and backward (db, dA) of l = sum w^T x + logdet A, store vs
    recompute."""
    import torch

    from nalgebra_gb300 import _lib
    from nalgebra_gb300 import workloads as W

    L = _lib.load()
    count, n = args.count or 2048, 128
    out = {}
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    for dtype, pre, tdt in ((np.float64, "d", torch.float64), (np.float32, "s", torch.float32)):
        a, b, w = W.spd_uniform(count, n, seed=rank, dtype=dtype)
        d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
        A, B, Wt = d(a), d(b), d(w)
        X = torch.zeros((count, n), dtype=tdt, device="cuda")
        Lf = torch.zeros_like(A)
        logdet = torch.zeros(count, dtype=tdt, device="cuda")
        info = torch.zeros(count, dtype=torch.int32, device="cuda")
        dA = torch.zeros_like(A)
        db = torch.zeros_like(X)
        res = {}
        for mode in ("store", "recompute"):
            rec = mode == "recompute"

            def fwd():
                _lib.call(f"nacu_{pre}posv_logdet_forward", n, A.data_ptr(), n * n, B.data_ptr(), X.data_ptr(),
                          0 if rec else Lf.data_ptr(), logdet.data_ptr(), info.data_ptr(), count, sp)

            def bwd():
                _lib.call(f"nacu_{pre}posv_logdet_backward", n, (A if rec else Lf).data_ptr(), n * n, 1 if rec else 0,
                          X.data_ptr(), Wt.data_ptr(), None, dA.data_ptr(), db.data_ptr(), info.data_ptr(), count, sp)

            for _ in range(args.warmup):
                fwd(); bwd()
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
            for _ in range(args.steps):
                fwd()
            e[1].record(stream)
            for _ in range(args.steps):
                bwd()
            e[2].record(stream)
            torch.cuda.synchronize()
            fms, bms = e[0].elapsed_time(e[1]) / args.steps, e[1].elapsed_time(e[2]) / args.steps
            res[mode] = {"forward_ms": fms, "backward_ms": bms,
                         "systems_per_s_fwd_bwd": count / ((fms + bms) * 1e-3),
                         "stored_intermediate_bytes": 0 if rec else int(count * n * n * np.dtype(dtype).itemsize)}
        out[pre + "_" + np.dtype(dtype).name] = res
    # FP64 work per system (store form): forward n^3/3 + 2n^2 (factor, solve, log-det); backward the
    # triangular inverse n^3/3, A^-1 = L^-T L^-1 n^3/3, v = A^-1 w 2n^2 and the gradient 4n^2
    peak = ctypes_probe(L)
    st = out["d_float64"]["store"]
    flops_sys = n ** 3 + 8.0 * n * n
    achieved = count * flops_sys / ((st["forward_ms"] + st["backward_ms"]) * 1e-3)
    return {"metric": "adjoint of batched Cholesky solve + logdet (2048 x 128, f64 and f32)",
            "value": out["d_float64"]["store"]["systems_per_s_fwd_bwd"], "unit": "systems/s (forward+backward, f64)",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "adjoint", "count": count, "n": n}, "forms": out,
            "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": fp64_peak_source(),
                         "note": "FP64 store form, forward + backward: n^3 + 8 n^2 flops per system"},
            "gpu_launches": 2 * args.steps}


# ----------------------------------------------------------------------------- GEMM

def bench_gemm_ours(args, rank, world):
    """Matrix::gemm on m = n = k (default 8192) f64, A = N(0,1) 2^k per row,
    B = N(0,1) 2^k per column, k uniform in [-20, 20]: native FP64 (nacu_dgemm)
    vs BF16-split / FP32-accumulate tensor-core form (nacu_dgemm_split_bf16);
    error of both against a compensated FP64 oracle on sampled entries."""
    import ctypes

    import torch

    from nalgebra_gb300 import _lib

    L = _lib.load()
    n = args.count or 8192
    g = torch.Generator(device="cuda")
    g.manual_seed(1234 + rank)
    A = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=g)
    # column-major: A[i, k] stored at k*n + i -> use the transposed views as storage
    rs = torch.pow(2.0, torch.randint(-20, 21, (n,), device="cuda", generator=g).double())
    cs = torch.pow(2.0, torch.randint(-20, 21, (n,), device="cuda", generator=g).double())
    Acm = (A * rs[:, None]).t().contiguous()  # memory = column-major A
    Bcm = (B * cs[None, :]).t().contiguous()  # memory = column-major B
    C64 = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    C16 = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    wsb = L.nacu_gemm_split_workspace_bytes(n, n, n)
    ws = torch.empty(wsb + 1024, dtype=torch.uint8, device="cuda")
    wp = (ws.data_ptr() + 1023) // 1024 * 1024
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)

    def fp64():
        _lib.call("nacu_dgemm", n, n, n, 1.0, Acm.data_ptr(), n, Bcm.data_ptr(), n, 0.0, C64.data_ptr(), n, sp)

    def split():
        _lib.call("nacu_dgemm_split_bf16", n, n, n, 1.0, Acm.data_ptr(), n, Bcm.data_ptr(), n, 0.0, C16.data_ptr(), n,
                  3, wp, wsb, sp)

    res = {}
    for name, fn, steps in (("split_bf16x3", split, args.steps), ("fp64", fp64, max(1, min(args.steps, 2)))):
        for _ in range(max(1, min(args.warmup, 2) if name == "fp64" else args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(torch.cuda.current_device()) as clk:
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res[name] = {"ms": ms, "tflops_fp64_equivalent": 2.0 * n ** 3 / (ms * 1e-3) / 1e12, "clocks": clk.summary()}
    flag = ctypes.c_int(0)
    L.nacu_split_gemm_error(ctypes.byref(flag))
    # error on sampled entries against the compensated oracle (64 x 64 sample)
    import oracle as O
    rng = np.random.default_rng(5)
    ri = np.sort(rng.choice(n, 64, replace=False))
    ci = np.sort(rng.choice(n, 64, replace=False))
    a_rows = Acm.view(n, n).t()[ri, :].cpu().numpy()      # rows of A
    b_cols = Bcm.view(n, n).t()[:, ci].cpu().numpy()      # columns of B
    ref = O.gemm_dot2(1.0, a_rows, b_cols)
    scale = np.abs(a_rows) @ np.abs(b_cols)
    got64 = C64.view(n, n).t()[ri][:, ci].cpu().numpy()
    got16 = C16.view(n, n).t()[ri][:, ci].cpu().numpy()
    res["fp64"]["max_err_rel_to_absAabsB"] = float(np.max(np.abs(got64 - ref) / scale))
    res["split_bf16x3"]["max_err_rel_to_absAabsB"] = float(np.max(np.abs(got16 - ref) / scale))
    res["split_bf16x3"]["pipeline_error_flag"] = flag.value
    peaks = read_peaks()
    bf16_peak = peaks.get("bf16_tflops", 1917.6)
    split_tensor_tflops = 6 * 2.0 * n ** 3 / (res["split_bf16x3"]["ms"] * 1e-3) / 1e12
    return {"metric": "GEMM f64 8192^3 (N(0,1) 2^k scaled rows/columns): split BF16 x3 tensor-core vs native FP64",
            "value": res["split_bf16x3"]["tflops_fp64_equivalent"], "unit": "TFLOP/s (FP64-equivalent)",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 -> f32 accumulate -> f64", "data": "synthetic",
            "config": {"workload": "gemm", "m": n, "n": n, "k": n, "slices": 3},
            "forms": res,
            "roofline": {"bound": "tensor", "achieved": split_tensor_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": split_tensor_tflops / bf16_peak, "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)",
                         "note": "achieved = 6 BF16 slice products x 2 n^3 / time (includes the split pre-pass)"},
            "gpu_launches": args.steps * 5}


# ----------------------------------------------------------------------------- batched Mul

def bench_mul_batched_ours(args, rank, world):
    """Many `&a * &b` products of the reference's mat100_mul_mat100 shape
    (benches/core/matrix.rs:211-224): 4096 products of 100 x 100 f64 matrices
    (entries N(0,1)) in one nacu_dgemm_batched launch, the FMA form and the
    EXACT form (nalgebra's gemv order).  Inputs (3 x 328 MB) exceed L2."""
    import torch

    from nalgebra_gb300 import _lib

    L = _lib.load()
    count = args.count or 4096
    m = n = k = 100
    g = torch.Generator(device="cuda")
    g.manual_seed(100 + rank)
    A = torch.randn((count, k, m), dtype=torch.float64, device="cuda", generator=g)  # column-major images
    B = torch.randn((count, n, k), dtype=torch.float64, device="cuda", generator=g)
    C = torch.empty((count, n, m), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    flops = 2.0 * m * n * k * count
    peak = ctypes_probe(L)
    res = {}
    for name, flags in (("fma", 0), ("exact", 1)):
        def launch():
            _lib.call("nacu_dgemm_batched", m, n, k, 1.0, A.data_ptr(), m, m * k, B.data_ptr(), k, k * n, 0.0,
                      C.data_ptr(), m, m * n, count, flags, sp)

        for _ in range(args.warmup):
            launch()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            for i in range(args.steps):
                ev[i][0].record(stream)
                launch()
                ev[i][1].record(stream)
            torch.cuda.synchronize()
        ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))
        res[name] = {"ms": ms, "products_per_s": count / (ms * 1e-3), "gflops": flops / (ms * 1e-3) / 1e9,
                     "frac_of_fp64_peak": flops / (ms * 1e-3) / peak, "clocks": clk.summary()}
    # accuracy on a sample: EXACT against the oracle's gemv order (bit for bit),
    # the FMA form against the compensated oracle
    import oracle as O

    sample = np.arange(0, count, max(1, count // 16))
    a_s = np.transpose(A[sample].cpu().numpy(), (0, 2, 1))
    b_s = np.transpose(B[sample].cpu().numpy(), (0, 2, 1))
    exact_c = np.transpose(C[sample].cpu().numpy(), (0, 2, 1))  # the last launch was the EXACT form
    identical = bool(np.array_equal(exact_c, O.gemm_gemv_order(1.0, a_s, b_s)))
    _lib.call("nacu_dgemm_batched", m, n, k, 1.0, A.data_ptr(), m, m * k, B.data_ptr(), k, k * n, 0.0, C.data_ptr(), m,
              m * n, count, 0, sp)
    fma_c = np.transpose(C[sample].cpu().numpy(), (0, 2, 1))
    err = max(float(np.max(np.abs(fma_c[i] - O.gemm_dot2(1.0, a_s[i], b_s[i])) / (np.abs(a_s[i]) @ np.abs(b_s[i]))))
              for i in range(len(sample)))
    # CPU: nalgebra's gemv-order product restated (the oracle), all host threads, a bounded sample
    threads = O.max_threads()
    ks = count
    a_h = np.transpose(A[:ks].cpu().numpy(), (0, 2, 1))
    b_h = np.transpose(B[:ks].cpu().numpy(), (0, 2, 1))
    t0 = time.perf_counter()
    O.gemm_gemv_order(1.0, a_h, b_h, nthreads=threads)
    dt = time.perf_counter() - t0
    fr = res["fma"]
    return {"metric": "products/s (batched Mul, 4096 x (100x100 * 100x100) f64)", "value": fr["products_per_s"],
            "unit": "products/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": fr["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mul_batched", "count": count, "m": m, "n": n, "k": k,
                       "shape": "benches/core/matrix.rs mat100_mul_mat100", "l2": "inputs 983 MB, larger than L2"},
            "gflops": fr["gflops"], "forms": res,
            "roofline": {"bound": "fp64", "achieved": fr["gflops"] / 1e3, "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": fr["frac_of_fp64_peak"], "traffic": None, "peak_source": fp64_peak_source(),
                         "note": "2 m n k flops per product"},
            "accuracy": {"exact_bit_identical_to_gemv_order_sample": identical, "sample": int(len(sample)),
                         "fma_max_err_rel_to_absAabsB": err},
            "cpu_baseline": {"value": ks / dt, "unit": "products/s", "cores": threads, "kind": "port",
                             "sample": f"{ks} products, nalgebra's gemv-order product (the oracle), {dt:.2f} s"},
            "gpu_launches": 2 * args.steps, "clocks": fr["clocks"]}


# ----------------------------------------------------------------------------- mixed LU + refinement

def bench_mixed_lu_ours(args, rank, world):
    """One dense f64 system at n = 4096 and 8192 (or --count n), A = U diag(s) V^T
    with cond 1e2, 1e5, 1e8, one RHS: plain FP64 blocked LU + solve
    (nacu_dgetrf + nacu_dgetrs) vs the mixed form (nacu_dgesv_mixed_ir: FP32 LU
    with BF16-split tensor-core trailing updates, FP64 refinement to backward
    error <= n eps64, FP64 fallback).  Work is counted as the FP64-equivalent
    2/3 n^3 + 2 n^2 per solve."""
    import ctypes

    import torch

    import oracle as O
    from nalgebra_gb300 import _lib, workloads

    L = _lib.load()
    sizes = [args.count] if args.count else [4096, 8192]
    conds = [1e2, 1e5, 1e8]
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    forms = {}
    headline = None
    for n in sizes:
        wsm = torch.empty(L.nacu_gesv_mixed_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        wsf = torch.empty(L.nacu_getrf_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        work = torch.empty(n * n, dtype=torch.float64, device="cuda")
        x = torch.empty(n, dtype=torch.float64, device="cuda")
        ipiv = torch.empty(n, dtype=torch.int32, device="cuda")
        info = torch.empty(4, dtype=torch.int32, device="cuda")
        flops = 2.0 / 3.0 * n ** 3 + 2.0 * n ** 2
        for cond in conds:
            A, b = workloads.conditioned_torch(n, cond, seed=int(np.log10(cond)) + n)
            a_host = b_host = None
            it, berr, fb = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)

            def mixed():
                _lib.call("nacu_dgesv_mixed_ir", n, A.data_ptr(), n, b.data_ptr(), x.data_ptr(), 1.0, 30,
                          ctypes.byref(it), ctypes.byref(berr), ctypes.byref(fb), wsm.data_ptr(), wsm.numel(), sp)

            def plain():
                _lib.call("nacu_dgetrf", n, work.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(), wsf.data_ptr(),
                          wsf.numel(), sp)
                x.copy_(b)
                _lib.call("nacu_dgetrs", n, work.data_ptr(), n, ipiv.data_ptr(), x.data_ptr(), info[1:].data_ptr(),
                          wsf.data_ptr(), wsf.numel(), sp)

            res, xs = {}, {}
            steps = max(1, args.steps if n <= 4096 else min(args.steps, 3))
            for name, fn in (("mixed_ir", mixed), ("fp64", plain)):
                times = []
                with ClockSampler(torch.cuda.current_device()) as clk:
                    for i in range(max(1, min(args.warmup, 2)) + steps):
                        work.copy_(A)  # the plain form factors in place; the mixed form reads A only
                        torch.cuda.synchronize()
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        fn()
                        e1.record(stream)
                        torch.cuda.synchronize()
                        if i >= max(1, min(args.warmup, 2)):
                            times.append(e0.elapsed_time(e1))
                ms = float(np.median(times))
                xr = x.clone()
                xs[name] = xr
                # backward error with the residual by Dot2 on the host (outside the timed events)
                if a_host is None:
                    a_host, b_host = A.cpu().numpy(), b.cpu().numpy()
                be = O.dense_backward_error(a_host, n, xr.cpu().numpy(), b_host)
                res[name] = {"ms": ms, "solves_per_s": 1e3 / ms, "gflops_fp64_equivalent": flops / (ms * 1e-3) / 1e9,
                             "backward_error": be, "backward_error_over_n_eps": be / (n * 2.220446049250313e-16),
                             "clocks": clk.summary()}
                if name == "mixed_ir":
                    res[name].update({"refinement_steps": it.value, "fp64_fallback": fb.value == 1,
                                      "path": {0: "classical refinement", 1: "FP64 refactorization",
                                               2: "GMRES-IR (FP32 LU preconditioner)"}.get(fb.value)})
            res["speedup_mixed_over_fp64"] = res["fp64"]["ms"] / res["mixed_ir"]["ms"]
            res["mixed_ir"]["forward_error_vs_fp64_form"] = float((xs["mixed_ir"] - xs["fp64"]).abs().max() /
                                                                  xs["fp64"].abs().max())
            forms[f"n{n}_cond{cond:.0e}"] = res
            if headline is None or (n == max(sizes) and cond == 1e5):
                headline = (n, cond, res)
            del A, b, a_host, b_host
    n, cond, res = headline
    peak = ctypes_probe(L)
    fp64_rate = res["fp64"]["gflops_fp64_equivalent"] * 1e9
    roof = {"bound": "fp64", "achieved": fp64_rate / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": fp64_rate / peak, "traffic": None, "peak_source": fp64_peak_source(),
            "note": ("the plain FP64 form (blocked LU, FP64 DGEMM trailing updates): 2/3 n^3 + 2 n^2 per solve; "
                     "the mixed form's trailing updates run on the BF16 tensor pipe (split_gemm_kernel<float>) "
                     "and its panel is latency-bound")}
    return {"metric": "mixed-precision LU + FP64 refinement (backward error <= n eps64) vs plain FP64 GPU LU",
            "value": res["mixed_ir"]["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 factor (bf16x3 tensor-core updates) + f64 refinement", "data": "synthetic",
            "config": {"workload": "mixed_lu", "n": n, "cond": cond, "nrhs": 1, "sizes": sizes,
                       "conds": conds, "inputs": "A = U diag(s) V^T, U, V from QR of N(0,1), s log-uniform"},
            "forms": forms, "roofline": roof, "gpu_launches": None}


# ----------------------------------------------------------------------------- every config in one line

def _summary(res: dict, keep=()) -> dict:
    out = {k: res.get(k) for k in ("metric", "value", "unit", "ms_per_step", "gflops", "dtype", "config", "roofline",
                                   "clocks", "gpu_launches") if k in res}
    for k in keep:
        if k in res:
            out[k] = res[k]
    return out


def other_configs(args, rank, world) -> dict:
    """The workloads of the other configurations, each measured in this same
    run with its own CUDA-event timing and clocks, so that one default bench
    line carries all of them: batched LU (4096 x 64), mixed LU + refinement
    (n = 8192 at three condition numbers), the adjoint (2048 x 128, f64 and
    f32), GEMM 8192^3 (split and FP64), batched QR least squares (8192
    problems), and the next rows at the reference's bench shapes: batched Mul
    (100 x 100), the 1000 x 1000 triangular solves, the batched 100 x 100 QR
    solve and the QR of one 4096 x 4096 matrix.  Steps are capped for the
    large single-matrix workloads."""
    import copy

    import torch

    out = {}
    plan = (
        ("1_lu_batched", bench_lu_ours, dict(), ("accuracy",)),
        ("3_mixed_lu_n8192", bench_mixed_lu_ours, dict(count=8192, steps=min(args.steps, 2), warmup=1), ("forms",)),
        ("4_adjoint", bench_adjoint_ours, dict(count=0), ("forms",)),
        ("5a_gemm", bench_gemm_ours, dict(count=0, steps=min(args.steps, 10)), ("forms",)),
        ("5b_ls_qr", bench_ls_ours, dict(count=0), ("accuracy",)),
        ("f2_mul_batched_100", bench_mul_batched_ours, dict(count=0), ("forms", "accuracy", "cpu_baseline")),
        ("f2_trsv_large_1000", bench_trsv_large_ours, dict(count=0, steps=min(args.steps, 5)),
         ("forms", "cpu_baseline")),
        ("f_qr_square_100", bench_qr_square_ours, dict(count=0), ("cpu_baseline", "backward_error_sample_in_eps")),
        ("a8_qr_large_4096", bench_qr_large_ours, dict(count=0, steps=min(args.steps, 3)), ("forms", "cpu_baseline")),
    )
    for name, fn, over, keep in plan:
        a = copy.copy(args)
        a.count = 0
        a.exact = False
        for k, v in over.items():
            setattr(a, k, v)
        t0 = time.perf_counter()
        try:
            res = fn(a, rank, world)
            out[name] = _summary(res, keep)
        except Exception as e:  # one workload's failure is reported, not fatal to the headline
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 2)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ragged_cholesky", choices=["ragged_cholesky", "lu_batched", "ls_qr", "adjoint", "gemm",
                                                                  "mixed_lu", "lu_inverse", "trsv_batched", "chol_update",
                                                                        "full_piv_lu", "col_piv_qr", "mul_batched",
                                                                        "trsv_large", "qr_square", "qr_large"])
    ap.add_argument("--exact", action="store_true")
    ap.add_argument("--single-launch", action="store_true",
                    help="ragged_cholesky: one launch over a host-sorted order with the default tile "
                         "(instead of the size-bucketed launches with the tuned tiles)")
    ap.add_argument("--autotune", action="store_true",
                    help="ragged_cholesky: re-run the tile autotuner before timing (not saved)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--count", type=int, default=0, help="ragged_cholesky: override the number of systems")
    ap.add_argument("--e2e-chunks", type=int, default=8,
                    help="ragged_cholesky e2e: chunks of the host-memory pipeline (copy in / solve / copy out)")
    ap.add_argument("--profile", action="store_true", help="timed kernel only (for ncu captures)")
    ap.add_argument("--profile-mixed", action="store_true", help="with --profile: also run the mixed-precision form")
    ap.add_argument("--headline-only", action="store_true",
                    help="ragged_cholesky: skip the other configurations' workloads in the line's `configs` map")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(bench_ragged_reference(args, rank, world)))
        return

    import torch

    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from nalgebra_gb300 import build

    if rank == 0:
        build.build()
    if world > 1:
        torch.distributed.barrier()

    if args.workload in ("lu_batched", "ls_qr", "adjoint", "gemm", "mixed_lu", "lu_inverse", "trsv_batched",
                         "chol_update", "full_piv_lu", "col_piv_qr", "mul_batched", "trsv_large", "qr_square",
                         "qr_large"):
        res = {"lu_batched": bench_lu_ours, "ls_qr": bench_ls_ours, "adjoint": bench_adjoint_ours,
               "gemm": bench_gemm_ours, "mixed_lu": bench_mixed_lu_ours,
               "lu_inverse": bench_lu_inverse_ours, "trsv_batched": bench_trsv_ours,
               "chol_update": bench_chol_update_ours,
               "full_piv_lu": bench_full_piv_lu_ours,
               "col_piv_qr": bench_col_piv_qr_ours, "mul_batched": bench_mul_batched_ours,
               "trsv_large": bench_trsv_large_ours, "qr_square": bench_qr_square_ours,
               "qr_large": bench_qr_large_ours}[args.workload](args, rank, world)
        if rank == 0:
            print(json.dumps(res))
        return

    res, data = bench_ragged_ours(args, rank, world)
    if args.profile:
        print(json.dumps(res))
        return
    res = combine_over_ranks(res, res["config"]["count"], world)
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline_ragged(data)
    del data
    if not args.headline_only and world == 1:
        res["configs"] = other_configs(args, rank, world)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
