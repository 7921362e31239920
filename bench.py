"""Benchmark of the SurfATT travel-time + adjoint path on GB300.

One step = one gradient evaluation of the 3-D-iso workload (config 2/3):
80 stations as sources x 16 periods = 1280 (source, period) solves on a
120x120 lon/lat grid (0.05 deg), each a factored eikonal forward solve,
receiver interpolation (79 receivers), misfit, two adjoint solves (residual
and density sources), mask and the per-period kernel sums (/svel^3).

Headline (`value`): the batched FP32-factored path (tau swept in FP32; T0,
misfit, kernel sums and the convergence test in FP64) in solves/s with the
problem resident in HBM, timed with CUDA events on the engine's stream.
The plain FP64 path runs on the same workload and is reported beside it, with
the FP32-vs-FP64 error.  `e2e` is the same metric through the C ABI with host
buffers: upload of the whole problem from pinned memory + run + download of
kernels, misfit and synthetic times, every step.

`--impl reference` times the reference algorithm's CPU implementation (the
C restatement in oracle/, all host threads, the reference's contiguous
work-list split) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

# Up to 32 hardware work queues for the process's streams (CUDA's default is
# 8): the drop-in workload's 16 caller threads each have their own stream,
# and two streams sharing a queue serialise their launches (a short launch
# waits behind another thread's forward solve).  Read when the CUDA context
# is created, so set before anything initialises CUDA.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "surfatt-iso_gb300"))

# Reference-formulation flops per visit (src/eikon_solver_2d.f90 as written,
# add/sub/mul/div/sqrt = 1 flop), counted on a 32-solve stratified sample of
# this workload by `python oracle/count_flops.py config2 32`.
FWD_FLOPS_PER_VISIT = 351.8
ADJ_FLOPS_PER_VISIT = 16.0
KERNEL_NAMES = {0: "k_batch_fp64", 1: "k_batch_fp32", 2: "k_batch_fp32w"}
# DRAM bytes (read + write) per launch of the FP32 row kernel
# (k_batch_fp32w, variant 0) on the full 1280-solve workload, from one ncu
# capture of the first launch of this bench command (dram__bytes_read.sum
# 14.28 GB + dram__bytes_write.sum 4.57 GB in 17.43 ms):
# profiles/k_batch_fp32w_config3.md.  The per-solve workspaces of the 1216
# resident solves (about 1 GB) do not fit in L2, so operands are re-read
# from DRAM every sweep.  Reported only when the autotuner picked that
# kernel.
DRAM_BYTES_PER_LAUNCH = {"config2": 18.85e9}
METRIC = "eikonal+adjoint solves/s (batched FP32-factored, rel err<=1e-5 vs FP64)"


def _hbm_view(traffic, kernel_ms):
    """The same launch against the HBM roof: its DRAM bytes (ncu) per
    CUDA-event second, over the measured copy bandwidth of this machine."""
    if not traffic:
        return None
    peak = None
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        source = "MEASURED_PEAKS.json hbm_gbs (measured)"
    except (OSError, ValueError, KeyError):
        peak, source = 6800.0, "fallback 6.8 TB/s"
    achieved = traffic / (kernel_ms * 1e-3) / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": source}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2",
                    choices=["config1", "config2", "config2s", "config4", "serving", "smooth",
                             "kernel3d", "worklist", "topo", "dropin"])
    ap.add_argument("--requests", type=int, default=40,
                    help="serving: requests in the Poisson stream")
    ap.add_argument("--load", type=float, default=0.7,
                    help="serving: offered load as a fraction of the closed-loop capacity")
    ap.add_argument("--sigma", type=float, default=0.2,
                    help="smooth: smoothing length in degrees (the example's sigma_2d)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the config 4 and serving side runs")
    return ap.parse_args()


def _workload(name):
    from surfatt_gb300 import workloads as W
    if name == "config1":
        obs = W.read_src_rec_tt(os.path.join(ROOT, "tests", "golden", "config1_src_rec.csv"))
        pb = W.config1(observed_tt=obs)
        desc = "config1: 2-D, 81x81 grid, 25 stations (600 paths), 1 period"
    elif name == "config2s":
        pb = W.config2(nsta=20)
        desc = ("config2s: config 2 with 20 stations (16 periods, 320 solves, 120x120), "
                "a bounded case for profiler captures")
    elif name == "config4":
        pb = W.config4()
        desc = "config4: 120 sources x 25 periods = 3000 solves, grids 64^2..384^2, 3-D mode"
    else:
        pb = W.config2()
        desc = ("config3 (config2 with tau swept in FP32): 3-D-iso gradient evaluation, "
                "80 stations x 16 periods = 1280 solves, 120x120 grid at 0.05 deg, "
                "79 receivers/solve, two adjoints/solve")
    return pb, desc


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist, rank, ws, local


def _barrier(dist, local):
    import torch
    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize(local)


def _max_over_ranks(dist, v, local):
    if dist is None:
        return v
    import torch
    dev = f"cuda:{local}" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.cpu()[0])


class Clocks:
    """nvidia-smi sampling (every 50 ms) around the timed region: start()
    returns once the sampler has written its first sample, and stop() keeps
    the samples stamped between the two calls."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None
        self.t0 = self.t1 = 0.0

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        deadline = time.time() + 2.0
        while self.p is not None and time.time() < deadline:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)
        self.t0 = time.time()

    def stop(self):
        self.t1 = time.time()
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.06)  # the sample that closes the window
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        import datetime
        rows = []
        for line in self.f.read().strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((t, float(parts[2]), float(parts[3]), float(parts[4]), parts[6:10]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        inside = [r for r in rows if self.t0 - 0.06 <= r[0] <= self.t1 + 0.06]
        window = "timed region"
        if not inside:
            inside, window = rows, "whole sampling (no sample inside the timed region)"
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = {n for r in inside for n, v in zip(names, r[4]) if v.lower() == "active"}
        return {"sm_mhz": statistics.median(r[1] for r in inside) if inside else None,
                "sm_max_mhz": max(r[2] for r in inside) if inside else None,
                "power_w_max": max(r[3] for r in inside) if inside else None,
                "samples": len(inside), "window": window,
                "region_s": round(self.t1 - self.t0, 3), "reasons": sorted(reasons)}


def _flush_l2(buf):
    """Write a buffer larger than L2 (129 MB) between timed steps."""
    import torch
    buf.zero_()
    torch.cuda.synchronize()


def _reduce_step(eng, dist):
    """The evaluation's exchange step on N ranks: one NCCL all-reduce of this
    rank's adj_s, adj_density, tt_fwd and chi (device memory, no host copy);
    returns its device time in ms (CUDA events on torch's current stream)."""
    import torch
    from surfatt_gb300 import parallel as par
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    out = par.reduce_device(eng.device_results(), dist)
    b.record()
    b.synchronize()
    return a.elapsed_time(b), out


def _time_steps(eng, pb, prec, steps, warmup, flush, dist=None):
    """Per step: the evaluation's device time (CUDA events on the engine's
    stream) plus, on N > 1 ranks, the all-reduce's (events on the stream it
    runs on)."""
    for _ in range(warmup):
        eng.run(pb.mode, prec)
        eng.sync()
        if dist is not None:
            _reduce_step(eng, dist)
    totals, kernels, launches = [], [], 0
    for _ in range(steps):
        _flush_l2(flush)
        eng.run(pb.mode, prec)
        st = eng.sync()
        t, k, n = eng.timing()
        if dist is not None:
            t += _reduce_step(eng, dist)[0]
        totals.append(t)
        kernels.append(k)
        launches += n
        if st not in (0, 3):
            raise RuntimeError(f"run status {st}")
    return totals, kernels, launches


def _errors(a, b, pb):
    out = {}
    m = b["tt_fwd"] != 0
    out["tt_rel_max"] = float(np.max(np.abs(a["tt_fwd"][m] - b["tt_fwd"][m]) / np.abs(b["tt_fwd"][m])))
    out["chi_rel"] = float(abs(a["chi"] - b["chi"]) / abs(b["chi"]))
    for key in ("adj_s", "adj_density"):
        worst = 0.0
        for p in range(pb.nperiod):
            g0, n = int(pb.goff[p]), int(pb.nx[p] * pb.ny[p])
            den = np.max(np.abs(b[key][g0:g0 + n]))
            if den > 0:
                worst = max(worst, float(np.max(np.abs(a[key][g0:g0 + n] - b[key][g0:g0 + n])) / den))
        out[key + "_rel_max_per_period"] = worst
    return out


def _errors_per_period(a, b, pb):
    """Per period: travel times at the receivers (max pointwise relative
    error), the period's misfit (0.5 sum w (t - tt)^2 over its paths, from
    each side's synthetic times), and adj_s / adj_density (max norm-wise
    relative error).  a: result under test, b: reference result."""
    rows = []
    pid = np.asarray(pb.pidx)
    for p in range(pb.nperiod):
        sol = np.flatnonzero(pid == p)
        if len(sol) == 0:
            continue
        ridx = np.concatenate([np.arange(pb.rec_off[s], pb.rec_off[s] + pb.nrec[s]) for s in sol])
        paths = np.asarray(pb.path)[ridx]
        ta, tb = a["tt_fwd"][paths], b["tt_fwd"][paths]
        m = tb != 0
        w, tt = np.asarray(pb.weight)[ridx], np.asarray(pb.tt)[ridx]
        ca = 0.5 * np.sum(w * (ta - tt) ** 2)
        cb = 0.5 * np.sum(w * (tb - tt) ** 2)
        g0, n = int(pb.goff[p]), int(pb.nx[p] * pb.ny[p])
        row = {"period": p, "grid": f"{int(pb.nx[p])}x{int(pb.ny[p])}", "solves": int(len(sol)),
               "tt_rel_max": float(np.max(np.abs(ta[m] - tb[m]) / np.abs(tb[m]))) if m.any() else 0.0,
               "chi_rel": float(abs(ca - cb) / abs(cb)) if cb else 0.0}
        for key in ("adj_s", "adj_density"):
            den = np.max(np.abs(b[key][g0:g0 + n]))
            row[key + "_rel"] = float(np.max(np.abs(a[key][g0:g0 + n] - b[key][g0:g0 + n])) / den) \
                if den > 0 else 0.0
        rows.append(row)
    return rows


def _config(pb, desc, world):
    """The `config` object of both arms' JSON lines (same keys, same values)."""
    grids = sorted({f"{int(x)}x{int(y)}" for x, y in zip(pb.nx, pb.ny)})
    return {"workload": desc, "solves_per_step": int(pb.nsolve),
            "grid": grids[0] if len(grids) == 1 else grids,
            "periods": int(pb.nperiod), "receivers": int(len(pb.tt)),
            "mode": {3: "3-D (adj and density /svel^3)", 2: "2-D (adj /svel^2)",
                     0: "forward only"}[int(pb.mode)],
            "l2": "flushed (256 MB write) between timed steps",
            "parallelism": (f"{world} GPU(s): the work list split by predicted cost (cells x "
                            f"iterations), one NCCL all-reduce of adj_s, adj_density, tt_fwd and "
                            f"chi per step" if world > 1 else "1 GPU")}


def _pinned_problem(pb):
    """Copies of the problem's arrays in pinned host memory."""
    import dataclasses
    import torch

    def pin(a):
        a = np.ascontiguousarray(a)
        t = torch.empty(a.shape, dtype={np.dtype(np.float64): torch.float64,
                                        np.dtype(np.int32): torch.int32,
                                        np.dtype(np.int64): torch.int64}[a.dtype],
                        pin_memory=True)
        v = t.numpy()
        v[...] = a
        return v, t

    keep, kw = [], {}
    for f in dataclasses.fields(pb):
        v = getattr(pb, f.name)
        if isinstance(v, np.ndarray):
            arr, t = pin(v)
            keep.append(t)
            kw[f.name] = arr
    return dataclasses.replace(pb, **kw), keep


def run_ours(args):
    import torch
    import surfatt_gb300 as sg
    from surfatt_gb300 import parallel as par
    dist, rank, world, local = _dist()
    sg.build()
    pb_full, desc = _workload(args.workload)
    # N ranks: one gradient evaluation split by predicted cost, each rank its
    # shard (same periods and path table), results summed every step
    pb = par.shard(pb_full, world, rank) if world > 1 else pb_full
    dev = local
    torch.cuda.set_device(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{dev}")
    fp64_peak, fp32_peak = sg.measure_peaks(dev)
    eng = sg.Engine(dev)
    eng.load(pb)
    # both paths get the autotuner (FP64: solves cut into work items or whole)
    tuned64 = eng.autotune(pb.mode, sg.PREC_FP64)
    # correctness of the headline against the plain FP64 path on this workload
    eng.run(pb.mode, sg.PREC_FP64)
    eng.sync()
    r64 = eng.results()
    fwd64, adj64 = eng.work()
    launch64 = dict(eng.launch_config(), **eng.kernel_variant())
    tuned = eng.autotune(pb.mode, sg.PREC_FP32)
    eng.run(pb.mode, sg.PREC_FP32)
    eng.sync()
    r32 = eng.results()
    fwd32, adj32 = eng.work()
    launch32 = dict(eng.launch_config(), **eng.kernel_variant())
    err32 = _errors(r32, r64, pb)

    # plain FP64 (reported beside the headline)
    t64, k64, _ = _time_steps(eng, pb, sg.PREC_FP64, max(1, min(args.steps, 3)), 1, flush)
    # headline: FP32-factored, timed region bracketed by barrier + synchronize
    clocks = Clocks(dev)
    _barrier(dist, dev)
    clocks.start()
    t0 = time.perf_counter()
    t32, k32, launches = _time_steps(eng, pb, sg.PREC_FP32, args.steps, args.warmup, flush, dist)
    wall = time.perf_counter() - t0
    _barrier(dist, dev)
    ck = clocks.stop()
    ms_step = statistics.mean(t32)
    ms_step_max = _max_over_ranks(dist, ms_step, dev)
    value = pb_full.nsolve / (ms_step_max / 1e3)

    e2e = None
    if not args.no_e2e:
        ppb, keep = _pinned_problem(pb)
        into = {}
        for name, n, dt in (("adj_s", pb.ncell, np.float64), ("adj_density", pb.ncell, np.float64),
                            ("tt_fwd", pb.npath, np.float64), ("status", pb.nsolve, np.int32),
                            ("fwd_iters", pb.nsolve, np.int32), ("adj_iters", pb.nsolve, np.int32),
                            ("chi", 1, np.float64)):
            t = torch.empty(max(n, 1), dtype=torch.float64 if dt == np.float64 else torch.int32,
                            pin_memory=True)
            keep.append(t)
            into[name] = t.numpy()
        h2d = sum(getattr(ppb, f).nbytes for f in ("xgrid", "ygrid", "svel", "m11", "m12", "m22",
                                                    "pidx", "srcx", "srcy", "rec_off", "nrec",
                                                    "recx", "recy", "tt", "weight", "path"))
        d2h = sum(into[k].nbytes for k in into)
        e2e_t = []
        for i in range(args.warmup + args.steps):
            _flush_l2(flush)
            _barrier(dist, dev)
            a = time.perf_counter()
            eng.load(ppb)
            eng.run(pb.mode, sg.PREC_FP32)
            eng.sync()
            if dist is not None:
                # this rank's per-solve results, then the sums over the ranks
                eng.results(adj=False, density=False, tt=False, into=into)
                red = _reduce_step(eng, dist)[1]
                for k in ("adj_s", "adj_density", "tt_fwd", "chi"):
                    if red[k] is not None:
                        torch.from_numpy(into[k][:red[k].numel()]).copy_(red[k])
            else:
                eng.results(into=into)
            b = time.perf_counter()
            if i >= args.warmup:
                e2e_t.append(b - a)
        e2e_s = _max_over_ranks(dist, statistics.mean(e2e_t), dev)
        e2e = {"value": pb_full.nsolve / e2e_s, "unit": "solves/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": e2e_s * 1e3, "host_buffers": "pinned"}

    # roofline of the dominant kernel (the fused batched solve kernel)
    flops32 = fwd32 * FWD_FLOPS_PER_VISIT + adj32 * ADJ_FLOPS_PER_VISIT
    flops64 = fwd64 * FWD_FLOPS_PER_VISIT + adj64 * ADJ_FLOPS_PER_VISIT
    k32_ms = statistics.mean(k32)
    k64_ms = statistics.mean(k64)
    ach32 = flops32 / (k32_ms * 1e-3) / 1e12
    ach64 = flops64 / (k64_ms * 1e-3) / 1e12
    traffic = DRAM_BYTES_PER_LAUNCH.get(args.workload) if launch32.get("kind") == 2 else None

    # where the solve kernel's time goes: one more evaluation with the
    # per-phase SM cycle counters on (outside the timed region)
    eng.set_profile(True)
    eng.run(pb.mode, sg.PREC_FP32)
    eng.sync()
    ph = eng.phase_cycles()
    eng.set_profile(False)
    phases = {k: v / max(pb.nsolve, 1) / 1e6 for k, v in ph.items()}

    cpu = None
    parity = {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        nthr = os.cpu_count() or 1
        # parity against the -ffp-contract=off build (untimed), the CPU
        # baseline timed on the -O3 build of the same sources
        ref = O.gradient_eval(pb, mode=pb.mode, nthreads=nthr)
        a = time.perf_counter()
        O.gradient_eval(pb, mode=pb.mode, nthreads=nthr, timed=True)
        b = time.perf_counter()
        cpu = {"value": pb.nsolve / (b - a), "unit": "solves/s", "cores": nthr, "kind": "port",
               "sample": f"the full workload ({pb.nsolve} solves), one evaluation, "
                         f"{nthr} threads, contiguous work-list blocks",
               "build": O.FAST_FLAGS, "seconds": b - a}
        parity = {"fp64_vs_oracle": _errors(r64, ref, pb), "fp32_vs_oracle": _errors(r32, ref, pb),
                  "oracle_build": O.STRICT_FLAGS,
                  "fp32_vs_oracle_per_period": _errors_per_period(r32, ref, pb),
                  "fp64_vs_oracle_per_period": _errors_per_period(r64, ref, pb)}

    side = {}
    if rank == 0 and world == 1 and not args.no_extras and args.workload == "config2":
        side["config4"] = _side_config4(sg, flush, dev)
        side["serving"] = _side_serving(sg, dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step_max,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32 sweep / f64 T0, misfit, kernels", "data": "synthetic",
            "config": _config(pb_full, desc, world),
            "p50_ms": statistics.median(t32), "p99_ms": float(np.percentile(t32, 99)),
            "cell_updates_per_s": (fwd32 + adj32) * world / (ms_step_max / 1e3),
            "plain_fp64": {"value": pb_full.nsolve / (statistics.mean(t64) / 1e3),
                           "unit": "solves/s", "ms_per_step": statistics.mean(t64),
                           "solve_kernel_ms": k64_ms, "achieved_tflops": ach64,
                           "peak_tflops_fp64": fp64_peak, "frac": ach64 / fp64_peak},
            "speedup_fp32_vs_fp64": statistics.mean(t64) / ms_step,
            "fp32_vs_fp64_error": err32,
            "clocks": ck, "e2e": e2e, "gpu_launches": launches,
            "roofline": {"bound": "fp32", "bound_note": "FP32 issue (no contraction: no tensor "
                         "cores); algorithmic flops = reference formulation per visit",
                         "achieved": ach32, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": ach32 / fp32_peak, "traffic": traffic,
                         "peak_source": "surfatt_measure_peaks (FP32 FMA chains), this run",
                         "kernel": KERNEL_NAMES.get(launch32.get("kind"), "k_batch_fp32"),
                         "kernel_ms": k32_ms,
                         "flops_per_launch": flops32,
                         "hbm_view": _hbm_view(traffic, k32_ms)},
            "cpu_baseline": cpu, "parity": parity,
            "phase_mcycles_per_solve": phases,
            "launch": {"fp32": launch32, "fp64": launch64, "autotune": tuned,
                       "autotune_fp64": tuned64},
            "iterations": {"fwd_mean": float(np.mean(r32["fwd_iters"])),
                           "adj_mean": float(np.mean(r32["adj_iters"]))},
            "wall_s_timed_region": wall,
        }
        line.update(side)
        print(json.dumps(line))
    eng.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def run_reference(args):
    dist, rank, world, local = _dist()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    if args.workload == "smooth":
        return _run_reference_smooth(args, O, dist)
    if args.workload == "kernel3d":
        return _run_reference_kernel3d(args, O, dist)
    if args.workload == "worklist":
        return _run_reference_worklist(args, O, dist)
    if args.workload == "topo":
        return _run_reference_topo(args, O, dist)
    if args.workload == "dropin":
        return _run_reference_dropin(args, O, dist)
    pb, desc = _workload(args.workload)
    nthr = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.gradient_eval(pb, mode=pb.mode, nthreads=nthr, timed=True)
    ts = []
    for _ in range(args.steps):
        a = time.perf_counter()
        r = O.gradient_eval(pb, mode=pb.mode, nthreads=nthr, timed=True)
        ts.append(time.perf_counter() - a)
        if r["rc"] not in (0, 3):
            raise RuntimeError(f"oracle status {r['rc']}")
    s = statistics.mean(ts)
    v = pb.nsolve / s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(pb, desc, world),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": nthr, "kind": "port",
                             "sample": f"the full workload ({pb.nsolve} solves) per step",
                             "build": O.FAST_FLAGS},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/ on all host threads"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def _run_reference_smooth(args, O, dist):
    """Reference arm of the smoothing workload: the oracle's
    gaussian_smooth_geo_2 of every period's adj_s, periods spread over
    worker processes as the reference spreads them over MPI ranks."""
    import multiprocessing as mp
    from surfatt_gb300 import workloads as W
    nthr = min(os.cpu_count() or 1, 16)
    pool = mp.get_context("spawn").Pool(nthr)
    pb = W.config2(mode=2)
    adj = O.gradient_eval(pb, mode=2, nthreads=os.cpu_count() or 1)["adj_s"]
    jobs = [(f, *_period_axes(pb, p), args.sigma) for p, f in enumerate(_period_views(pb, adj))]
    ts = []
    for i in range(args.warmup + args.steps):
        a = time.perf_counter()
        pool.map(_oracle_smooth_one, jobs)
        if i >= args.warmup:
            ts.append(time.perf_counter() - a)
    pool.close()
    pool.join()
    s = statistics.mean(ts)
    v = pb.nperiod / s
    line = {"impl": "reference",
            "metric": "kernel smoothing periods/s (gaussian_smooth_geo_2 of every period's adj_s)",
            "value": v, "unit": "periods/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "tomo2d kernel smoothing on config 2's grids: 16 periods, "
                                   "120x120 at 0.05 deg", "sigma_deg": args.sigma},
            "cpu_baseline": {"value": v, "unit": "periods/s", "cores": nthr, "kind": "port",
                             "sample": f"all {pb.nperiod} periods per step, one per process"},
            "e2e": {"value": v, "unit": "periods/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def _latency_breakdown(reqs, lat):
    """p50 / p99 request latency per grid side and per request kind, with
    the requests' solve counts: whether a tail is queueing or the large
    grids' own run time."""
    out = {}
    for key, groups in (("by_grid", sorted({r["n"] for r in reqs})),
                        ("by_kind", ("gradient", "linesearch", "checkerboard"))):
        tab = {}
        for g in groups:
            idx = [q for q, r in enumerate(reqs) if r["n" if key == "by_grid" else "kind"] == g]
            if not idx:
                continue
            v = np.asarray([lat[q] for q in idx])
            tab[f"{g}^2" if key == "by_grid" else g] = {
                "requests": len(idx), "solves_mean": float(np.mean([reqs[q]["nsolve"] for q in idx])),
                "p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99))}
        out[key] = tab
    return out


def _serving_measure(sg, S, local, nreq, load, warmup, dist=None):
    """Closed-loop capacity, then a Poisson stream at `load` of it."""
    cat = S.Catalog()
    reqs = S.make_requests(cat, nreq, seed=4)
    srv = sg.Server(local, hbm_budget_bytes=16 << 30, max_inflight=8)
    mids = {n: srv.add_model(cat.models[n]) for n in cat.models}
    # warm-up: the first requests of the stream, run once and discarded
    warm = S.run_poisson(srv, reqs[:max(3, warmup)], 1e6, sg.PREC_FP32, model_ids=mids)
    closed = S.run_poisson(srv, reqs, 1e6, sg.PREC_FP32, model_ids=mids)
    cap_rate = len(reqs) / closed["wall_s"]
    rate = load * cap_rate
    clocks = Clocks(local)
    _barrier(dist, local)
    clocks.start()
    res = S.run_poisson(srv, reqs, rate, sg.PREC_FP32, seed=5, model_ids=mids)
    _barrier(dist, local)
    ck = clocks.stop()
    st = srv.stats()
    srv.close()
    return cat, reqs, warm, closed, res, cap_rate, rate, ck, st


def _side_serving(sg, dev):
    """The serving loop beside the headline (30 requests at 70 % of the
    closed-loop capacity): solves/s, p50 / p99 and their breakdown."""
    from surfatt_gb300 import serving as S
    cat, reqs, warm, closed, res, cap, rate, ck, st = _serving_measure(sg, S, dev, 30, 0.7, 3)
    lat = np.asarray(res["latency_ms"])
    bad = [x for x in res["status"] + closed["status"] + warm["status"] if x not in (0, 3)]
    return {"metric": "serving solves/s (Poisson request stream, FP32-factored)",
            "value": res["solves"] / res["wall_s"], "unit": "solves/s",
            "requests": len(reqs), "solves": res["solves"], "load": 0.7,
            "offered_rate_per_s": rate, "closed_loop_rate_per_s": cap,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "closed_loop_solves_per_s": closed["solves"] / closed["wall_s"],
            "breakdown": _latency_breakdown(reqs, lat), "failed_requests": len(bad),
            "inflight_peak": st["inflight_peak"], "clocks": ck}


def _side_config4(sg, flush, dev):
    """Config 4 beside the headline: 120 sources x 25 periods = 3000 solves
    on grids of 64^2 .. 384^2 (3-D mode), FP32-factored and plain FP64 on
    the same engine (each path's kernel variant picked by the autotuner),
    each timed with CUDA events on the engine's stream (L2 flushed between
    steps), the FP32 error against the FP64 results."""
    from surfatt_gb300 import workloads as W
    pb = W.config4()
    eng = sg.Engine(dev)
    eng.load(pb)
    eng.autotune(pb.mode, sg.PREC_FP64)
    eng.autotune(pb.mode, sg.PREC_FP32)
    eng.run(pb.mode, sg.PREC_FP64)
    eng.sync()
    r64 = eng.results()
    eng.run(pb.mode, sg.PREC_FP32)
    eng.sync()
    r32 = eng.results()
    variant = eng.kernel_variant()
    t64, k64, _ = _time_steps(eng, pb, sg.PREC_FP64, 2, 1, flush)
    clocks = Clocks(dev)
    clocks.start()
    t32, k32, n32 = _time_steps(eng, pb, sg.PREC_FP32, 3, 2, flush)
    ck = clocks.stop()
    eng.close()
    ms32, ms64 = statistics.mean(t32), statistics.mean(t64)
    return {"workload": "config4: 120 sources x 25 periods = 3000 solves, grids 64^2..384^2, "
                        "3-D mode", "solves_per_step": pb.nsolve,
            "fp32": {"value": pb.nsolve / (ms32 / 1e3), "unit": "solves/s", "ms_per_step": ms32,
                     "solve_kernel_ms": statistics.mean(k32), "steps": 3, "warmup": 2,
                     "kernel": variant, "gpu_launches": n32},
            "plain_fp64": {"value": pb.nsolve / (ms64 / 1e3), "unit": "solves/s",
                           "ms_per_step": ms64, "solve_kernel_ms": statistics.mean(k64)},
            "speedup_fp32_vs_fp64": ms64 / ms32,
            "fp32_vs_fp64_error": _errors(r32, r64, pb), "clocks": ck}


def run_serving(args):
    """Serving workload (curved surface, seed 4): a closed-loop pass (every
    request queued at once) measures the server's capacity; the Poisson
    stream then offers `--load` of that capacity and its p50/p99 request
    latency and solves/s are reported.  Each rank serves its own stream."""
    import torch
    import surfatt_gb300 as sg
    from surfatt_gb300 import serving as S
    dist, rank, world, local = _dist()
    sg.build()
    torch.cuda.set_device(local)
    cat, reqs, warm, closed, res, cap_rate, rate, ck, st = _serving_measure(
        sg, S, local, args.requests, args.load, args.warmup, dist)
    lat = np.asarray(res["latency_ms"])
    bad = [s for s in res["status"] + closed["status"] + warm["status"] if s not in (0, 3)]
    wall = _max_over_ranks(dist, res["wall_s"], local)
    kinds = {k: sum(1 for r in reqs if r["kind"] == k) for k in ("gradient", "linesearch",
                                                                   "checkerboard")}
    if rank == 0:
        line = {
            "metric": "serving solves/s (Poisson request stream, FP32-factored)",
            "value": res["solves"] * world / wall, "unit": "solves/s", "n_gpus": world,
            "steps": len(reqs), "warmup": len(warm["status"]), "ms_per_step": float(np.mean(lat)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 sweep / f64 T0, misfit, kernels", "data": "synthetic",
            "config": {"workload": "serving on a curved surface (seed 4): Gaussian island 4 km "
                                   "+ 200 m roughness, surface-metric eikonal, grids 64^2..512^2, "
                                   "15 periods, 140 stations; requests of 10-120 sources x 1-15 "
                                   "periods (gradient / line-search trial / checkerboard forward)",
                       "requests": len(reqs), "request_kinds": kinds,
                       "solves": res["solves"], "offered_rate_per_s": rate,
                       "closed_loop_rate_per_s": cap_rate, "load": args.load,
                       "hbm_budget_bytes": st["hbm_budget_bytes"], "max_inflight": 8},
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "closed_loop": {"solves_per_s": closed["solves"] / closed["wall_s"],
                            "p50_ms": float(np.percentile(closed["latency_ms"], 50)),
                            "p99_ms": float(np.percentile(closed["latency_ms"], 99))},
            "server_stats": st, "failed_requests": len(bad), "clocks": ck,
            "breakdown": _latency_breakdown(reqs, lat),
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _oracle_smooth_one(job):
    """One period of the oracle's gaussian_smooth_geo_2 (a pool worker)."""
    if os.path.join(ROOT, "oracle") not in sys.path:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    data, lons, lats, sigma = job
    return O.gaussian_smooth_geo_2(data, lons, lats, sigma)


def _period_views(pb, a):
    out = []
    for p in range(pb.nperiod):
        nx, ny, g = int(pb.nx[p]), int(pb.ny[p]), int(pb.goff[p])
        out.append(a[g:g + nx * ny].reshape((nx, ny), order="F"))
    return out


def _period_axes(pb, p):
    return (pb.xgrid[pb.xoff[p]:pb.xoff[p] + pb.nx[p]],
            pb.ygrid[pb.yoff[p]:pb.yoff[p] + pb.ny[p]])


def run_smooth(args):
    """Kernel smoothing of tomo2d's optimize step (gaussian_smooth_geo_2 of
    every period's adj_s, src/tomo2d.f90:216-222) on config 2's grids:
    16 periods of 120x120 at 0.05 deg, sigma 0.2 deg.  value: periods/s from
    the device time of the engine's two smoothing kernels on the resident
    adj_s; e2e: the drop-in call per period with host buffers."""
    import multiprocessing as mp
    import torch
    import surfatt_gb300 as sg
    from surfatt_gb300 import workloads as W
    dist, rank, world, local = _dist()
    # the oracle's process pool starts before the first GPU call
    pool = None
    nthr = os.cpu_count() or 1
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pool = mp.get_context("spawn").Pool(min(nthr, 16))
    sg.build()
    dev = local
    torch.cuda.set_device(dev)
    pb = W.config2(mode=2)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{dev}")
    fp64_peak, _ = sg.measure_peaks(dev)
    eng = sg.Engine(dev)
    eng.load(pb)
    eng.run(2, sg.PREC_FP64)
    eng.sync()
    adj = eng.results()["adj_s"]
    ker = eng.smooth(args.sigma)  # builds the weight table (kept for later calls)
    first_ms, _, first_n = eng.smooth_timing()
    for _ in range(args.warmup):
        eng.smooth(args.sigma, host=False)
        eng.sync()
    clocks = Clocks(dev)
    _barrier(dist, dev)
    clocks.start()
    kms, launches = [], 0
    for _ in range(args.steps):
        _flush_l2(flush)
        eng.smooth(args.sigma, host=False)
        eng.sync()
        ms, taps, n = eng.smooth_timing()
        kms.append(ms)
        launches += n
    _barrier(dist, dev)
    ck = clocks.stop()
    ms_step = _max_over_ranks(dist, statistics.mean(kms), dev)
    value = pb.nperiod * world / (ms_step / 1e3)
    ach = 2.0 * taps / (statistics.mean(kms) * 1e-3) / 1e12

    # end to end: the drop-in per period, pinned host buffers
    e2e = None
    if not args.no_e2e:
        keep, jobs = [], []
        for p, f in enumerate(_period_views(pb, adj)):
            lons, lats = _period_axes(pb, p)
            d = torch.empty(f.size, dtype=torch.float64, pin_memory=True)
            d.numpy()[:] = f.ravel(order="F")
            keep.append(d)
            jobs.append((d.numpy().reshape(f.shape, order="F"), lons, lats))
        h2d = sum(j[0].nbytes + j[1].nbytes + j[2].nbytes for j in jobs)
        d2h = sum(j[0].nbytes for j in jobs)
        ts = []
        for i in range(args.warmup + args.steps):
            _flush_l2(flush)
            a = time.perf_counter()
            for data, lons, lats in jobs:
                sg.gaussian_smooth_geo_2(data, lons, lats, args.sigma)
            b = time.perf_counter()
            if i >= args.warmup:
                ts.append(b - a)
        e2e_s = _max_over_ranks(dist, statistics.mean(ts), dev)
        e2e = {"value": pb.nperiod * world / e2e_s, "unit": "periods/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": e2e_s * 1e3, "host_buffers": "pinned input, pageable output",
               "call": "surfatt_gaussian_smooth_geo_2 once per period"}

    cpu, parity = None, {}
    if pool is not None:
        jobs = [(f, *_period_axes(pb, p), args.sigma)
                for p, f in enumerate(_period_views(pb, adj))]
        a = time.perf_counter()
        refs = pool.map(_oracle_smooth_one, jobs)
        b = time.perf_counter()
        pool.close()
        pool.join()
        cpu = {"value": pb.nperiod / (b - a), "unit": "periods/s", "cores": min(nthr, 16),
               "kind": "port", "seconds": b - a,
               "sample": f"all {pb.nperiod} periods, one per worker process (the reference "
                         "splits periods over MPI ranks, src/tomo2d.f90:210)"}
        worst = 0.0
        for p, (g, r) in enumerate(zip(_period_views(pb, ker), refs)):
            worst = max(worst, float(np.max(np.abs(g - r)) / np.max(np.abs(r))))
        parity = {"ker_s_rel_max_per_period_vs_oracle": worst}

    if rank == 0:
        line = {
            "metric": "kernel smoothing periods/s (gaussian_smooth_geo_2 of every period's adj_s)",
            "value": value, "unit": "periods/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "tomo2d kernel smoothing on config 2's grids: 16 periods, "
                                   "120x120 at 0.05 deg, adj_s of an FP64 gradient evaluation "
                                   "(80 stations)", "sigma_deg": args.sigma,
                       "window_taps_per_step": taps,
                       "weight_table": "built by the first call (grid and sigma fixed), "
                                       "kept for the timed steps",
                       "l2": "flushed (256 MB write) between timed steps"},
            "first_call_ms": {"table_and_apply": first_ms, "launches": first_n},
            "clocks": ck, "e2e": e2e, "gpu_launches": launches,
            "roofline": {"bound": "fp64", "bound_note": "FP64 issue: one fma per window tap "
                         "(2 flops)",
                         "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ach / fp64_peak, "traffic": None,
                         "peak_source": "surfatt_measure_peaks (FP64 FMA chains), this run",
                         "kernel": "k_smooth_apply",
                         "kernel_ms": statistics.mean(kms)},
            "cpu_baseline": cpu, "parity": parity,
        }
        print(json.dumps(line))
    eng.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _dropin_case():
    """Config 1 as the unchanged tomo2d drives the solver drop-ins: per
    source the forward solve, the adjoint solve with the residual sources
    and the mask (src/measadj.f90:62-90, called from src/tomo2d.f90:177-189),
    every call with host arrays.  The adjoint sources come from one FP64
    evaluation of the same model (outside the timed region)."""
    from surfatt_gb300 import workloads as W
    obs = W.read_src_rec_tt(os.path.join(ROOT, "tests", "golden", "config1_src_rec.csv"))
    pb = W.config1(observed_tt=obs)
    F = lambda a: np.asfortranarray(a, dtype=np.float64)
    xx, yy = (np.ascontiguousarray(v, dtype=np.float64) for v in pb.grid(0))
    a, b, c = F(pb.field("m11", 0)), F(pb.field("m22", 0)), F(-pb.field("m12", 0))
    fun = F(1.0 / pb.field("svel", 0))
    srcs = []
    for s in range(pb.nsolve):
        r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
        sl = slice(r0, r0 + nr)
        srcs.append(dict(x0=float(pb.srcx[s]), y0=float(pb.srcy[s]),
                         xr=np.ascontiguousarray(pb.recx[sl]), yr=np.ascontiguousarray(pb.recy[sl]),
                         tt=np.asarray(pb.tt[sl]), w=np.asarray(pb.weight[sl]),
                         path=np.asarray(pb.path[sl])))
    return pb, xx, yy, a, b, c, fun, srcs


def _dropin_sadj(srcs, tt_fwd):
    """sourceAdj = weight*(tekio-tt) after the outlier zeroing (src/measadj.f90:82-88)."""
    for d in srcs:
        tek = tt_fwd[d["path"]]
        w = np.where(np.abs(tek - d["tt"]) / d["tt"] > 0.5, 0.0, d["w"])
        d["sadj"] = np.ascontiguousarray(w * (tek - d["tt"]))


def _dropin_blocks(n, parts):
    """Contiguous split of n sources over `parts` callers, the first ones one
    larger (src/shared/parallel.f90 scatter_all_i)."""
    q, r = divmod(n, parts)
    out, lo = [], 0
    for k in range(parts):
        hi = lo + q + (1 if k < r else 0)
        out.append(range(lo, hi))
        lo = hi
    return out


def _oracle_dropin_block(job):
    """One caller's sources through the oracle's forward, adjoint and mask."""
    import oracle as O
    xx, yy, a, b, c, fun, block = job
    for d in block:
        T, _, _ = O.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, d["x0"], d["y0"])
        Ta, _, _ = O.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, T, d["xr"], d["yr"], d["sadj"])
        O.mask(xx, yy, Ta, d["x0"], d["y0"])
    return len(block)


def run_dropin(args):
    """The gfortran-mangled drop-ins (fsm_uw_ps_lonlat_2d_, fsm_o1_jse_lonlat_2d_,
    mask_) on config 1, called per source exactly as the unchanged Fortran
    calls them, from 1 host thread and from one thread per host core (the
    reference runs one MPI rank per core, each calling the solver for its
    block of sources).  Each call copies its host arrays in and its result
    out: `value` and `e2e` are the same measurement."""
    import ctypes
    import multiprocessing as mp
    import threading
    import torch
    import surfatt_gb300 as sg
    dist, rank, world, local = _dist()
    ncores = os.cpu_count() or 1
    pool = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        pool = mp.get_context("spawn").Pool(1)
    sg.build()
    torch.cuda.set_device(local)
    pb, xx, yy, a, b, c, fun, srcs = _dropin_case()
    eng = sg.Engine(local)
    _dropin_sadj(srcs, eng.evaluate(pb, mode=2)["tt_fwd"])
    eng.close()
    fp64_peak, _ = sg.measure_peaks(local)
    nx, ny = len(xx), len(yy)
    N = nx * ny
    L = sg.lib()
    # The callers are Python threads: every drop-in call releases the GIL,
    # but a thread returning from one waits for the GIL up to the switch
    # interval (5 ms by default) while another runs Python code between its
    # calls.  Fortran callers (MPI ranks) have no such lock: a short switch
    # interval keeps the harness's own lock out of the measured calls.
    sys.setswitchinterval(1e-5)
    dp = lambda v: v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ci = lambda v: ctypes.byref(ctypes.c_int(v))
    cd = lambda v: ctypes.byref(ctypes.c_double(v))
    fwd_fn, adj_fn, mask_fn = L.fsm_uw_ps_lonlat_2d_, L.fsm_o1_jse_lonlat_2d_, L.mask_
    status, iterations = L.surfatt_last_status, L.surfatt_last_iterations

    def prepare(blocks):
        """Per caller (block of sources): its own T, Ta and scratch arrays and
        the ctypes arguments of every call, built once outside the timed
        region (Fortran passes its arrays by reference; building ctypes
        pointers would hold the GIL inside the measurement)."""
        out = []
        for block in blocks:
            T = np.zeros((nx, ny), order="F")
            Ta = np.zeros((nx, ny), order="F")
            u = np.zeros((nx, ny), order="F")
            common = (dp(xx), dp(yy), ci(nx), ci(ny), dp(a), dp(b), dp(c))
            calls = []
            for k in block:
                d = srcs[k]
                calls.append(((*common, dp(T), dp(fun), cd(d["x0"]), cd(d["y0"]), dp(u)),
                              (*common, dp(T), dp(Ta), dp(d["xr"]), dp(d["yr"]), dp(d["sadj"]),
                               ci(len(d["xr"]))),
                              (dp(xx), dp(yy), ci(nx), ci(ny), dp(Ta), cd(d["x0"]),
                               cd(d["y0"]))))
            out.append((calls, (T, Ta, u)))
        return out

    def run_block(job):
        calls, _ = job
        its = [0, 0]
        for fa, aa, ma in calls:
            fwd_fn(*fa)
            if status() != sg.OK:
                raise RuntimeError(f"forward drop-in status {status()}")
            its[0] += iterations()
            adj_fn(*aa)
            if status() != sg.OK:
                raise RuntimeError(f"adjoint drop-in status {status()}")
            its[1] += iterations()
            mask_fn(*ma)
        return its

    def timed(nthreads):
        """One persistent thread per caller, each owning its block of sources
        for the whole run (as an MPI rank owns its sources), started and
        joined every step by two barriers; a step lasts from the start
        barrier until the last caller's last call returns."""
        jobs = prepare(_dropin_blocks(len(srcs), nthreads))
        nstep = args.warmup + args.steps
        go = threading.Barrier(nthreads + 1)
        done = threading.Barrier(nthreads + 1)
        res = [[None] * nthreads for _ in range(nstep)]
        err = []

        def caller(r):
            for i in range(nstep):
                go.wait()
                try:
                    res[i][r] = run_block(jobs[r])
                except Exception as e:  # reported after the step
                    err.append(e)
                    res[i][r] = [0, 0]
                done.wait()

        threads = [threading.Thread(target=caller, args=(r,), daemon=True)
                   for r in range(nthreads)]
        for t in threads:
            t.start()
        ts, its = [], [0, 0]
        for i in range(nstep):
            go.wait()
            t0 = time.perf_counter()
            done.wait()
            t1 = time.perf_counter()
            if err:
                raise err[0]
            if i >= args.warmup:
                ts.append(t1 - t0)
                its = [its[0] + sum(r[0] for r in res[i]), its[1] + sum(r[1] for r in res[i])]
        for t in threads:
            t.join()
        return statistics.mean(ts), its

    clocks = Clocks(local)
    _barrier(dist, local)
    clocks.start()
    s_many, its = timed(ncores)
    _barrier(dist, local)
    ck = clocks.stop()
    s_one, _ = timed(1)
    s_many = _max_over_ranks(dist, s_many, local)
    value = len(srcs) * world / s_many
    # FP64 work of the timed calls (reference formulation), over wall time
    fwd_visits = its[0] / args.steps * 4 * N
    adj_visits = its[1] / args.steps * 4 * (nx - 2) * (ny - 2)
    flops = fwd_visits * FWD_FLOPS_PER_VISIT + adj_visits * ADJ_FLOPS_PER_VISIT
    ach = flops / s_many / 1e12
    nr_tot = sum(len(d["xr"]) for d in srcs)
    h2d = len(srcs) * ((4 * N + nx + ny) + (4 * N + nx + ny) + (N + nx + ny)) * 8 + nr_tot * 3 * 8
    d2h = len(srcs) * 3 * N * 8

    # parity of the drop-ins on two sources against the oracle (outside timing)
    parity, cpu = {}, None
    if pool is not None:
        worst_t = worst_a = 0.0
        for k in (0, len(srcs) - 1):
            d = srcs[k]
            T, _, _ = sg.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, d["x0"], d["y0"])
            Ta, _, _ = sg.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, T, d["xr"], d["yr"], d["sadj"])
            Ta = sg.mask(xx, yy, Ta, d["x0"], d["y0"])
            Tr, _, _ = O.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, d["x0"], d["y0"])
            Tar, _, _ = O.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, Tr, d["xr"], d["yr"], d["sadj"])
            Tar = O.mask(xx, yy, Tar, d["x0"], d["y0"])
            worst_t = max(worst_t, float(np.max(np.abs(T - Tr) / np.abs(Tr).clip(1e-30))))
            worst_a = max(worst_a, float(np.linalg.norm(Ta - Tar) / np.linalg.norm(Tar)))
        parity = {"tt_rel_max_vs_oracle": worst_t, "adjoint_rel_norm_vs_oracle": worst_a}
        # the oracle's same calls on one core, a sample of 8 sources
        sample = list(range(8))
        t0 = time.perf_counter()
        pool.map(_oracle_dropin_block, [(xx, yy, a, b, c, fun, [srcs[k] for k in sample])])
        t1 = time.perf_counter()
        pool.close()
        pool.join()
        cpu = {"value": len(sample) / (t1 - t0), "unit": "sources/s", "cores": 1,
               "kind": "port", "seconds": t1 - t0,
               "sample": "8 of the 25 sources, forward + adjoint + mask each, one process"}

    if rank == 0:
        line = {
            "metric": "drop-in solves/s (forward + adjoint + mask per source through the "
                      "gfortran-mangled symbols, host arrays)",
            "value": value, "unit": "sources/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s_many * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "config1 through the drop-ins: 81x81, 25 sources x 24 "
                                   "receivers, 2-D mode (one adjoint per source)",
                       "callers": ncores, "caller_kind": "persistent host threads (one "
                       "per core, as the reference's MPI ranks), each owning a contiguous "
                       "block of sources; a step runs from a start barrier to the last "
                       "caller's last call",
                       "single_caller": {"value": len(srcs) / s_one, "unit": "sources/s",
                                         "ms_per_step": s_one * 1e3},
                       "note": "every call takes host arrays and returns its result in "
                               "host arrays: value and e2e are the same measurement; a "
                               "calling thread's inputs that equal, bit for bit, what its "
                               "context already holds on the device (grid, metric and "
                               "slowness of its previous call, the travel times or adjoint "
                               "field its previous call returned) are not copied again, so "
                               "h2d_bytes_per_step counts the arrays passed, not the bytes "
                               "moved",
                       "l2": "no flush: consecutive calls reuse their thread's device copies",
                       "harness": "Python threads, GIL switch interval 10 us"},
            "clocks": ck,
            "e2e": {"value": value, "unit": "sources/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": s_many * 1e3,
                    "host_buffers": "pageable (the caller's arrays), copied through "
                                    "per-thread pinned staging"},
            # per source: forward, adjoint and mask kernels (the grid's
            # precompute runs only when a thread's model changes)
            "gpu_launches": 3 * len(srcs) * args.steps,
            "roofline": {"bound": "fp64", "bound_note": "a call is one solve: the forward "
                         "on a cluster of six blocks (six SMs, one share of the update's cases "
                         "each), the adjoint on one block; achieved = reference-formulation FP64 "
                         "flops of the timed calls over wall time, copies included, against the "
                         "whole GPU's FP64 peak",
                         "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ach / fp64_peak, "traffic": None,
                         "peak_source": "surfatt_measure_peaks (FP64 FMA chains), this run",
                         "kernel": "k_uw_cluster + k_jse_single"},
            "iterations": {"fwd_per_source": its[0] / args.steps / len(srcs),
                           "adj_per_source": its[1] / args.steps / len(srcs)},
            "cpu_baseline": cpu, "parity": parity,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _run_reference_dropin(args, O, dist):
    """Reference arm of the drop-in workload: the oracle's forward, adjoint
    and mask per source, sources split over one process per core (the
    reference's MPI ranks)."""
    import multiprocessing as mp
    nthr = os.cpu_count() or 1
    pb, xx, yy, a, b, c, fun, srcs = _dropin_case()
    _dropin_sadj(srcs, O.gradient_eval(pb, mode=2, nthreads=nthr)["tt_fwd"])
    pool = mp.get_context("spawn").Pool(nthr)
    jobs = [(xx, yy, a, b, c, fun, [srcs[k] for k in blk])
            for blk in _dropin_blocks(len(srcs), nthr)]
    ts = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        pool.map(_oracle_dropin_block, jobs)
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    pool.close()
    pool.join()
    s = statistics.mean(ts)
    v = len(srcs) / s
    line = {"impl": "reference",
            "metric": "drop-in solves/s (forward + adjoint + mask per source through the "
                      "gfortran-mangled symbols, host arrays)",
            "value": v, "unit": "sources/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "config1 through the solver routines: 81x81, 25 sources x "
                                   "24 receivers, 2-D mode", "callers": nthr},
            "cpu_baseline": {"value": v, "unit": "sources/s", "cores": nthr, "kind": "port",
                             "sample": "all 25 sources per step, contiguous blocks over one "
                                       "process per core"},
            "e2e": {"value": v, "unit": "sources/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def _kernel3d_inputs(sg_or_none, O=None):
    """Config 2's model (60 x 60 x 30, 16 periods) with the adj_s /
    adj_density of an FP64 3-D-mode gradient evaluation on the model grid
    (80 stations, forward grid = model grid 60 x 60 at 0.1 deg), from the
    engine (ours) or the oracle (reference arm); seeded stand-ins for the
    surfdisp96 depth kernels."""
    from surfatt_gb300 import workloads as W
    pb = W.config2(n=60, d=0.1, mode=3)
    if sg_or_none is not None:
        eng = sg_or_none.Engine(0)
        r = eng.evaluate(pb, mode=3, precision=sg_or_none.PREC_FP64)
        eng.close()
    else:
        r = O.gradient_eval(pb, mode=3, nthreads=os.cpu_count() or 1)
    P = int(pb.nperiod)
    adj = np.stack([r["adj_s"][int(pb.goff[p]):int(pb.goff[p]) + 3600].reshape((60, 60), order="F")
                    for p in range(P)])
    den = np.stack([r["adj_density"][int(pb.goff[p]):int(pb.goff[p]) + 3600]
                    .reshape((60, 60), order="F") for p in range(P)])
    k = W.kernel3d_case(adj_s=adj, adj_density=den)
    k.chi0 = float(r["chi"])
    return k


KERNEL3D_METRIC = "3-D kernel combination + multigrid projection steps/s (combine_kernels + " \
                  "post_processing_for_kernel)"
KERNEL3D_DESC = ("config 2's model: 60x60x30 nodes, 16 periods, adj_s / adj_density of an FP64 "
                 "gradient evaluation, 5 inversion grids of 8x9x8 (ncomponents 5, n_inv_grid "
                 "[8,9,8]), use_alpha_beta_rho false, kdensity_coe 0")


def _kernel3d_bytes(k):
    """Algorithmic DRAM bytes of one step: combine reads adj_s, adj_density,
    three sensitivity kernels, vs, vp and writes ker, ker_density; the
    post-processing reads ker, writes and reads the scaled kernel, reads and
    writes gradient_s (gk and the tables are L2-sized)."""
    P, nx, ny, nz = k.sen_vs.shape
    N2, N3 = nx * ny, nx * ny * nz
    return 8 * (2 * P * N2 + 3 * P * N3 + 2 * N3 + 2 * N3 + N3 + 2 * N3 + 2 * N3)


def run_kernel3d(args):
    import torch
    import surfatt_gb300 as sg
    dist, rank, world, local = _dist()
    sg.build()
    dev = local
    torch.cuda.set_device(dev)
    k = _kernel3d_inputs(sg)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{dev}")
    # pinned host copies of every input and output of the call
    keep = []

    def pin(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        keep.append(t)
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        return v
    for f in ("adj_s", "adj_density", "sen_vs", "sen_vp", "sen_rho", "vs3d", "vp3d"):
        setattr(k, f, pin(np.asfortranarray(getattr(k, f))))
    out = {n: pin(np.zeros((1, 60, 60, 30), order="F")) for n in ("ker", "ker_density",
                                                                  "gradient_s")}
    for _ in range(args.warmup):
        out["gradient_s"][...] = 0
        sg.kernel_gradient(k, out=out)
    clocks = Clocks(dev)
    _barrier(dist, dev)
    clocks.start()
    kms, walls, launches = [], [], 0
    for _ in range(args.steps):
        _flush_l2(flush)
        out["gradient_s"][...] = 0
        a = time.perf_counter()
        sg.kernel_gradient(k, out=out)
        walls.append(time.perf_counter() - a)
        ms, n = sg.kernel_gradient_timing()
        kms.append(ms)
        launches += n
    _barrier(dist, dev)
    ck = clocks.stop()
    ms_step = _max_over_ranks(dist, statistics.mean(kms), dev)
    e2e_s = _max_over_ranks(dist, statistics.mean(walls), dev)
    algo = _kernel3d_bytes(k)
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
    except Exception:
        peak = 6800.0
    ach = algo / (ms_step * 1e-3) / 1e9
    cpu, parity = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        a = time.perf_counter()
        rk, rkd = O.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                    k.vs3d, k.vp3d)
        rk2, rg = O.post_process_kernels(rk, rkd, 0.0, k.xinv, k.yinv, k.zinv, k.xgrids,
                                         k.ygrids, k.zgrids, k.chi0, k.weight,
                                         np.zeros_like(rk))
        b = time.perf_counter()
        cpu = {"value": 1.0 / (b - a), "unit": "steps/s", "cores": 1, "kind": "port",
               "seconds": b - a,
               "sample": "one full step (the reference runs it on rank 0 alone, "
                         "src/acqui.f90:208, :258)"}
        parity = {"bitwise_equal_vs_oracle": bool(np.array_equal(out["ker"], rk2) and
                                                  np.array_equal(out["ker_density"], rkd) and
                                                  np.array_equal(out["gradient_s"], rg))}
    if rank == 0:
        h2d = sum(getattr(k, f).nbytes for f in ("adj_s", "adj_density", "sen_vs", "sen_vp",
                                                 "sen_rho", "vs3d", "vp3d", "xinv", "yinv",
                                                 "zinv"))
        line = {
            "metric": KERNEL3D_METRIC, "value": world / (ms_step / 1e3), "unit": "steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": KERNEL3D_DESC,
                       "l2": "flushed (256 MB write) between timed steps"},
            "clocks": ck,
            "e2e": {"value": world / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(sum(v.nbytes for v in out.values())),
                    "ms_per_step": e2e_s * 1e3, "host_buffers": "pinned",
                    "call": "surfatt_kernel_gradient"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "traffic": None,
                         "algorithmic_bytes_per_step": algo,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                         "kernel": "k_combine + k_post_prep + k_inv_grid + k_inv2fwd (whole step)",
                         "kernel_ms": ms_step},
            "cpu_baseline": cpu, "parity": parity,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _run_reference_kernel3d(args, O, dist):
    k = _kernel3d_inputs(None, O)
    ts = []
    for i in range(args.warmup + args.steps):
        a = time.perf_counter()
        rk, rkd = O.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                    k.vs3d, k.vp3d)
        O.post_process_kernels(rk, rkd, 0.0, k.xinv, k.yinv, k.zinv, k.xgrids, k.ygrids,
                               k.zgrids, k.chi0, k.weight, np.zeros_like(rk))
        if i >= args.warmup:
            ts.append(time.perf_counter() - a)
    s = statistics.mean(ts)
    line = {"impl": "reference", "metric": KERNEL3D_METRIC, "value": 1.0 / s, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": KERNEL3D_DESC},
            "cpu_baseline": {"value": 1.0 / s, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": "one full step per timed step (rank 0 alone in the "
                                       "reference)"},
            "e2e": {"value": 1.0 / s, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


WORKLIST_METRIC = "work-list builds/s (src_rec table -> solves + receiver gathers)"
WORKLIST_DESC = ("config 2's acquisition as a src_rec table: 80 stations, each an event with "
                 "the other 79 as receivers, 16 periods (101,120 paths, 1,280 solves)")


def _worklist_rows():
    from surfatt_gb300 import workloads as W
    return W.config2_srcrec_rows()


def _oracle_worklist(O, rows):
    return O.srcrec_worklist([r["evtname"] for r in rows], [r["staname"] for r in rows],
                             [r["stla"] for r in rows], [r["stlo"] for r in rows],
                             [r["evla"] for r in rows], [r["evlo"] for r in rows],
                             [r["period"] for r in rows], [r["tt"] for r in rows],
                             [r["weight"] for r in rows])


def run_worklist(args):
    import torch
    import surfatt_gb300 as sg
    dist, rank, world, local = _dist()
    sg.build()
    dev = local
    torch.cuda.set_device(dev)
    rows = _worklist_rows()
    t0 = time.perf_counter()
    tab = sg.SrcRec.from_arrays(*[[r[k] for r in rows] for k in
                                  ("evtname", "staname", "stla", "stlo", "evla", "evlo",
                                   "period", "tt")], weight=[r["weight"] for r in rows])
    index_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{dev}")
    for _ in range(args.warmup):
        tab.build_worklist(dev)
    clocks = Clocks(dev)
    _barrier(dist, dev)
    clocks.start()
    kms, walls, launches = [], [], 0
    for _ in range(args.steps):
        _flush_l2(flush)
        a = time.perf_counter()
        ns = tab.build_worklist(dev)
        walls.append(time.perf_counter() - a)
        ms, n = tab.build_timing()
        kms.append(ms)
        launches += n
    _barrier(dist, dev)
    ck = clocks.stop()
    ms_step = _max_over_ranks(dist, statistics.mean(kms), dev)
    e2e_s = _max_over_ranks(dist, statistics.mean(walls), dev)
    info = tab.info()
    cpu, parity = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        a = time.perf_counter()
        o = _oracle_worklist(O, rows)
        b = time.perf_counter()
        cpu = {"value": 1.0 / (b - a), "unit": "builds/s", "cores": 1, "kind": "port",
               "seconds": b - a,
               "sample": "one full build: get_periods, get_sta, scatter_src_gather and a "
                         "get_evt_gather per solve with the reference's string scans"}
        wl = tab.worklist()
        parity = {"equal_to_oracle": bool(all(np.array_equal(wl[k], o[k]) for k in
                                              ("pidx", "sta", "srcx", "srcy", "rec_off",
                                               "nrec")) and
                                          all(np.array_equal(wl[k], o[k][:len(wl[k])]) for k in
                                              ("recx", "recy", "tt", "weight", "path")))}
    if rank == 0:
        n = info["npath"]
        h2d = n * (3 * 4 + 2 * 8) + info["nsta"] * 16 + info["nperiod"]
        d2h = ns * (4 * 4 + 2 * 8) + n * (4 + 4 * 8)
        line = {
            "metric": WORKLIST_METRIC, "value": world / (ms_step / 1e3), "unit": "builds/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 ids, f64 values", "data": "synthetic",
            "config": {"workload": WORKLIST_DESC, "paths": n, "solves": ns,
                       "stations": info["nsta"], "periods": info["nperiod"],
                       "host_indexing_s": index_s,
                       "l2": "flushed (256 MB write) between timed steps"},
            "clocks": ck,
            "e2e": {"value": world / e2e_s, "unit": "builds/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                    "call": "surfatt_srcrec_build_worklist (device buffers allocated per call)"},
            "gpu_launches": launches,
            "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None,
                         "frac": None, "traffic": None,
                         "note": "five small integer kernels; one block builds the solve order",
                         "kernel": "k_wl_count + k_wl_solves + k_wl_scatter + k_wl_gather",
                         "kernel_ms": ms_step},
            "cpu_baseline": cpu, "parity": parity,
        }
        print(json.dumps(line))
    tab.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _run_reference_worklist(args, O, dist):
    rows = _worklist_rows()
    ts = []
    for i in range(args.warmup + args.steps):
        a = time.perf_counter()
        _oracle_worklist(O, rows)
        if i >= args.warmup:
            ts.append(time.perf_counter() - a)
    s = statistics.mean(ts)
    line = {"impl": "reference", "metric": WORKLIST_METRIC, "value": 1.0 / s, "unit": "builds/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "strings, f64", "data": "synthetic", "config": {"workload": WORKLIST_DESC},
            "cpu_baseline": {"value": 1.0 / s, "unit": "builds/s", "cores": 1, "kind": "port",
                             "sample": "one full build per timed step"},
            "e2e": {"value": 1.0 / s, "unit": "builds/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


TOPO_METRIC = "surface-metric builds/s (get_topo: smoothing + gradient + metric, all periods)"
TOPO_DESC = ("config 5's topography: 150x200 grid at 0.02 deg (Gaussian island 4 km, radius "
             "40 km, 200 m roughness), 15 periods with sigma from 0.04 to 0.4 deg")


def _topo_inputs():
    from surfatt_gb300 import workloads as W
    xx, yy, topo, *_ = W.config5_model()
    return xx, yy, topo, np.geomspace(0.04, 0.4, 15)


def run_topo(args):
    import torch
    import surfatt_gb300 as sg
    dist, rank, world, local = _dist()
    sg.build()
    dev = local
    torch.cuda.set_device(dev)
    xx, yy, topo, sig = _topo_inputs()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{dev}")
    for _ in range(args.warmup):
        sg.topo_metric(topo, xx, yy, sig)
    clocks = Clocks(dev)
    _barrier(dist, dev)
    clocks.start()
    kms, walls, launches = [], [], 0
    for _ in range(args.steps):
        _flush_l2(flush)
        a = time.perf_counter()
        out = sg.topo_metric(topo, xx, yy, sig)
        walls.append(time.perf_counter() - a)
        ms, n = sg.topo_metric_timing()
        kms.append(ms)
        launches += n
    _barrier(dist, dev)
    ck = clocks.stop()
    ms_step = _max_over_ranks(dist, statistics.mean(kms), dev)
    e2e_s = _max_over_ranks(dist, statistics.mean(walls), dev)
    cpu, parity = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        a = time.perf_counter()
        ref = O.topo_metric(topo, xx, yy, sig[:2])
        b = time.perf_counter()
        per_period = (b - a) / 2
        cpu = {"value": 1.0 / (per_period * len(sig)), "unit": "builds/s", "cores": 1,
               "kind": "port", "seconds": b - a,
               "sample": f"2 of the {len(sig)} periods on one core, scaled to all periods "
                         "(the reference spreads periods over MPI ranks, src/grid.f90:106)"}
        worst = 0.0
        for g, r in zip(out, ref):
            for p in range(2):
                worst = max(worst, float(np.max(np.abs(g[p] - r[p])) / np.max(np.abs(r[p]))))
        parity = {"rel_max_vs_oracle_first_two_periods": worst}
    if rank == 0:
        nx, ny = topo.shape
        line = {
            "metric": TOPO_METRIC, "value": world / (ms_step / 1e3), "unit": "builds/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": TOPO_DESC, "periods": len(sig),
                       "l2": "flushed (256 MB write) between timed steps"},
            "clocks": ck,
            "e2e": {"value": world / e2e_s, "unit": "builds/s",
                    "h2d_bytes_per_step": int(topo.nbytes + 8 * (nx + ny + len(sig))),
                    "d2h_bytes_per_step": int(4 * len(sig) * topo.nbytes),
                    "ms_per_step": e2e_s * 1e3, "call": "surfatt_topo_metric"},
            "gpu_launches": launches,
            "roofline": {"bound": "fp64", "achieved": None, "peak": None, "unit": "TFLOP/s",
                         "frac": None, "traffic": None,
                         "note": "dominated by the smoothing (see --workload smooth)",
                         "kernel": "k_smooth_table + k_smooth_apply + k_topo_metric",
                         "kernel_ms": ms_step},
            "cpu_baseline": cpu, "parity": parity,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def _run_reference_topo(args, O, dist):
    xx, yy, topo, sig = _topo_inputs()
    ts = []
    for i in range(args.warmup + args.steps):
        a = time.perf_counter()
        O.topo_metric(topo, xx, yy, sig[:1])
        if i >= args.warmup:
            ts.append((time.perf_counter() - a) * len(sig))
    s = statistics.mean(ts)
    line = {"impl": "reference", "metric": TOPO_METRIC, "value": 1.0 / s, "unit": "builds/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": TOPO_DESC},
            "cpu_baseline": {"value": 1.0 / s, "unit": "builds/s", "cores": 1, "kind": "port",
                             "sample": "one period per timed step on one core, scaled to all "
                                       "periods"},
            "e2e": {"value": 1.0 / s, "unit": "builds/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference Fortran cannot be built (no Fortran compiler); its algorithm "
                    "is timed through the C restatement in oracle/"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "serving":
        run_serving(a)
    elif a.workload == "smooth":
        run_smooth(a)
    elif a.workload == "kernel3d":
        run_kernel3d(a)
    elif a.workload == "worklist":
        run_worklist(a)
    elif a.workload == "topo":
        run_topo(a)
    elif a.workload == "dropin":
        run_dropin(a)
    else:
        run_ours(a)
