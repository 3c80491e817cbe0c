"""Benchmark: batched CCM S-map/simplex predictions per second on GB300.

Workload (one step): convergent cross mapping x -> y on a seeded coupled
logistic map, T = 50000, E = 4, 20 log-spaced library sizes 100..40000, 200
random-library replicates, simplex (k = E+1) and S-map (theta = 2, k = E+2)
-- two fedm_run_command calls, 2 x 20 x 200 x 49997 ~= 4.0e8 forecasts.

  value  forecasts / device time (inputs uploaded, first kernel to statistics)
  e2e    forecasts / wall time of the C ABI calls from host buffers (host
         preparation, splitter, uploads, kernels, downloads)

Also reported: the plain FP64 GPU form and |delta rho| against it on a
2-replicate sample, the roofline of the dominant kernel (the S-map
scan + re-rank + solve kernel, FP64-bound: its FP64 operations, counted by
the kernel, over its CUDA-event time, against this GPU's measured unfused
FP64 multiply/add rate) with the simplex kernel's FP32 figure beside it, and
the CPU oracle on a bounded sample.  `--impl reference` times the CPU
restatement of the reference path (all host threads) instead.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "tests"))
METRIC = "CCM S-map predictions/s: batched FP32+FP64-fix vs plain FP64 GPU @|Δρ|≤1e-6"
# DRAM bytes per S-map prediction point of the S-map kernel
# (knn_one_kernel<4,8,4,1024,1,6>): ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one launch over the 2-replicate x 20-library
# workload (4231.5 MB + 11340.9 MB) divided by its 1 999 880 points.  The
# traffic is the solver's per-thread scratch and spills leaving L1, so it
# scales with the points of a launch.
SMAP_DRAM_BYTES_PER_POINT = 7786.6


def concurrent_calls(fedm, w, a, local, rhos, steps=2):
    """The step's two calls from two host threads on two contexts whose mixed
    kernels share the SMs: the FP64-bound S-map capped at five resident CTAs
    per SM, the FP32-bound simplex at one (fedm_set_ctas_per_sm).  The forms
    are fixed (no autotuning: the two calls would disturb each other's
    probes).  Reports the throughput and whether rho equals the sequential
    run's."""
    saved = os.environ.get("FEDM_AUTOTUNE")
    os.environ["FEDM_AUTOTUNE"] = "0"
    try:
        ctxs = {}
        for alg, cap in (("simplex", 1), ("smap", 5)):
            ctxs[alg] = fedm.Context(local, precision=fedm.PRECISION_MIXED)
            ctxs[alg].set_ctas_per_sm(cap)
    finally:
        if saved is None:
            os.environ.pop("FEDM_AUTOTUNE", None)
        else:
            os.environ["FEDM_AUTOTUNE"] = saved
    calls = {alg: ccm_args(fedm, w, alg, a.reps) for alg in ctxs}

    def step():
        out = {}

        def run(alg):
            out[alg] = ctxs[alg].run_command(calls[alg])

        threads = [threading.Thread(target=run, args=(alg,)) for alg in ctxs]
        t0 = time.perf_counter()
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        dt = time.perf_counter() - t0
        for alg in ctxs:
            if out[alg]["rc"] != 0:
                raise RuntimeError(f"concurrent {alg} call rc={out[alg]['rc']}")
        return dt, out

    for _ in range(3):
        step()
        flush_l2(local)
    times, out = [], None
    for _ in range(steps):
        dt, out = step()
        times.append(dt)
        flush_l2(local)
    preds = sum(ctxs[alg].timing()["predictions"] for alg in ctxs)
    same = all(np.array_equal(np.asarray(out[alg]["stats"]["rho"]), np.asarray(r), equal_nan=True)
               for alg, r in zip(("simplex", "smap"), rhos))
    for c in ctxs.values():
        c.close()
    wall = statistics.mean(times)
    return {"value": preds / wall, "unit": "predictions/s", "wall_ms_per_step": wall * 1e3, "steps": steps,
            "how": "simplex and S-map fedm_run_command calls from two host threads on two contexts, "
                   "CTAs per SM capped at 1 (simplex) and 5 (S-map); wall time of both calls",
            "rho_identical_to_sequential": bool(same)}


def form_kernel(form, alg):
    """The kernel a mixed run used (fedm_timing.mixed_form), for the E = 4, k <= 6 benchmark."""
    return {0: f"knn_mixed_kernel<E=4,C=8,{alg},2 points per thread>",
            1: f"knn_one_kernel<E=4,C=8,{alg},6 CTAs/SM>",
            2: "knn_smap_ws_kernel<E=4,C=8,4 solver warps>",
            3: "knn_smap_ws_kernel<E=4,C=8,8 solver warps>",
            4: f"knn_one_kernel wide form ({alg})",
            5: f"knn_one_kernel<E=4,C=16,{alg},4 CTAs/SM>",
            6: "knn_one_kernel<E=4,C=8,lists> + smap_list_kernel<4> (split S-map)"}.get(int(form), "none")


def hbm_peak():
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]), "MEASURED_PEAKS.json"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback (no MEASURED_PEAKS.json)"


def load_pkg():
    from fedm_loader import fedm, workloads

    return fedm, workloads


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[3:7]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(device):
    import torch

    buf = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    buf.zero_()
    torch.cuda.synchronize(device)
    del buf


def ccm_args(fedm, w, algorithm, reps, libraries=None):
    return fedm.normalise(w["t"], w["x"], w["y"], E=w["E"], library=libraries or w["libraries"], numReps=reps,
                          seed=w["seed"], algorithm=algorithm, theta=2.0 if algorithm == "smap" else 1.0)


def algorithmic_units(w, reps):
    """Pairs and bytes the distance/neighbour step must touch per step."""
    E = w["E"]
    npred = w["n_pred"]
    pairs = 0
    bytes_ = 0
    for L in w["libraries"]:
        pairs += npred * L
        for k in (E + 1, E + 2):
            bytes_ += 4 * E * (L + npred) + 4 * L + 12 * k * npred
    return 2 * reps * pairs, reps * bytes_


def run_ours(a):
    fedm, workloads = load_pkg()
    world, rank, local = dist_setup()
    w = workloads.ccm_config(T=a.T, reps=a.reps, n_libs=a.n_libs, hi=a.lib_max)
    w["n_pred"] = a.T - (w["E"] - 1)
    ctx = fedm.Context(local, precision=fedm.PRECISION_MIXED)
    fp32_peak = ctx.measure_peak(0)
    fp64_unfused_peak = ctx.measure_peak(3)
    fp64_fma_peak = ctx.measure_peak(1)
    calls = [ccm_args(fedm, w, alg, a.reps) for alg in ("simplex", "smap")]

    def step():
        tot = dict(device_ms=0.0, knn_kernel_ms=0.0, knn_launches=0, predictions=0, distance_pairs=0,
                   h2d_bytes=0, d2h_bytes=0, fallback_points=0, kernel_launches=0, fp64_ops=0, host_ms=0.0,
                   list_wait_ms=0.0, setup_ms=0.0, finish_ms=0.0, exact_points=0, autotune_probes=0, prep_ms=0.0,
                   manifold_ms=0.0, wall_ms=0.0)
        base_keys = [k for k in tot if k != "wall_ms"]
        rhos = []
        for args, alg in zip(calls, ("simplex", "smap")):
            t0 = time.perf_counter()
            r = ctx.run_command(args)
            tot["wall_ms"] += (time.perf_counter() - t0) * 1e3
            if r["rc"] != 0:
                raise RuntimeError(f"run_command rc={r['rc']}: {r.get('error')}")
            tm = ctx.timing()
            for k in base_keys:
                tot[k] += tm[k]
            for k in ("knn_kernel_ms", "knn_launches", "fp64_ops", "distance_pairs", "predictions", "mixed_form",
                      "scanned_pairs"):
                tot[f"{alg}_{k}"] = tm[k]
            rhos.append(r["stats"]["rho"])
        return tot, rhos

    warm_probes = 0
    for _ in range(max(3, a.warmup)):
        warm_probes += step()[0]["autotune_probes"]
        flush_l2(local)
    per_step = []
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(a.steps):
            tot, rhos = step()
            per_step.append(tot)
            flush_l2(local)
    barrier(world)
    dev_s = sum(s["device_ms"] for s in per_step) / 1e3
    wall_s = sum(s["wall_ms"] for s in per_step) / 1e3
    preds = sum(s["predictions"] for s in per_step)
    dev_s_max = allreduce_max(world, dev_s)
    wall_s_max = allreduce_max(world, wall_s)
    if rank != 0:
        return
    s0 = per_step[0]
    value = preds * world / dev_s_max
    e2e = preds * world / wall_s_max
    pairs, alg_bytes = algorithmic_units(w, a.reps)
    hbm_gbs, hbm_src = hbm_peak()

    def mean_of(key):
        return statistics.mean(s[key] for s in per_step)

    # dominant kernel: S-map scan + FP64 re-rank + solve (one launch per step
    # plus the exact kernels of its few uncertified points, timed with it)
    sm_ms = mean_of("smap_knn_kernel_ms")
    sm_launches = mean_of("smap_knn_launches")
    sm_ops = mean_of("smap_fp64_ops")
    sm_points = mean_of("smap_predictions")
    sm_fp64 = sm_ops / (sm_ms * 1e-3) / 1e12
    # FP32 scan: the reference's work (every pair, 3 E flops) and the pairs
    # the one-point kernels actually scored (spatially ordered libraries
    # skip tiles that no point can use)
    sm_scanned = mean_of("smap_scanned_pairs")
    sx_scanned = mean_of("simplex_scanned_pairs")
    sm_fp32_alg = 3.0 * w["E"] * pairs / 2 / (sm_ms * 1e-3) / 1e12
    sm_fp32 = 3.0 * w["E"] * sm_scanned / (sm_ms * 1e-3) / 1e12
    traffic = None
    if SMAP_DRAM_BYTES_PER_POINT is not None:
        traffic = SMAP_DRAM_BYTES_PER_POINT * sm_points / sm_launches
    # simplex kernel: FP32 scan + re-rank + forecast
    sx_ms = mean_of("simplex_knn_kernel_ms")
    sx_fp32_alg = 3.0 * w["E"] * pairs / 2 / (sx_ms * 1e-3) / 1e12
    sx_fp32 = 3.0 * w["E"] * sx_scanned / (sx_ms * 1e-3) / 1e12
    knn_ms_step = sm_ms + sx_ms

    # plain FP64 GPU form and |delta rho| on a 2-replicate sample
    fp64 = None
    if not a.no_fp64:
        sample_reps = 2
        ctx64 = fedm.Context(local, precision=fedm.PRECISION_FP64)
        t_fp64 = 0.0
        p_fp64 = 0
        drho = 0.0
        for alg in ("simplex", "smap"):
            args = ccm_args(fedm, w, alg, sample_reps)
            r64 = ctx64.run_command(args)
            tm = ctx64.timing()
            t_fp64 += tm["device_ms"] / 1e3
            p_fp64 += tm["predictions"]
            rmx = ctx.run_command(args)
            drho = max(drho, float(np.max(np.abs(np.asarray(r64["stats"]["rho"]) - np.asarray(rmx["stats"]["rho"])))))
        ctx64.close()
        fp64 = {"value": p_fp64 / t_fp64, "unit": "predictions/s",
                "sample": f"{sample_reps} replicates, both algorithms", "mixed_over_fp64": value / (p_fp64 / t_fp64),
                "max_abs_drho_vs_fp64": drho}

    concurrent = None
    if world == 1 and not a.no_concurrent:
        concurrent = concurrent_calls(fedm, w, a, local, rhos)

    cpu = None
    if world == 1 and not a.no_cpu:
        cpu = cpu_baseline(fedm, w, a)

    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": "predictions/s", "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": dev_s_max / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic (seeded coupled logistic map)",
        "config": {
            "workload": f"ccm_xmap_T{a.T}_E4_L{a.n_libs}x100-{a.lib_max}_reps{a.reps}_simplex+smap",
            "T": a.T, "E": w["E"], "libraries": w["libraries"], "replicates": a.reps,
            "algorithms": ["simplex k=E+1", "smap theta=2 k=E+2"], "predictions_per_step": preds // a.steps,
            "l2": "flushed between steps (512 MiB write)", "parallelism": f"replicas x{world}",
        },
        "e2e": {"value": e2e, "unit": "predictions/s", "h2d_bytes_per_step": int(s0["h2d_bytes"]),
                "d2h_bytes_per_step": int(s0["d2h_bytes"]), "wall_ms_per_step": wall_s_max / a.steps * 1e3,
                "host_ms_per_step": {k: mean_of(k) for k in ("host_ms", "prep_ms", "manifold_ms", "list_wait_ms",
                                                             "setup_ms", "finish_ms")}},
        "gpu_launches": int(sum(s["kernel_launches"] for s in per_step)),
        "roofline": {
            "kernel": form_kernel(s0["smap_mixed_form"], "smap") + " (FP32 scan + FP64 re-rank + JacobiSVD solve)",
            "bound": "fp64_simt", "achieved": sm_fp64, "peak": fp64_unfused_peak, "unit": "TFLOP/s",
            "frac": sm_fp64 / fp64_unfused_peak,
            "peak_source": "measured FP64 multiply+add rate without fusion on this GPU (fedm_measure_peak kind 3; "
                           "the bit-exact solve uses no FMA); MEASURED_PEAKS.json has no FP64 figure",
            "fp64_fma_peak": fp64_fma_peak,
            "algorithmic_fp64_ops_per_launch": sm_ops / sm_launches,
            "fp64_ops_per_forecast": sm_ops / max(sm_points, 1),
            "kernel_ms_per_step": sm_ms, "share_of_device_time": sm_ms / (dev_s_max / a.steps * 1e3),
            "traffic": traffic,
            "fp32_scan": {"achieved": sm_fp32, "peak": fp32_peak, "frac": sm_fp32 / fp32_peak,
                          "flops": "3*E per (prediction, library) pair scored",
                          "scored_fraction_of_pairs": sm_scanned / max(pairs / 2, 1),
                          "algorithmic_achieved": sm_fp32_alg},
            "simplex_kernel": {"kernel": form_kernel(s0["simplex_mixed_form"], "simplex"), "bound": "fp32_simt",
                               "achieved": sx_fp32, "peak": fp32_peak, "frac": sx_fp32 / fp32_peak,
                               "kernel_ms_per_step": sx_ms,
                               "flops": "3*E per (prediction, library) pair scored",
                               "scored_fraction_of_pairs": sx_scanned / max(pairs / 2, 1),
                               "algorithmic_achieved": sx_fp32_alg,
                               "peak_source": "measured FFMA rate of this GPU (fedm_measure_peak kind 0)"},
            "hbm": {"achieved_gbs": alg_bytes / (knn_ms_step * 1e-3) / 1e9, "peak_gbs": hbm_gbs,
                    "frac": alg_bytes / (knn_ms_step * 1e-3) / 1e9 / hbm_gbs, "peak_source": hbm_src},
        },
        "fp64_plain": fp64,
        "concurrent_calls": concurrent,
        "fallback_points_per_step": int(s0["fallback_points"]),
        "exact_points_per_step": int(s0["exact_points"]),
        "autotune": {"smap_form": form_kernel(s0["smap_mixed_form"], "smap"),
                     "simplex_form": form_kernel(s0["simplex_mixed_form"], "simplex"),
                     "probes_during_warmup": warm_probes, "probes_during_timed_steps": int(s0["autotune_probes"])},
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out), flush=True)


def cpu_baseline(fedm, w, a, reps=1, n_libs=None, stride=8):
    """The oracle (CPU restatement of the reference path), all host threads,
    on a bounded sample: the first replicate of every library size (the same
    MT19937-64 library membership), forecasting every `stride`-th prediction
    row, so per-forecast cost matches the full workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import edm_oracle

    cores = os.cpu_count() or 1
    libs = w["libraries"] if n_libs is None else w["libraries"][:n_libs]
    npred = len(range(0, w["n_pred"], stride))
    edm_oracle.set_pred_stride(stride)
    try:
        t0 = time.perf_counter()
        preds = 0
        for alg in ("simplex", "smap"):
            args = edm_oracle.normalise(w["t"], w["x"], w["y"], E=w["E"], library=libs, numReps=reps,
                                        seed=w["seed"], algorithm=alg, theta=2.0 if alg == "smap" else 1.0,
                                        numThreads=cores)
            r = edm_oracle.run_command(args)
            if r["rc"] != 0:
                raise RuntimeError(f"oracle rc={r['rc']}")
            preds += len(r["stats"]["rho"]) * npred
        dt = time.perf_counter() - t0
    finally:
        edm_oracle.set_pred_stride(1)
    return {"value": preds / dt, "unit": "predictions/s", "cores": cores, "kind": "port",
            "sample": f"{reps} replicate x {len(libs)} library sizes, simplex + smap, every {stride}th prediction "
                      f"row ({preds} forecasts, {dt:.1f} s)"}


# Other benchmark configurations at full size (--workload).  Each step runs
# the configuration through the library's C ABI from host buffers; `value`
# is forecasts per second of device time, `e2e` per second of wall time.
# They are measurements of the parity-test configurations, not the headline.
# Each line carries the roofline of the configuration's dominant kernel
# (algorithmic work per launch over its CUDA-event time, against this GPU's
# measured rate for the pipe that bounds it) and the oracle on a bounded
# sample of the same workload.
def config_steps(fedm, workloads, ctx, name):
    """Returns (description, step function -> list of (timing dict, wall s),
    CPU-sample function -> (forecasts, seconds, description))."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import edm_oracle

    cores = os.cpu_count() or 1
    if name == "simplex_explore":
        w = workloads.simplex_config()
        args = {E: fedm.normalise(w["t"], w["x"], E=E, theta=1.0) for E in w["Es"]}

        def step():
            out = []
            for E in w["Es"]:
                t0 = time.perf_counter()
                ctx.run_task(args[E], w["library_rows"], w["prediction_rows"], E, E + 1)
                out.append((ctx.timing(), time.perf_counter() - t0))
            return out

        def cpu():
            t0 = time.perf_counter()
            n = 0
            for E in w["Es"]:
                o = edm_oracle.oracle_task(edm_oracle.normalise(w["t"], w["x"], E=E, theta=1.0, numThreads=cores),
                                           w["library_rows"], w["prediction_rows"], E, E + 1)
                n += o["n_pred"]
            return n, time.perf_counter() - t0, "the whole workload (E = 1..10)"
        return {"workload": "simplex_T500_lib250_pred250_E1-10_k=E+1", "T": 500}, step, cpu
    if name == "smap_sweep":
        # edm()'s explore split of 20 000 rows: the first 9 998 usable rows
        # are the library, the other 9 998 the prediction set
        w = workloads.smap_config()
        kw = dict(E=w["E"], theta=w["thetas"], algorithm="smap", k=float("inf"))
        a_ = fedm.normalise(w["t"], w["x"], **kw)

        def step():
            t0 = time.perf_counter()
            ctx.run_command(a_)
            return [(ctx.timing(), time.perf_counter() - t0)]

        def cpu(stride=97):
            edm_oracle.set_pred_stride(stride)
            try:
                t0 = time.perf_counter()
                edm_oracle.oracle_edm(w["t"], w["x"], numThreads=cores, **kw)
                dt = time.perf_counter() - t0
            finally:
                edm_oracle.set_pred_stride(1)
            n = len(range(0, 9998, stride)) * len(w["thetas"])
            return n, dt, f"every {stride}th prediction row, all 81 thetas"
        return {"workload": "smap_kall_lib9998_pred9998_E5_theta0-8x81", "T": 20000}, step, cpu
    if name in ("panels", "panels_independent", "panels_penalty"):
        # independent panels (panelWeight = Inf) and penalised ones
        # (panelWeight = 0.1) are timed with two-fold cross-validation over
        # shuffled folds, so that every panel has library rows: edm()'s
        # default split (and unshuffled folds) give the library whole
        # panels, and almost no prediction panel a neighbour of its own
        w = workloads.panel_config()
        pw = {"panels": 0.0, "panels_independent": float("inf"), "panels_penalty": 0.1}[name]
        extra = dict(crossfold=2, shuffle=True, seed=1) if pw else {}
        kws = [dict(panel=w["panel"], E=[3, 4, 5, 6, 7, 8], dt=True, algorithm="simplex", panelWeight=pw, **extra),
               dict(panel=w["panel"], E=[3, 4, 5, 6, 7, 8], dt=True, algorithm="smap", theta=[0.0, 1.0, 2.0, 4.0],
                    panelWeight=pw, **extra)]

        def step():
            out = []
            for kw in kws:
                t0 = time.perf_counter()
                fedm.edm(w["t"], w["x"], ctx=ctx, **kw)
                out.append((ctx.timing(), time.perf_counter() - t0))
            return out

        def cpu(stride=50 if pw == float("inf") else 1000):
            edm_oracle.set_pred_stride(stride)
            n = 0
            try:
                t0 = time.perf_counter()
                for kw in kws:
                    r = edm_oracle.oracle_edm(w["t"], w["x"], numThreads=cores, **kw)
                    n += len(r["stats"]["rho"])
                dt = time.perf_counter() - t0
            finally:
                edm_oracle.set_pred_stride(1)
            n_pred = int(fedm.host_plan(fedm.normalise(w["t"], w["x"], **kws[0]))["pred"][0].sum())
            return n * len(range(0, n_pred, stride)), dt, f"every {stride}th prediction row, every E and theta"
        mode = {"panels": "mixed_library", "panels_independent": "independent_panels_crossfold2_shuffled",
                "panels_penalty": "penalty0.1_crossfold2_shuffled"}[name]
        return {"workload": f"panels512_rows{len(w['t'])}_E3-8_dt_simplex+smap4theta_{mode}",
                "rows": len(w["t"]), "panelWeight": "Inf" if pw == float("inf") else pw}, step, cpu
    if name == "easy_edm":
        # easy_edm()'s default (quantile) workflow, R/easy_edm.R:40-433, on a
        # coupled logistic pair of T = 5000: E search 3..10; a 101-theta
        # S-map with k = Inf; S-maps with k = 20 at theta = 0 and at the best
        # theta, 20 replicates each; a lag scan of 12 cross maps (simplex,
        # k = Inf); the max-library call with saveManifolds; 1000 replicates
        # at a tenth of the max library and one at the max library
        # (simplex, k = Inf, shuffle).  One step is the whole sequence.
        t, x, y = workloads.coupled_logistic(5000, seed=21)

        def tslag(v, lag):
            out = np.full(len(v), np.nan)
            if lag >= 0:
                out[lag:] = v[:len(v) - lag]
            else:
                out[:lag] = v[-lag:]
            return out

        def seq_calls():
            r = yield dict(args=(t, x), kw=dict(E=list(range(3, 11))))
            E = int(r["stats"]["E"][int(np.nanargmax(r["stats"]["rho"]))])
            r = yield dict(args=(t, x), kw=dict(E=E, theta=list(np.linspace(0, 5, 101)), algorithm="smap",
                                                 k=float("inf")))
            th = float(r["stats"]["theta"][int(np.nanargmax(r["stats"]["rho"]))])
            yield dict(args=(t, x), kw=dict(E=E, theta=0.0, numReps=20, k=20, algorithm="smap"))
            yield dict(args=(t, x), kw=dict(E=E, theta=th, numReps=20, k=20, algorithm="smap"))
            for lag in range(-5, 7):
                yield dict(args=(t, x, tslag(y, lag)), kw=dict(E=E, theta=th, algorithm="simplex", k=float("inf")))
            r = yield dict(args=(t, y), kw=dict(E=E, algorithm="simplex", full=True, saveManifolds=True))
            lib_max = r["Ms"][0].shape[0]
            small = max(E + 2, lib_max // 10)
            yield dict(args=(t, y, x), kw=dict(E=E, library=small, numReps=1000, theta=th, algorithm="simplex",
                                                k=float("inf"), shuffle=True))
            yield dict(args=(t, y, x), kw=dict(E=E, library=lib_max, theta=th, algorithm="simplex",
                                                k=float("inf"), shuffle=True))

        def step():
            out = []
            gen = seq_calls()
            call = next(gen)
            while True:
                t0 = time.perf_counter()
                r = fedm.edm(*call["args"], ctx=ctx, **call["kw"])
                if r["rc"] != 0:
                    raise RuntimeError(f"easy_edm call rc={r['rc']}")
                out.append((ctx.timing(), time.perf_counter() - t0))
                try:
                    call = gen.send(r)
                except StopIteration:
                    return out

        def cpu():
            # the sequence's calls on the oracle, the 1000-replicate call cut
            # to 20 replicates, every 10th prediction row
            edm_oracle.set_pred_stride(10)
            n = 0
            try:
                t0 = time.perf_counter()
                gen = seq_calls()
                call = next(gen)
                while True:
                    kw = dict(call["kw"])
                    if kw.get("numReps") == 1000:
                        kw["numReps"] = 20
                    r = edm_oracle.oracle_edm(*call["args"], numThreads=cores, **kw)
                    if "Ms" not in r and kw.get("saveManifolds"):
                        r["Ms"] = [np.zeros((len(t) - kw["E"], kw["E"]))]  # the oracle keeps no manifolds
                    # prediction rows: half the usable rows when exploring,
                    # all of them for cross maps and full
                    half = len(call["args"]) == 2 and not kw.get("full")
                    E = max(np.atleast_1d(kw["E"]))
                    n_pred = (len(t) - E if not half else (len(t) - E) // 2)
                    n += len(r["stats"]["rho"]) * ((n_pred + 9) // 10)
                    try:
                        call = gen.send(r)
                    except StopIteration:
                        break
                dt = time.perf_counter() - t0
            finally:
                edm_oracle.set_pred_stride(1)
            return n, dt, "the sequence with 20 instead of 1000 replicates, every 10th prediction row"
        return {"workload": "easy_edm_quantile_T5000_Esearch3-10_theta101_reps20_lags12_ccm1000", "T": 5000}, step, cpu
    if name == "adjoint":
        w = workloads.lorenz_config()
        a_ = fedm.normalise(w["t"], w["x"], E=6, tau=5)
        F = fedm.host_manifold(a_, 6)
        first = 5 * 5
        lib_rows = np.arange(first, first + 50000)
        pred_rows = np.arange(first + 50000, first + 70000)
        lib, lib_t = F[lib_rows], w["x"][lib_rows + 1]
        pred, pred_t = F[pred_rows], w["x"][pred_rows + 1]

        def step():
            t0 = time.perf_counter()
            ctx.smap_grad(lib, lib_t, pred, pred_t, 1.0, np.ones(6))
            tm = ctx.timing()
            tm = dict(tm, predictions=len(pred_rows))
            return [(tm, time.perf_counter() - t0)]

        def cpu(n=200):
            t0 = time.perf_counter()
            edm_oracle.smap_grad(lib, lib_t, pred[:n], pred_t[:n], 1.0, np.ones(6))
            return n, time.perf_counter() - t0, f"the first {n} prediction points, forward and backward, 1 thread"
        return {"workload": "lorenz_smap_grad_kall_lib50000_pred20000_E6_tau5", "T": 100000}, step, cpu
    if name == "wasserstein":
        # the Wasserstein distance (src/distances.cpp:270-527) through the
        # task seam: a coupled logistic series, E = 5 (5 x 5 transport
        # problems), library the first 2 000 rows, predictions the last
        # 2 000; simplex k = 6 and S-map k = 7
        t, x, _ = workloads.coupled_logistic(4000, seed=61)
        E = 5
        lib = np.zeros(4000, bool)
        lib[:2000] = True
        pred = ~lib
        calls = [(fedm.normalise(t, x, E=E, theta=1.0), E + 1),
                 (fedm.normalise(t, x, E=E, theta=1.0, algorithm="smap"), E + 2)]

        def step():
            out = []
            for a_, k in calls:
                t0 = time.perf_counter()
                ctx.run_task(a_, lib, pred, E, k, distance=2)
                out.append((ctx.timing(), time.perf_counter() - t0))
            return out

        def cpu(stride=1):
            sub_pred = np.zeros_like(pred)
            sub_pred[np.flatnonzero(pred)[::stride]] = True
            t0 = time.perf_counter()
            n = 0
            for alg, k in (("simplex", E + 1), ("smap", E + 2)):
                o = edm_oracle.oracle_task(edm_oracle.normalise(t, x, E=E, theta=1.0, algorithm=alg,
                                                                numThreads=cores), lib, sub_pred, E, k, distance=2)
                n += o["n_pred"]
            return n, time.perf_counter() - t0, ("every prediction row, both calls" if stride == 1 else
                                                 f"every {stride}th prediction row, both calls")
        return {"workload": "wasserstein_T4000_lib2000_pred2000_E5_simplex_k6+smap_k7", "T": 4000}, step, cpu
    raise ValueError(name)


# FP64 instructions per (prediction, library) pair of the Wasserstein
# neighbour kernel at E = 5 (ncu, profiles/knn_exact_kernel_wasserstein_E5.md)
WASS_FP64_PER_PAIR = 1006.6


def config_roofline(name, precision, steps_tm, peaks):
    """Roofline of a configuration's dominant kernel from the timings of one
    step (a list of per-call timing dicts)."""
    def tot(key):
        return sum(tm[key] for tm in steps_tm)

    if name == "simplex_explore":
        # rows 0..E-2 of the explicit library lack lags, which keeps the
        # tasks on the exact FP64 scan (3 E_a FP64 operations per pair,
        # unfused) unless a mixed form reports it served them
        ms = tot("knn_kernel_ms")
        flops = tot("scan_flops")
        mixed = any(tm["mixed_form"] >= 0 for tm in steps_tm)
        peak = peaks["fp32"] if mixed else peaks["fp64_unfused"]
        return {"kernel": "knn_one_kernel (FP32 scan + FP64 re-rank)" if mixed else
                          "knn_exact_kernel (FP64 distances + exact top-k)",
                "bound": "fp32_simt" if mixed else "fp64_simt",
                "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                "frac": flops / (ms * 1e-3) / 1e12 / peak, "traffic": None,
                "kernel_ms_per_step": ms, "launches_per_step": tot("knn_launches"),
                "work": "3 E_actual operations per (prediction, library) pair",
                "peak_source": "measured FFMA rate (fedm_measure_peak kind 0)" if mixed else
                               "measured unfused FP64 multiply/add rate (fedm_measure_peak kind 3)"}
    if name == "smap_sweep":
        tm = steps_tm[0]
        ms = tm["forecast_kernel_ms"]
        E, n_th = 5, 81
        n = E + 1
        flops = 2.0 * tm["distance_pairs"] * n_th * (n * (n + 1) / 2 + n)
        fast = precision == "fast"
        peak = peaks["fp32"] if fast else peaks["fp64_unfused"]
        if fast and tm.get("tensor_core_tiles", 0) > 0:
            # the tensor-core pass computes 15 bf16 slice products of the
            # 32-column padded GEMM: 15 x 2 N_p Theta N_L 32 tensor flops
            tflops = 15 * 2.0 * tm["distance_pairs"] * n_th * 32
            return {"kernel": "all_df_prep_kernel + gram_tc_kernel (tcgen05, bf16 slices, FP32 in TMEM) + "
                              "all_smap_gram_kernel<5> (FP64 JacobiSVD)",
                    "bound": "tensor", "achieved": tflops / (ms * 1e-3) / 1e12, "peak": peaks["bf16"],
                    "unit": "TFLOP/s", "frac": tflops / (ms * 1e-3) / 1e12 / peaks["bf16"], "traffic": None,
                    "kernel_ms_per_step": ms, "launches_per_step": tm["forecast_launches"],
                    "tensor_core_tiles": tm["tensor_core_tiles"],
                    "work": "15 slice products x 2 N_p Theta N_L x 32 (padded) columns of bf16 tensor flops over "
                            "the prep, tensor-core and solve kernels' time",
                    "peak_source": peaks["bf16_source"],
                    "algorithmic_fp64_equivalent": {"achieved": flops / (ms * 1e-3) / 1e12, "flops": flops}}
        return {"kernel": ("all_df_prep_kernel + all_smap_df_kernel<5> (FP32 weights, double-float normal "
                           "equations)") if fast else "all_smap_kernel<5> (FP64 weights and normal equations)",
                "bound": "fp32_simt" if fast else "fp64_simt", "achieved": flops / (ms * 1e-3) / 1e12,
                "peak": peak, "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / 1e12 / peak, "traffic": None,
                "kernel_ms_per_step": ms, "launches_per_step": tm["forecast_launches"],
                "work": "2 N_p Theta N_L ((E_a+1)(E_a+2)/2 + E_a+1) flops of the weighted normal equations",
                "peak_source": ("measured FFMA rate (fedm_measure_peak kind 0); each double-float multiply-add "
                                "takes ~11 FP32 instructions") if fast else
                               "measured unfused FP64 multiply/add rate (fedm_measure_peak kind 3)"}
    if name in ("panels", "panels_independent", "panels_penalty"):
        # two pipes share the kernel: the FP32 scan and the FP64 re-rank and
        # S-map solves (up to 17 x 17 Jacobi SVDs at E = 8 with dt); the
        # bound is the one with the larger fraction, the other is given beside
        ms = tot("knn_kernel_ms")
        flops = tot("scan_flops")
        ops = tot("fp64_ops")
        fp32 = {"achieved": flops / (ms * 1e-3) / 1e12, "peak": peaks["fp32"],
                "frac": flops / (ms * 1e-3) / 1e12 / peaks["fp32"],
                "work": "3 E_actual FP32 flops per (prediction, library) pair scanned" +
                        (" (own-panel pairs only)" if name == "panels_independent" else ""),
                "peak_source": "measured FFMA rate (fedm_measure_peak kind 0)"}
        fp64 = {"achieved": ops / (ms * 1e-3) / 1e12, "peak": peaks["fp64_unfused"],
                "frac": ops / (ms * 1e-3) / 1e12 / peaks["fp64_unfused"],
                "work": "FP64 operations of the re-rank and forecasts, counted by the kernels",
                "peak_source": "measured unfused FP64 multiply/add rate (fedm_measure_peak kind 3)"}
        main, other, bound = (fp64, fp32, "fp64_simt") if fp64["frac"] >= fp32["frac"] else (fp32, fp64, "fp32_simt")
        return {"kernel": "knn_one_kernel (one point per thread; wide form for E_a 10..16) + re-rank + forecast",
                "bound": bound, "achieved": main["achieved"], "peak": main["peak"], "unit": "TFLOP/s",
                "frac": main["frac"], "traffic": None, "kernel_ms_per_step": ms,
                "launches_per_step": tot("knn_launches"), "work": main["work"], "peak_source": main["peak_source"],
                "fp32" if bound == "fp64_simt" else "fp64": other}
    if name == "easy_edm":
        # the sequence mixes the exact FP64 neighbour search (k = 20), the
        # mixed scan and the k = all forecasts; the figure is the FP64
        # distance work (3 E_a per pair) over the neighbour and forecast
        # kernels' time
        ms = tot("knn_kernel_ms") + tot("forecast_kernel_ms")
        flops = tot("scan_flops")
        return {"kernel": "neighbour search + k = all forecast kernels over the sequence's 20 calls",
                "bound": "fp64_simt", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peaks["fp64_unfused"],
                "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / 1e12 / peaks["fp64_unfused"], "traffic": None,
                "kernel_ms_per_step": ms, "launches_per_step": tot("knn_launches") + tot("forecast_launches"),
                "work": "3 E_actual operations per (prediction, library) pair scanned",
                "peak_source": "measured unfused FP64 multiply/add rate (fedm_measure_peak kind 3)",
                "per_call_ms": [{"device": tm["device_ms"], "host": tm["host_ms"], "prep": tm["prep_ms"],
                                 "manifold": tm["manifold_ms"], "setup": tm["setup_ms"],
                                 "finish": tm["finish_ms"]} for tm in steps_tm]}
    if name == "wasserstein":
        # combinatorial work: the cost matrix (3 operations per entry) and the
        # transport solver's shortest-path rounds; its FP64 instructions per
        # (prediction, library) pair were counted once by ncu on this workload
        # (sm__sass_thread_inst_executed_op_fp64_pred_on over the neighbour
        # kernel's pairs) and are the work unit here
        ms = tot("knn_kernel_ms")
        pairs = tot("distance_pairs")
        if WASS_FP64_PER_PAIR is None:
            return None
        ops = WASS_FP64_PER_PAIR * pairs
        return {"kernel": "knn_exact_kernel<Wasserstein> (cost matrix + successive-shortest-path transport per pair)",
                "bound": "fp64_simt", "achieved": ops / (ms * 1e-3) / 1e12, "peak": peaks["fp64_unfused"],
                "unit": "TFLOP/s", "frac": ops / (ms * 1e-3) / 1e12 / peaks["fp64_unfused"], "traffic": None,
                "kernel_ms_per_step": ms, "launches_per_step": tot("knn_launches"),
                "pairs_per_s": pairs / (ms * 1e-3),
                "work": f"{WASS_FP64_PER_PAIR} FP64 instructions per (prediction, library) pair (ncu count)",
                "peak_source": "measured unfused FP64 multiply/add rate (fedm_measure_peak kind 3)"}
    if name == "adjoint":
        tm = steps_tm[0]
        ms = tm["knn_kernel_ms"]
        E = 6
        n = E + 1
        per_pair = 2 * (n * (n + 1) / 2 + n) + 2 * (3 * E + 1) + 4 * n
        flops = per_pair * 50000 * tm["predictions"]
        return {"kernel": "smap_grad_kernel<6> (three passes per point: distances, normal equations, adjoint sums; "
                          "per-row values cached per warp)",
                "bound": "fp64_simt", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peaks["fp64_fma"],
                "unit": "TFLOP/s", "frac": flops / (ms * 1e-3) / 1e12 / peaks["fp64_fma"], "traffic": None,
                "kernel_ms_per_step": ms, "launches_per_step": 2,
                "work": f"{per_pair:.0f} flops per (prediction, library row): the normal equations "
                        "2((E+1)(E+2)/2 + E+1), the adjoint sums 2(3E+1) and the residual and g.u products 4(E+1)",
                "peak_source": "measured DFMA rate (fedm_measure_peak kind 1): the adjoint passes use FMA"}
    return None


def run_config(a):
    fedm, workloads = load_pkg()
    world, rank, local = dist_setup()
    ctx = fedm.Context(local, precision={"mixed": fedm.PRECISION_MIXED, "fast": fedm.PRECISION_FAST}[a.precision])
    peaks = {"fp32": ctx.measure_peak(0), "fp64_fma": ctx.measure_peak(1), "fp64_unfused": ctx.measure_peak(3)}
    try:
        peaks["bf16"] = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"])
        peaks["bf16_source"] = "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM, burst), of measured"
    except (OSError, ValueError, KeyError):
        peaks["bf16"] = 1900.0
        peaks["bf16_source"] = "fallback 1.9 PFLOP/s bf16"
    cfg, step, cpu = config_steps(fedm, workloads, ctx, a.workload)
    for _ in range(max(3, a.warmup)):
        step()
        flush_l2(local)
    barrier(world)
    dev = wall = 0.0
    preds = launches = fallback = exact = 0
    host = {k: 0.0 for k in ("host_ms", "prep_ms", "manifold_ms", "list_wait_ms", "setup_ms", "finish_ms")}
    step_tms = []
    with Clocks(local) as clk:
        for _ in range(a.steps):
            tms = step()
            step_tms.append([tm for tm, _ in tms])
            for tm, ws in tms:
                dev += tm["device_ms"] / 1e3
                wall += ws
                preds += tm["predictions"]
                launches += tm["kernel_launches"]
                fallback += tm.get("fallback_points", 0)
                exact += tm.get("exact_points", 0)
                for k in host:
                    host[k] += tm.get(k, 0.0)
            flush_l2(local)
    dev = allreduce_max(world, dev)
    wall = allreduce_max(world, wall)
    if rank != 0:
        return
    roof = config_roofline(a.workload, a.precision, step_tms[-1], peaks)
    if roof is not None:
        roof["share_of_device_time"] = roof["kernel_ms_per_step"] / (dev / a.steps * 1e3)
    cpu_line = None
    if world == 1 and not a.no_cpu:
        n, dt, what = cpu()
        cpu_line = {"value": n / dt, "unit": "predictions/s", "cores": os.cpu_count() or 1, "kind": "port",
                    "sample": f"{what} ({n} forecasts, {dt:.1f} s)"}
        if a.workload == "adjoint":
            cpu_line["cores"] = 1
    cfg["l2"] = "flushed between steps (512 MiB write)"
    cfg["parallelism"] = f"replicas x{world}"
    out = {
        "metric": f"{a.workload} predictions/s (full-size configuration, {a.precision} precision path)", "value":
        preds * world / dev, "unit": "predictions/s", "n_gpus": world, "steps": a.steps, "warmup": max(3, a.warmup),
        "ms_per_step": dev / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32+fp64", "data": "synthetic (seeded generators)", "config": cfg,
        "e2e": {"value": preds * world / wall, "unit": "predictions/s", "wall_ms_per_step": wall / a.steps * 1e3,
                "host_ms_per_step": {k: v / a.steps for k, v in host.items()}},
        "gpu_launches": launches, "predictions_per_step": preds // a.steps,
        "fallback_points_per_step": fallback // a.steps, "exact_points_per_step": exact // a.steps,
        "roofline": roof, "cpu_baseline": cpu_line,
        "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)


def run_reference(a):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    _, workloads = load_pkg()
    w = workloads.ccm_config(T=a.T, reps=a.reps, n_libs=a.n_libs, hi=a.lib_max)
    w["n_pred"] = a.T - (w["E"] - 1)
    for _ in range(max(3, a.warmup)):
        cpu_baseline(None, w, a, reps=1, n_libs=a.ref_libs)
    vals = []
    last = None
    for _ in range(a.steps):
        last = cpu_baseline(None, w, a, reps=1, n_libs=a.ref_libs)
        vals.append(last["value"])
    v = statistics.mean(vals)
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "predictions/s", "n_gpus": world,
        "steps": a.steps, "warmup": max(3, a.warmup), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded coupled logistic map)",
        "config": {"workload": f"ccm_xmap_T{a.T}_E4_L{a.n_libs}x100-{a.lib_max}_reps{a.reps}_simplex+smap",
                   "T": a.T, "E": w["E"], "libraries": w["libraries"], "replicates": a.reps,
                   "sample_per_step": last["sample"]},
        "cpu_baseline": {"value": v, "unit": "predictions/s", "cores": last["cores"], "kind": "port",
                         "sample": last["sample"]},
        "e2e": {"value": v, "unit": "predictions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--T", type=int, default=50000)
    ap.add_argument("--reps", type=int, default=200)
    ap.add_argument("--n-libs", dest="n_libs", type=int, default=20)
    ap.add_argument("--lib-max", dest="lib_max", type=int, default=40000)
    ap.add_argument("--ref-libs", dest="ref_libs", type=int, default=None,
                    help="library sizes in each CPU reference sample (default: all)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-concurrent", dest="no_concurrent", action="store_true",
                    help="skip the concurrent two-context measurement of the headline workload")
    ap.add_argument("--no-fp64", dest="no_fp64", action="store_true",
                    help="skip the plain FP64 sample (profiling runs)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fast"],
                    help="context precision for the non-headline workloads: mixed (bit-exact) or fast (FP32 "
                         "weights and double-float normal equations for the k = all S-map)")
    ap.add_argument("--workload", default="ccm",
                    choices=["ccm", "simplex_explore", "smap_sweep", "panels", "panels_independent",
                             "panels_penalty", "adjoint", "easy_edm", "wasserstein"],
                    help="ccm (default): the headline CCM benchmark; the others time the other benchmark "
                         "configurations at full size")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload != "ccm":
        run_config(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
