#!/usr/bin/env python3
"""Benchmark: fitted tracks/s of the GB300 Kalman fitter.

Headline workload (FP64 fit at scale): 1M tracks per GPU through the 10-plane
telescope (x = 100..1000 mm, normal +x, no material) in a uniform 2 T field;
pi+- with |p| in [1, 10] GeV, phi in +-0.1, theta in pi/2 +- 0.1; 50 um hits;
seeds smeared by 50 um / 1 mrad / 5 %.  Synthetic, seeded, generated on the
host.  One step = one fit of the whole batch: in the batched form (default)
one CUDA-graph launch (work-queue sort + persistent fit kernel, shape picked
by the autotuner beforehand), in the plain form one grid kernel launch.  The
line carries both forms on the same batch ("forms"), and a suite of one-GPU
comparisons: 4M uneven tracks with holes and outliers on 30 planes, 1M tracks
on 30 planes in the FP32 field map (plain FP64 against batched FP64 and
batched mixed precision), the chi2 adjoint (gradients with respect to plane
alignment, start parameters and field scale) on 256k tracks of a misaligned
20-plane telescope against one forward fit of the same batch, 1M tracks
through 0.5 mm of silicon per plane (material effects), the output writers
(params CSV, states obj, params table) on 256k fitted tracks, and input
production: 4M uneven tracks simulated on the GPU against the host generator.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--form batched|plain] [--workload W] [--precision fp64|mixed]
                  [--tracks N] [--no-suite] [--no-e2e] [--no-cpu-baseline]

The reference arm (--impl reference) times the reference algorithm's CPU
path (the C++ FP64 restatement in oracle/, OpenMP over all host cores, the
reference's -d cpu loop shape) on the same workload, config and track count
as the GPU arm; its inputs come from the oracle library's copy of the host
generator, so that arm never loads the product library.  With --gpus N the
GPU arm splits one global batch of N x tracks over the ranks
(gpukalmanfitter_gb300.shard); the reference arm runs on rank 0 alone.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fitted tracks/s on 1 GB300, plain vs batched form at equal accuracy; grads/s"
UNIT = "tracks/s"
OVERSTEP = 0.1  # mm; the reference's fixed 0.01 mm skips planes on this workload
SINGLE_THREAD_SAMPLE = 20_000  # tracks of the one-thread CPU leg (about 0.4 s a step)
DATA = "synthetic (seeded generator, analytic-helix truth)"

# workload name -> (description, make_telescope keyword arguments, fit config extras)
WORKLOADS = {
    "uniform10": ("telescope of 10 planes x=100..1000 mm, uniform 2 T, pi+- |p| 1-10 GeV, "
                  "50 um hits, seeds 50 um/1 mrad/5 %", {}, {}),
    "map30": ("telescope of 30 planes x=50..1500 mm, 101^3 FP32 field map over +-1.5 m "
              "(Bz = 2 T (1 - 0.2 (r/1.5 m)^2) exp(-(z/3 m)^2), Br from div B = 0), trilinear",
              dict(n_planes=30, x_first=50., x_step=50., field_map=True), {}),
    "holes30": ("telescope of 30 planes x=50..1500 mm, uniform 2 T, path length U{5..30} planes, "
                "hit probability 0.9, 2 % outliers shifted U(+-5 mm), outlier chi2 cut 25",
                dict(n_planes=30, x_first=50., x_step=50., min_len=5, max_len=30, hit_prob=0.9,
                     outlier_prob=0.02), dict(outlier_chi2_cut=25.0)),
    "material10": ("telescope of 10 planes x=100..1000 mm, uniform 2 T, 0.5 mm silicon per plane "
                   "(Highland scattering, Bethe loss, Landau width in the fit and in the truth)",
                   dict(material=0.5), dict(material_effects=3)),
}
PRECISIONS = {"fp64": 0, "mixed": 1}
# chi2 adjoint workload: truth planes misaligned, the fit uses the nominal geometry
ALIGN20 = ("telescope of 20 planes x=50..1000 mm, uniform 2 T, truth planes misaligned by "
           "N(0, 100 um) shifts and N(0, 1 mrad) rotations (nominal geometry in the fit)",
           dict(n_planes=20, x_first=50., x_step=50., mis_shift=0.1, mis_rot=1e-3))


def workload_config(name: str, n_tracks: int, precision: str) -> dict:
    desc, kw, _ = WORKLOADS[name]
    return {"workload": f"{name}: {desc}", "tracks_per_gpu": n_tracks,
            "precision": precision, "overstep_limit_mm": OVERSTEP, "rk_tolerance": 1e-4,
            "mass_in_fit": "muon (reference default)",
            "l2": "inputs larger than the 129 MB L2 at 1M tracks"}


def make_workload(kf, name: str, n: int, seed: int, lib=None):
    """The named workload (host arrays).  lib: the library whose host
    generator makes it (the oracle's for the reference arm, so that arm never
    maps the product library; both carry the same generator code)."""
    return kf.make_telescope(n, seed=seed, lib=lib, **WORKLOADS[name][1])


def fit_config(kf, name: str, precision: str):
    return kf.default_config(overstep_limit=OVERSTEP, precision=PRECISIONS[precision],
                             **WORKLOADS[name][2])


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ---------------------------------------------------------------------------
def cpu_oracle_rate(tel, cfg, reps: int, warmup: int, threads: int = 0) -> dict:
    """The reference algorithm's CPU path (the oracle, OpenMP over the track
    loop as the reference's -d cpu driver runs it) on the tracks of `tel`:
    wall clock around the track loop alone, median over `reps` steps.
    threads = 0: every host thread OpenMP offers."""
    import oracle
    fitter = oracle.Fitter(tel, cfg)
    threads = threads or int(fitter.lib.oracle_num_threads())
    for _ in range(warmup):
        fitter.run(threads)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fitter.run(threads)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    ok = float(np.mean(fitter.out["status"] == 0))
    return {"value": tel.n / med, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"all {tel.n} tracks of the workload per step, median of {reps} timed steps "
                      f"({warmup} warm-up), wall clock around the OpenMP track loop",
            "seconds_per_step": med, "seconds": times, "fitted_fraction": ok}


def run_reference(args) -> None:
    """The reference arm: the reference algorithm's CPU path on the host
    cores, on the GPU arm's workload, config and track count.  Inputs come
    from the oracle library's copy of the host generator and the fit from the
    oracle: the product library is never loaded here."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import gpukalmanfitter_gb300 as kf  # Python helpers only (structs, array layout)
    import oracle
    lib = oracle.load()
    tel = make_workload(kf, args.workload, args.tracks, 1234567890, lib=lib)
    cfg = oracle.default_config(overstep_limit=OVERSTEP, **WORKLOADS[args.workload][2])
    base = cpu_oracle_rate(tel, cfg, args.steps, args.warmup)
    ms = base["seconds_per_step"] * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": workload_config(args.workload, args.tracks, "fp64"),
            "reference_path": "the reference algorithm's -d cpu path restated in C++ FP64 "
                              "(oracle/kf_oracle.cpp, OpenMP track loop); the reference binary "
                              "needs Eigen3, Boost and ROOT, absent here",
            "fitted_fraction": base["fitted_fraction"],
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_id: str | None):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        cmd = ["nvidia-smi", f"--query-gpu={QUERY}", "--format=csv,noheader,nounits", "-lms", "200"]
        if gpu_id:
            cmd += ["-i", gpu_id]
        try:
            self.p = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def gpu_uuid() -> str | None:
    import torch
    try:
        u = str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
        return u if u.startswith("GPU-") else f"GPU-{u}"
    except Exception:
        return None


def param_diff(a: dict, b: dict) -> float:
    """Largest |a - b| of the fitted parameters over max(|b|, sigma_b), over
    the tracks both fitted."""
    ok = (a["status"] == 0) & (b["status"] == 0)
    if not ok.any():
        return 0.0
    sig = np.sqrt(np.abs(b["cov"][[0, 6, 11, 15, 18, 20]][:, ok]))
    sc = np.maximum(np.abs(b["params"][:, ok]), sig)
    sc = np.where(sc > 0, sc, 1.0)
    return float(np.max(np.abs(a["params"][:, ok] - b["params"][:, ok]) / sc))


def timed_steps(step, stream, steps: int, warmup: int, barrier) -> tuple:
    """W untimed steps, then K steps between events on the launching stream,
    bracketed by a barrier and a device synchronize on both sides.  Returns
    (total ms, per-step ms list)."""
    import torch
    for _ in range(warmup):
        step()
    barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for a, b in evs:
        a.record(stream)
        step()
        b.record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    return t_start.elapsed_time(t_end), [a.elapsed_time(b) for a, b in evs]


def batched_step(batch, stream, ctas_per_sm: int = 0, block_size: int = 128) -> tuple:
    """Autotune the persistent kernel shape on this batch (or take the given
    threads per CTA and CTAs per SM), capture the sort and the fit into a CUDA
    graph; one step = one graph launch (4 kernels)."""
    if ctas_per_sm:
        batch.cfg.block_size, batch.cfg.min_blocks_per_sm = block_size, ctas_per_sm
        batch.cfg.kernel = 2
        tuned, tune_ms = batch.cfg, 0.0
    else:
        tuned, tune_ms = batch.autotune(stream)
    batch.make_plan(stream)
    shape = {"threads_per_cta": tuned.block_size, "ctas_per_sm": tuned.min_blocks_per_sm,
             "tracks_per_warp": 32, "autotune_best_ms_on_sample": round(tune_ms, 3)}
    return (lambda: batch.launch_plan(stream)), 4, shape


def suite_entry(kf, name: str, n: int, seed: int, stream, barrier, steps: int, warmup: int,
                pairs) -> dict:
    """Time the plain form (FP64 grid kernel) and the batched form of one
    workload on the same inputs; pairs = [(label, precision), ...] batched."""
    import torch
    tel = make_workload(kf, name, n, seed)
    out = {"workload": f"{name}: {WORKLOADS[name][0]}", "tracks": n}
    with torch.cuda.stream(stream):
        plain = kf.DeviceBatch(tel, fit_config(kf, name, "fp64"))
    ms, _ = timed_steps(lambda: plain.fit(stream), stream, steps, warmup, barrier)
    out["plain_fp64_tracks_per_s"] = n * steps / (ms * 1e-3)
    out["plain_fp64_ms_per_step"] = ms / steps
    del plain
    for label, prec in pairs:
        with torch.cuda.stream(stream):
            b = kf.DeviceBatch(tel, fit_config(kf, name, prec))
        step, _, shape = batched_step(b, stream)
        ms, _ = timed_steps(step, stream, steps, warmup, barrier)
        out[f"{label}_tracks_per_s"] = n * steps / (ms * 1e-3)
        out[f"{label}_ms_per_step"] = ms / steps
        out[f"{label}_shape"] = shape
        out[f"{label}_vs_plain_fp64"] = out[f"{label}_tracks_per_s"] / out["plain_fp64_tracks_per_s"]
        b.destroy_plan()
        del b
    torch.cuda.empty_cache()
    return out


def adjoint_entry(kf, n: int, seed: int, stream, barrier, steps: int, warmup: int) -> dict:
    """d(total smoothed chi2)/d(alignment 6 x 20, start parameters 6 per track,
    field scale) with kf_adjoint_batch, against one forward fit of the same
    batch (plain FP64 grid kernel and batched form)."""
    import torch
    tel = kf.make_telescope(n, seed=seed, **ALIGN20[1])
    cfg = kf.default_config(overstep_limit=OVERSTEP)
    with torch.cuda.stream(stream):
        fit = kf.DeviceBatch(tel, cfg)
    fit_ms, _ = timed_steps(lambda: fit.fit(stream), stream, steps, warmup, barrier)
    fit_ms /= steps
    step, _, shape = batched_step(fit, stream)
    bat_ms, _ = timed_steps(step, stream, steps, warmup, barrier)
    bat_ms /= steps
    fit.destroy_plan()
    del fit
    torch.cuda.empty_cache()
    with torch.cuda.stream(stream):
        ab = kf.AdjointBatch(tel, cfg)
    lib = kf.load()
    geo, keep = tel.geometry()
    field = tel.field(scale=1.0)

    def call(grad):
        rc = lib.kf_adjoint_batch(C.byref(ab.ins), C.byref(ab.aout), C.byref(ab.cfg),
                                  C.byref(geo), C.byref(field), C.c_int32(grad),
                                  C.c_void_p(ab.ws.data_ptr()), C.c_size_t(ab.ws_bytes),
                                  C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.kf_last_error_string().decode())

    adj_ms, _ = timed_steps(lambda: call(1), stream, steps, warmup, barrier)
    adj_ms /= steps
    fwd_ms, _ = timed_steps(lambda: call(0), stream, steps, warmup, barrier)
    fwd_ms /= steps
    st = ab.out["status"].cpu().numpy()
    del ab
    torch.cuda.empty_cache()
    return {"workload": f"align20: {ALIGN20[0]}", "tracks": n,
            "gradients": "d chi2_total / d (6 x 20 alignment, 6 start parameters per track, field scale)",
            "tracks_differentiated_per_s": n / (adj_ms * 1e-3),
            "adjoint_ms": adj_ms, "adjoint_forward_only_ms": fwd_ms,
            "fit_plain_fp64_ms": fit_ms, "fit_batched_fp64_ms": bat_ms,
            "adjoint_over_plain_fit": adj_ms / fit_ms, "adjoint_over_batched_fit": adj_ms / bat_ms,
            "differentiated_fraction": float((st == 0).mean()),
            "checkpoint_every_states": 5}


def simulation_entry(kf, n: int, seed: int, stream, barrier, host_sample: int) -> dict:
    """Input production: the uneven 30-plane workload generated on the GPU
    (kf_simulate_tracks, one thread per track, arrays written in HBM) against
    the host generator (kf_synth_tracks, OpenMP over all host cores) on a
    bounded sample of the same tracks; and the map workload's RK4 truth."""
    import torch
    _, kw, _ = WORKLOADS["holes30"]
    with torch.cuda.stream(stream):
        tel = kf.make_telescope(n, seed=seed, device="cuda", **kw)
    ms, _ = timed_steps(lambda: tel.simulate(stream), stream, 3, 3, barrier)
    out = {"workload": f"holes30: {WORKLOADS['holes30'][0]}", "tracks": n,
           "gpu_tracks_per_s": n * 3 / (ms * 1e-3), "gpu_ms": ms / 3,
           "bytes_written_per_track": 30 * 5 * 8 + 8 + 4 + (6 + 21 + 3 + 6) * 8}
    out["gpu_write_gbs"] = out["bytes_written_per_track"] * out["gpu_tracks_per_s"] / 1e9
    del tel
    torch.cuda.empty_cache()
    kf.make_telescope(1000, seed=seed, **kw)  # host warm-up (thread pool)
    t0 = time.perf_counter()
    kf.make_telescope(host_sample, seed=seed, **kw)
    sec = time.perf_counter() - t0
    out["host_tracks_per_s"] = host_sample / sec
    out["host_sample_tracks"] = host_sample
    out["host_threads"] = os.cpu_count()
    out["gpu_over_host"] = out["gpu_tracks_per_s"] / out["host_tracks_per_s"]
    # field-map truth (fixed-step RK4, 5 mm steps through the 101^3 map)
    _, mkw, _ = WORKLOADS["map30"]
    nm = max(1, n // 4)
    with torch.cuda.stream(stream):
        tm = kf.make_telescope(nm, seed=seed, device="cuda", **mkw)
    ms, _ = timed_steps(lambda: tm.simulate(stream), stream, 3, 3, barrier)
    out["map30_tracks"] = nm
    out["map30_gpu_tracks_per_s"] = nm * 3 / (ms * 1e-3)
    del tm
    torch.cuda.empty_cache()
    hm = max(1, host_sample // 10)
    t0 = time.perf_counter()
    kf.make_telescope(hm, seed=seed, **mkw)
    out["map30_host_tracks_per_s"] = hm / (time.perf_counter() - t0)
    out["map30_gpu_over_host"] = out["map30_gpu_tracks_per_s"] / out["map30_host_tracks_per_s"]
    return out


def output_entry(kf, n: int, seed: int, stream) -> dict:
    """The output writers (gb300kf_io.h, Run/Common/Writer.hpp) on one fitted
    batch with smoothed states: host seconds per file, written to a scratch
    directory that is removed afterwards."""
    import os
    import shutil
    import tempfile
    import torch
    from gpukalmanfitter_gb300 import writer
    tel = make_workload(kf, "uniform10", n, seed)
    with torch.cuda.stream(stream):
        b = kf.DeviceBatch(tel, fit_config(kf, "uniform10", "fp64"), smoothed=True)
    b.fit(stream)
    stream.synchronize()
    res = {k: v for k, v in b.results().items()}
    del b
    torch.cuda.empty_cache()
    d = tempfile.mkdtemp(prefix="kf_out_")
    out = {"workload": "uniform10: the headline telescope, smoothed states kept", "tracks": n,
           "threads": os.cpu_count()}
    try:
        for name, fn in (("params_csv", lambda p: writer.write_params_csv(p, res)),
                         ("states_obj", lambda p: writer.write_states_obj(p, res, tel)),
                         ("params_table", lambda p: writer.write_params_table(p, res, tel))):
            path = os.path.join(d, name)
            fn(path)  # warm-up (page cache, thread pool)
            t0 = time.perf_counter()
            fn(path)
            sec = time.perf_counter() - t0
            size = os.path.getsize(path)
            out[name] = {"seconds": sec, "tracks_per_s": n / sec, "mb": size / 1e6,
                         "mb_per_s": size / 1e6 / sec}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return out


def rank_workload(kf, name: str, n: int, rank: int, world: int, seed: int):
    """This rank's share of one global batch of world * n tracks.  One GPU:
    the host generator's n tracks (the reference arm's inputs exactly).
    Several: every rank simulates the global batch on its own GPU
    (kf_simulate_tracks, the host generator's tracks) and keeps the tracks
    shard.rank_tracks deals it (warp-sized chunks of the work-key order,
    round-robin), as host arrays."""
    if world == 1:
        return make_workload(kf, name, n, seed)
    import torch
    from gpukalmanfitter_gb300 import shard
    glob = kf.make_telescope(world * n, seed=seed, device="cuda", **WORKLOADS[name][1])
    torch.cuda.synchronize()
    mine = shard.subset(glob, shard.rank_tracks(glob, rank, world)).to_host()
    if mine.field_grid is not None and hasattr(mine.field_grid, "cpu"):
        mine.field_grid = mine.field_grid.cpu().numpy()
    del glob
    torch.cuda.empty_cache()
    return mine


def suite_summary(suite: dict | None, e2e: dict | None, ref_cpu: dict | None) -> dict:
    """The suite's times and ratios in a few hundred bytes, printed as the
    line's last key."""
    out = {}
    r = lambda v, d=3: None if v is None else round(float(v), d)
    if suite:
        b = suite.get("batching")
        if b:
            out["batching_4M_holes30_ms"] = {"plain_fp64": r(b["plain_fp64_ms_per_step"], 1),
                                             "batched_fp64": r(b["batched_fp64_ms_per_step"], 1),
                                             "batched_mixed": r(b["batched_mixed_ms_per_step"], 1)}
            out["batched_fp64_over_plain"] = r(b["batched_fp64_vs_plain_fp64"])
        m = suite.get("precision_map")
        if m:
            out["map30_1M_ms"] = {"plain_fp64": r(m["plain_fp64_ms_per_step"], 1),
                                  "batched_fp64": r(m["batched_fp64_ms_per_step"], 1),
                                  "batched_mixed": r(m["batched_mixed_ms_per_step"], 1)}
            out["mixed_over_plain_fp64"] = r(m["batched_mixed_vs_plain_fp64"])
            out["mixed_over_batched_fp64"] = r(m["batched_fp64_ms_per_step"] /
                                               m["batched_mixed_ms_per_step"])
        d = suite.get("differentiation")
        if d:
            out["adjoint_256k_ms"] = {"adjoint": r(d["adjoint_ms"], 1),
                                      "fit_plain_fp64": r(d["fit_plain_fp64_ms"], 1)}
            out["adjoint_over_plain_fit"] = r(d["adjoint_over_plain_fit"])
            out["grads_per_s"] = r(d["tracks_differentiated_per_s"], 0)
    if e2e and ref_cpu:
        out["e2e_over_cpu_baseline"] = r(e2e["value"] / ref_cpu["value"], 2)
    return out


def run_gpu(args) -> None:
    import torch
    import gpukalmanfitter_gb300 as kf
    from gpukalmanfitter_gb300 import flops as F

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    tel = rank_workload(kf, args.workload, args.tracks, rank, world, 1234567890)
    n = tel.n  # this rank's tracks (args.tracks, up to a warp chunk when sharded)
    cfg = fit_config(kf, args.workload, args.precision)
    lib = kf.load()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def total(count: int) -> int:
        if dist is None:
            return count
        t = torch.tensor([count], dtype=torch.int64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return int(t.item())

    n_total = total(n)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        batch = kf.DeviceBatch(tel, cfg)
    torch.cuda.synchronize()
    shape = None
    if args.form == "batched":
        step, per_step, shape = batched_step(batch, stream, args.ctas_per_sm, args.block_size)
    else:
        step, per_step = (lambda: batch.fit(stream)), 1

    # ---- kernel-resident timing: inputs in HBM
    barrier()
    sampler = ClockSampler(gpu_uuid())
    elapsed_ms, launch_ms = timed_steps(step, stream, args.steps, args.warmup, barrier)
    clocks = sampler.stop()
    if dist is not None:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    value = n_total * args.steps / (elapsed_ms * 1e-3)
    res = batch.results()

    # the other form on the same batch (same precision): plain vs batched
    forms = {args.form: value}
    if args.form == "batched":
        pms, _ = timed_steps(lambda: batch.fit(stream), stream, args.steps, args.warmup, barrier)
        if dist is not None:
            t = torch.tensor([pms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            pms = float(t.item())
        forms["plain"] = n_total * args.steps / (pms * 1e-3)
        forms["max_param_diff_over_scale"] = param_diff(batch.results(), res)
    batch.destroy_plan()

    ok_frac = float(np.mean(res["status"] == 0))
    flop = F.batch_flops(res["n_trials"], res["n_steps"], res["n_meas"], res["status"],
                         uniform=tel.field_grid is None)
    dense_flop = F.batch_flops(res["n_trials"], res["n_steps"], res["n_meas"], res["status"], dense=True)
    avg_launch_s = statistics.mean(launch_ms) * 1e-3
    peak = C.c_double(0)
    rc = lib.kf_diag_fp64_fma_rate(C.c_int32(20000), C.byref(peak), C.c_void_p(stream.cuda_stream))
    peak_tflops = peak.value / 1e3 if rc == 0 else None
    achieved = flop / avg_launch_s / 1e12
    traffic = traffic_estimate(args, n, shape)
    mb = F.batch_bytes(n, tel.n_surfaces)
    hbm_peak, hbm_src = hbm_peak_gbs()

    # ---- end to end through the public host-buffer call (pinned memory)
    e2e = None
    if not args.no_e2e:
        ecfg = fit_config(kf, args.workload, args.precision)
        if args.form == "batched":
            ecfg.kernel, ecfg.block_size = 2, shape["threads_per_cta"]
            ecfg.min_blocks_per_sm = shape["ctas_per_sm"]
        e2e = run_e2e(kf, lib, tel, ecfg, stream, args, barrier, dist, n_total)
    del batch
    torch.cuda.empty_cache()

    suite = None
    wanted = [] if args.no_suite else [x for x in args.suite.split(",") if x and x != "none"]
    if wanted and world == 1:
        # uneven tracks (4x the headline batch), the field map (1x), the adjoint
        # (262144 tracks at the default 1M, the differentiation workload's size)
        makers = {
            "batching": lambda: suite_entry(kf, "holes30", 4 * n, 1234567892, stream, barrier, 3, 3,
                                            [("batched_fp64", "fp64"), ("batched_mixed", "mixed")]),
            "precision_map": lambda: suite_entry(kf, "map30", n, 1234567893, stream, barrier, 3, 3,
                                                 [("batched_mixed", "mixed"), ("batched_fp64", "fp64")]),
            "differentiation": lambda: adjoint_entry(kf, max(1, n * 262144 // 1000000),
                                                     1234567894, stream, barrier, 3, 3),
            "material": lambda: suite_entry(kf, "material10", n, 1234567895, stream, barrier, 3, 3,
                                            [("batched_fp64", "fp64"), ("batched_mixed", "mixed")]),
            "output": lambda: output_entry(kf, max(1, n * 262144 // 1000000), 1234567896, stream),
            "simulation": lambda: simulation_entry(kf, 4 * n, 1234567897, stream, barrier,
                                                   max(1, n // 5)),
        }
        suite = {k: makers[k]() for k in makers if k in wanted}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the reference algorithm's CPU path on this run's own tracks, all host
        # threads, then one host thread on the first SINGLE_THREAD_SAMPLE tracks
        import oracle
        ocfg = oracle.default_config(overstep_limit=OVERSTEP, **WORKLOADS[args.workload][2])
        base = cpu_oracle_rate(tel, ocfg, 3, 1)
        cpu = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
        one = cpu_oracle_rate(make_workload(kf, args.workload, min(n, SINGLE_THREAD_SAMPLE),
                                            1234567890), ocfg, 3, 1, threads=1)
        cpu["single_thread"] = {"value": one["value"], "unit": UNIT, "cores": 1,
                                "sample": one["sample"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": DATA,
            "config": workload_config(args.workload, args.tracks, args.precision),
            "form": {"form": args.form, "kernel_shape": shape,
                     "parallelism": f"one global batch of {n_total} tracks in balanced shards "
                                    f"over {world} GPU(s), no collective on the fit"},
            "forms": forms,
            "fitted_fraction": ok_frac,
            "gpu_launches": args.steps * per_step,
            "e2e": e2e,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak_tflops,
                         "unit": "TFLOP/s", "frac": (achieved / peak_tflops) if peak_tflops else None,
                         "traffic": traffic,
                         "peak_source": "FP64 DFMA rate measured in this run by kf_diag_fp64_fma_rate "
                                        "(independent DFMA chains on all SMs): MEASURED_PEAKS.json "
                                        "has no FP64 entry (HBM and bf16 only)",
                         "algorithmic_flop_per_launch": flop,
                         "algorithmic_flop_per_track": flop / n,
                         "dense_reference_flop_per_track": dense_flop / n,
                         "avg_launch_ms": avg_launch_s * 1e3,
                         "launch_timed": "one step (graph of sort + fit kernels)" if args.form == "batched"
                                         else "one fit kernel launch",
                         "hbm_view": {"algorithmic_bytes_per_launch": mb["total"],
                                      "achieved_gbs": mb["total"] / avg_launch_s / 1e9,
                                      "peak_gbs": hbm_peak, "peak_source": hbm_src,
                                      "frac": mb["total"] / avg_launch_s / 1e9 / hbm_peak}},
            "clocks": clocks,
        }
        if suite is not None:
            line["suite"] = suite
        if cpu is not None:
            line["cpu_baseline"] = cpu
        line["suite_summary"] = suite_summary(suite, e2e, cpu)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def traffic_estimate(args, n: int, shape):
    """DRAM bytes per launch from a committed ncu capture of the same kernel
    instantiation and workload (scaled by tracks), or None."""
    tfile = ROOT / "profiles" / "traffic.json"
    if not tfile.exists():
        return None
    key = f"{args.workload}/{args.precision}/{args.form}"
    if shape:
        key += f"/{shape['threads_per_cta']}x{shape['ctas_per_sm']}"
    try:
        rec = json.loads(tfile.read_text()).get(key)
        return rec["dram_bytes_per_track"] * n if rec else None
    except (ValueError, KeyError, TypeError):
        return None


def hbm_peak_gbs() -> tuple:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            v = json.loads(f.read_text()).get("hbm_gbs")
            if v:
                return float(v), "MEASURED_PEAKS.json hbm_gbs (measured)"
        except ValueError:
            pass
    return 6800.0, "fallback 6.8 TB/s (no hbm_gbs in MEASURED_PEAKS.json)"


def run_e2e(kf, lib, tel, cfg, stream, args, barrier, dist, n_total: int) -> dict:
    import torch
    n, S = tel.n, tel.n_surfaces

    def pinned(a):
        t = torch.empty(a.shape, dtype={np.dtype(np.float64): torch.float64,
                                        np.dtype(np.int32): torch.int32,
                                        np.dtype(np.uint64): torch.int64}[a.dtype], pin_memory=True)
        arr = t.numpy().view(a.dtype)
        arr[...] = a
        return t, arr

    keep = []
    host_in = {}
    for k, v in kf.tel_arrays(tel).items():
        t, arr = pinned(np.ascontiguousarray(v))
        keep.append(t)
        host_in[k] = arr
    host_out = {}
    for k, v in kf.host_outputs(n, S).items():
        t, arr = pinned(v)
        keep.append(t)
        host_out[k] = arr
    ins = kf.inputs_struct(host_in, n, S, lambda x: x.ctypes.data)
    outs = kf._outputs_struct(host_out)
    geo, gkeep = tel.geometry()
    fld = tel.field()
    size = lib.kf_host_staging_size(C.byref(cfg), n, S, 0)
    staging = torch.empty(size, dtype=torch.uint8, device="cuda")

    def call():
        rc = lib.kf_fit_batch_host(C.byref(ins), C.byref(outs), C.byref(cfg), C.byref(geo),
                                   C.byref(fld), C.c_void_p(staging.data_ptr()), C.c_size_t(size),
                                   C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.kf_last_error_string().decode())

    for _ in range(args.warmup):
        call()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call()
    dt = time.perf_counter() - t0
    barrier()
    if dist is not None:
        t = torch.tensor([dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
    h2d = sum(v.nbytes for v in host_in.values() if v is not None)
    d2h = sum(host_out[k].nbytes for k in ("params", "cov", "chi2", "status", "n_meas", "n_steps", "n_trials"))
    return {"value": n_total * args.steps / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "path": "kf_fit_batch_host: pinned host SoA -> device staging -> fit -> host, synchronised per step"}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tracks", type=int, default=1_000_000, help="tracks per GPU")
    ap.add_argument("--workload", default="uniform10", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=sorted(PRECISIONS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--form", default="batched", choices=["batched", "plain"],
                    help="batched: sorted queue + persistent kernel in a CUDA graph; "
                         "plain: one thread per track, grid over the batch")
    ap.add_argument("--no-suite", action="store_true",
                    help="skip the uneven-track, field-map and adjoint comparisons")
    ap.add_argument("--ctas-per-sm", type=int, default=0, choices=[0, 1, 2, 3, 4, 5, 8],
                    help="batched form: persistent kernel CTAs per SM (0 = autotune)")
    ap.add_argument("--block-size", type=int, default=128, choices=[64, 128, 256],
                    help="batched form with --ctas-per-sm: threads per CTA; compiled "
                         "shapes 128 x 2..5, 64 x 4, 64 x 8, 256 x 1, 256 x 2")
    ap.add_argument("--suite",
                    default="batching,precision_map,differentiation,material,output,simulation",
                    help="comma list of suite entries to run (or 'none')")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
