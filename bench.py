"""Benchmark: DRR + grad-NCC pose evaluations per second on one GB300.

Workload (N=1): 256^3 float32 phantom at 1 mm, detector 1536^2 at 0.194 mm
downsampled 4x to 384^2, populations of lambda = 100 candidate poses (rotations
~ N(0, 10 deg), translations ~ N(0, 20 mm)), grad-NCC (5x5 Gaussian + Sobel) against
a noisy fixed image; one step = one population evaluation, captured as a CUDA
graph.  Inputs are seeded synthetic data with those shapes (no dataset exists
for this path).

  value     poses/s with the populations already in device memory, CUDA events
            around each step; L2 (129 MB) is flushed between steps by writing a
            256 MB buffer outside the timed events.
  e2e       poses/s through the public C ABI (xr_obj_eval) from pinned host
            poses to host similarity values, copies inside the timed region.
  roofline  DRR kernel (the dominant launch): bytes of the voxel cells it
            loads per launch over its CUDA-event duration, against the L2 read
            bandwidth measured in the same run; beside it the cost model's
            algorithmic bytes (8 neighbour reads x voxel bytes x every sample)
            against the measured HBM peak, ncu DRAM traffic, and the same
            figures with every sample loaded (skipping off, CT-like air).
  cpu_baseline  the CPU oracle (a restatement of xReg's TBB CPU path) on a
            bounded sample of the same workload, all host cores.
  errors_vs_oracle  DRR and grad-NCC errors of the float32 / FP16 / BF16 paths
            against the oracle's FP32 restatement and its FP64 twin.

--impl reference times that CPU path alone as the reference arm, one full
population per step, with nothing of the product loaded.
Multi-GPU: replicas only (each rank evaluates its own populations; no collective).
"""
from __future__ import annotations

import argparse
import dataclasses
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

POP = 100
PEAK_FALLBACK_GBS = 6800.0


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--voxel", default="f32", choices=["f32", "f16", "bf16"])
    p.add_argument("--path", default="split", choices=["fused", "split"],
                   help="evaluation path timed as the headline (the other is timed beside it)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU-baseline sample")
    p.add_argument("--no-extras", action="store_true")
    p.add_argument("--only", default="", choices=["", "plain-small", "precision", "multi-job", "serving"],
                   help="run one of the extra measurements alone and print its JSON (for profiling)")
    p.add_argument("--serving-requests", type=int, default=200,
                   help="requests per arrival rate in the serving measurement (0 = off)")
    p.add_argument("--serving-rates", default=",".join(str(r) for r in SERVING_RATES),
                   help="Poisson arrival rates (per second) of the serving measurement")
    p.add_argument("--launch-config", default="auto",
                   help="DRR kernel configuration 'layout,block_warps_x,unroll[,warp_rows]' (layout 0 linear, "
                        "1 cell8, 2 cell8 256-bit; warp_rows 4 = 8x4-pixel warps, 8 = 4x8) instead of the "
                        "autotuner's choice")
    return p.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _workload(seed=0):
    from xreg_gb300 import synth
    w = synth.batched_population(seed, POP)
    return w


def _populations(w, n, seed):
    from xreg_gb300 import synth
    rng = np.random.default_rng(seed)
    out = np.empty((n, POP, 4, 4))
    for k in range(n):
        out[k] = synth.sample_poses(w.vol, w.gt, POP, w.rot_sigma, w.trans_sigma, seed=int(rng.integers(1 << 30)))
    return out


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 50 ms; each line is stamped
    with the host time it arrived, so the summary can keep the samples of one
    timed window."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []  # (host time, line)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def wait_started(self, timeout_s: float = 5.0) -> None:
        """Returns once the first sample has arrived (or after timeout_s)."""
        t_end = time.time() + timeout_s
        while self.proc and not self.lines and time.time() < t_end:
            time.sleep(0.01)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0: float | None = None, t1: float | None = None):
        """Median SM clock under load and the throttle reasons seen, over the
        samples that arrived in [t0, t1] (host time.time(); all when None)."""
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        window = [ln for t, ln in self.lines if (t0 is None or t >= t0) and (t1 is None or t <= t1)]
        note = None
        if not window and t0 is not None:  # a window shorter than the sampling period
            window = [ln for t, ln in self.lines if t0 - 0.2 <= t <= (t1 or t0) + 0.2]
            note = "no sample inside the timed steps; samples within 0.2 s of them"
        for ln in window:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"], "samples": 0}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        out = {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": mx, "reasons": sorted(reasons),
               "samples": len(sm)}
        if note:
            out["window"] = note
        return out


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return PEAK_FALLBACK_GBS, "fallback"


def _ncu_traffic(workload_tag: str, what: str = "traffic_bytes_per_launch"):
    """A figure of the DRR kernel from a committed ncu summary (profiles/*.md line
    '<what>[<tag>]: N', or '<what>: N' when workload_tag is empty), else None:
    per-launch DRAM traffic, per-launch L2 traffic, the L2 sector peak."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    key = f"{what}[{workload_tag}]:" if workload_tag else f"{what}:"
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        with open(os.path.join(d, fn)) as f:
            for line in f:
                if line.strip().startswith(key):
                    try:
                        return float(line.split(":", 1)[1].strip())
                    except ValueError:
                        return None
    return None


def _drr_kernel_stats(rc, d_pose_ptr: int, reps: int, stream, flush):
    """The DRR launch alone for one device-resident population: mean CUDA-event
    duration over reps launches (L2 flushed before each, outside the events),
    the samples of the reference step rule and the samples loaded."""
    import torch
    rc.set_count_samples(True)
    rc.distribute_xforms_device(POP, d_pose_ptr)
    rc.compute()
    samples, loaded = rc.last_num_samples(), rc.last_num_loaded_samples()
    rc.set_count_samples(False)
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for i in range(reps):
            flush.fill_(float(i))
            kev[i][0].record(stream)
            rc.compute()
            kev[i][1].record(stream)
    torch.cuda.synchronize()
    return float(np.mean([s.elapsed_time(e) for s, e in kev])), samples, loaded


def _roofline(vt: int, layout: int, drr_ms: float, samples: int, loaded: int, l2_peak: float, tag: str) -> dict:
    """Gather roofline of the DRR kernel.  achieved = bytes of the voxel cells it
    loads (one CELL8 cell per loaded sample: 32 B float32, 16 B half; 8 corner
    reads for the linear layout) over its CUDA-event time; peak = the L2 read
    bandwidth measured in this run.  Beside it: the cost model's algorithmic
    bytes (8 neighbour reads x voxel bytes x every sample of the reference step
    rule) against the measured HBM copy peak, and the ncu DRAM traffic."""
    per_sample = (32 if vt == 0 else 16) if layout != 0 else 8 * (4 if vt == 0 else 2)
    t = drr_ms / 1e3
    gather = per_sample * loaded
    achieved = gather / t / 1e9
    hbm, hbm_kind = _peaks()
    alg = 8.0 * (4 if vt == 0 else 2) * samples
    traffic = _ncu_traffic(tag)
    out = {"bound": "l2", "achieved": round(achieved, 1), "peak": round(l2_peak, 1), "unit": "GB/s",
           "frac": round(achieved / l2_peak, 4), "traffic": traffic,
           "peak_source": "measured in this run: xr_measure_l2_read_bandwidth (48 MB made L2-resident, read 40 "
                          "times with 16-byte L2 loads from every SM, CUDA events)",
           "achieved_bytes": f"{per_sample} B of voxel cell per loaded sample x {loaded} loaded samples",
           "samples_per_launch": samples, "loaded_samples_per_launch": loaded,
           "loaded_frac": round(loaded / max(samples, 1), 4), "kernel_ms": round(drr_ms, 4),
           "warp_instructions_per_loaded_sample": _ncu_traffic(tag, "warp_instructions_per_loaded_sample"),
           "cost_model": {"achieved": round(alg / t / 1e9, 1), "peak": hbm, "unit": "GB/s",
                          "frac": round(alg / t / 1e9 / hbm, 4),
                          "peak_source": f"{hbm_kind} hbm_gbs (MEASURED_PEAKS.json)",
                          "bytes_per_launch": alg,
                          "note": "8 neighbour reads x voxel bytes x every sample, loaded or skipped; above 1 "
                                  "because the reads hit L1/L2 and proven-zero samples are not loaded"}}
    if traffic:
        out["hbm_traffic_frac"] = round(traffic / t / 1e9 / hbm, 4)
    return out


def _errors_vs_oracle(xr, w, fixed, dev, poses):
    """DRR and grad-NCC errors of the float32 / FP16 / BF16 volume paths on two
    poses of a timed population, against the oracle's FP32 restatement of
    xReg's ray caster and its FP64 twin, and the similarity values against the
    oracle's double arithmetic (on the oracle's FP32 DRRs and on the GPU's own)."""
    from oracle import oracle as O
    from tests.helpers import oracle_cams, oracle_geom
    O.set_threads(os.cpu_count() or 1)
    geom, cams = oracle_geom(w.vol), oracle_cams(w.cams)
    r32, ns = O.drr_f32(w.vol.voxels, geom, cams, poses, step=w.step, count=True)
    r64 = O.drr_f64(w.vol.voxels, geom, cams, poses, step=w.step)
    s32 = O.grad_ncc(fixed, r32)
    s64 = O.grad_ncc(fixed, r64.astype(np.float32))
    body = r64 > 0.1 * r64.max()
    out = {"poses": len(poses), "samples": int(ns.sum()),
           "fp32_oracle_itself": {"drr_max_rel_vs_fp64_body": float(np.max(np.abs(r32[body] - r64[body]) / r64[body]))}}
    tol = {0: 1e-4, 1: 2e-3, 2: 2e-3}
    for name, vt in (("f32", 0), ("f16", 1), ("bf16", 2)):
        rc = xr.RayCasterLineIntCUDA(dev)
        rc.set_volume(w.vol, vt)
        rc.set_camera_models(w.cams)
        rc.set_ray_step_size(w.step)
        m = xr.ImgSimMetric2DGradNCCCUDA(dev)
        m.set_fixed_image(fixed)
        obj = xr.PopulationObjective(rc, [m], len(poses))
        sims = obj.eval(poses)
        g = rc.projs()
        nz = r32 != 0
        rel32 = float(np.max(np.abs(g[nz] - r32[nz]) / r32[nz]))
        r64b = np.abs(g[body] - r64[body]) / r64[body]
        e = {"drr_max_rel_vs_fp32_oracle": rel32, "background_equal": bool(np.all(g[~nz] == 0)),
             "drr_max_rel_vs_fp64_oracle_body": float(r64b.max()),
             "drr_median_rel_vs_fp64_oracle_body": float(np.median(r64b)),
             "grad_ncc_max_abs_vs_oracle_fp32_drrs": float(np.max(np.abs(sims - s32))),
             "grad_ncc_max_abs_vs_oracle_fp64_drrs": float(np.max(np.abs(sims - s64))),
             "grad_ncc_max_abs_vs_oracle_on_same_drrs": float(np.max(np.abs(sims - O.grad_ncc(fixed, g)))),
             "drr_tolerance": tol[vt], "within_drr_tolerance": rel32 <= tol[vt]}
        if vt == 2:
            e["note"] = "BF16 volume: an 8-bit significand rounds a voxel by up to 2^-8; outside the 2e-3 " \
                        "half-precision tolerance (held to 2^-8 in the tests)"
        out[name] = e
        obj.close()
    return out


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(w, fixed, budget_s: float):
    """The oracle's FP32 DRR + grad-NCC on all host cores, on as many poses of the
    workload as fit the time budget (at least 1)."""
    from oracle import oracle as O
    from tests.helpers import oracle_cams, oracle_geom
    cores = O.set_threads(os.cpu_count() or 1)
    geom, cams = oracle_geom(w.vol), oracle_cams(w.cams)
    poses = _populations(w, 1, 999)[0]
    done, t_used, i = 0, 0.0, 0
    while True:
        t0 = time.perf_counter()
        d = O.drr_f32(w.vol.voxels, geom, cams, poses[i % POP][None], step=w.step)
        O.grad_ncc(fixed, d)
        t_used += time.perf_counter() - t0
        done += 1
        i += 1
        if t_used >= budget_s or done >= POP:
            break
    return {"value": done / t_used, "unit": "poses/s", "cores": cores, "kind": "port",
            "sample": f"{done} poses of the 256^3 / 384^2 / grad-NCC workload (FP32 DRR + grad-NCC, "
                      f"{t_used:.1f} s of CPU work)"}


# ----------------------------------------------------------------- our arm
def run_ours(a, rank, world, local):
    import torch
    import xreg_gb300 as xr
    from xreg_gb300 import synth

    torch.cuda.set_device(local)
    dev = local
    xr.load()
    w = _workload(seed=rank)
    vt = {"f32": 0, "f16": 1, "bf16": 2}[a.voxel]
    stream = torch.cuda.Stream(device=dev)

    # fixed image: DRR at the ground-truth pose + 1% noise (computed on the GPU)
    forced = None if a.launch_config == "auto" else tuple(int(v) for v in a.launch_config.split(","))
    rc0 = xr.RayCasterLineIntCUDA(dev)
    if forced:
        rc0.set_launch_config(*forced)
    rc0.set_volume(w.vol)
    rc0.set_camera_model(w.cams[0])
    rc0.set_ray_step_size(w.step)
    rc0.set_num_projs(1)
    rc0.allocate_resources()
    rc0.distribute_xforms_among_cam_models(synth.fixed_pose(w)[None])
    rc0.compute()
    fixed = synth.add_noise(rc0.proj(0), 0.01, w.seed + 2)
    rc0.close()

    rc = xr.RayCasterLineIntCUDA(dev)
    if forced:
        rc.set_launch_config(*forced)
    rc.set_stream(stream.cuda_stream)
    rc.set_volume(w.vol, vt)
    rc.set_camera_model(w.cams[0])
    rc.set_ray_step_size(w.step)
    m = xr.ImgSimMetric2DGradNCCCUDA(dev)
    m.set_fixed_image(fixed)
    obj = xr.PopulationObjective(rc, [m], POP)
    obj.set_fused(a.path == "fused")

    nsteps = a.warmup + a.steps
    pops = _populations(w, nsteps, 1234 + rank)
    d_pops = torch.from_numpy(pops.reshape(nsteps, POP, 16).copy()).to(f"cuda:{dev}")
    d_sims = torch.empty((nsteps, POP), dtype=torch.float32, device=f"cuda:{dev}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    torch.cuda.synchronize()

    def step(k):
        obj.eval_device(POP, d_pops[k].data_ptr(), d_sims[k].data_ptr())

    clk = ClockSampler(dev).__enter__()  # running before the warm-up: sampling during the timed steps
    clk.wait_started()
    with torch.cuda.stream(stream):
        for k in range(a.warmup):
            step(k)
    stream.synchronize()

    # ---- timed region (device-resident inputs)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    _barrier(world)
    torch.cuda.synchronize()
    t_clk0 = time.time()
    with torch.cuda.stream(stream):
        for i in range(a.steps):
            flush.fill_(float(i))  # > L2, outside the events
            evs[i][0].record(stream)
            step(a.warmup + i)
            evs[i][1].record(stream)
    torch.cuda.synchronize()
    t_clk1 = time.time()
    time.sleep(0.1)  # let the sample taken at the end of the window arrive
    clk.__exit__()
    ms = [s.elapsed_time(e) for s, e in evs]
    t_total = _max_over_ranks(sum(ms) / 1e3, world)
    value = world * a.steps * POP / t_total

    # ---- the other evaluation path on the same populations, for comparison
    other = "split" if a.path == "fused" else "fused"
    obj.set_fused(other == "fused")
    d_other = torch.empty((a.steps, POP), dtype=torch.float32, device=f"cuda:{dev}")
    with torch.cuda.stream(stream):
        for k in range(3):
            obj.eval_device(POP, d_pops[k].data_ptr(), d_other[0].data_ptr())
    oev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    with torch.cuda.stream(stream):
        for i in range(a.steps):
            flush.fill_(float(i))
            oev[i][0].record(stream)
            obj.eval_device(POP, d_pops[a.warmup + i].data_ptr(), d_other[i].data_ptr())
            oev[i][1].record(stream)
    torch.cuda.synchronize()
    t_other = sum(s0.elapsed_time(e0) for s0, e0 in oev) / 1e3
    paths = {a.path: round(a.steps * POP / (t_total / world), 2), other: round(a.steps * POP / t_other, 2),
             "values_identical": bool(torch.equal(d_other, d_sims[a.warmup:])),
             "fused_path": "one persistent kernel: DRR tiles, then each image's grad-NCC tile by tile behind "
                           "them (+ one geometry launch)",
             "split_path": "DRR launch, then grad-NCC moment and combine launches, replayed as a CUDA graph"}
    obj.set_fused(a.path == "fused")

    # ---- e2e through the C ABI with host buffers (pinned poses in, sims out)
    h_pops = torch.empty((a.steps, POP, 16), dtype=torch.float64, pin_memory=True)
    h_pops.copy_(torch.from_numpy(pops[a.warmup:].reshape(a.steps, POP, 16)))
    h_sims = torch.empty((a.steps, POP), dtype=torch.float32, pin_memory=True)
    hp, hs = h_pops.numpy(), h_sims.numpy()
    obj.eval(hp[0])  # settle the host-entry path
    e2e_t = 0.0
    for i in range(a.steps):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hs[i] = obj.eval(hp[i])
        e2e_t += time.perf_counter() - t0
    e2e_t = _max_over_ranks(e2e_t, world)
    e2e = world * a.steps * POP / e2e_t
    np.testing.assert_array_equal(hs, d_sims[a.warmup:].cpu().numpy())  # same values both ways

    # ---- DRR kernel alone: duration and sample counts (roofline)
    drr_ms, samples, loaded = _drr_kernel_stats(rc, d_pops[a.warmup].data_ptr(), a.steps, stream, flush)
    layout, bw, unroll, wrows = rc.launch_config_ex()
    lname = {0: "linear", 1: "cell8", 2: "cell8-256bit"}.get(layout, str(layout))
    wcols = 32 // wrows
    wshape = "" if wrows == 4 else f"-warp{wcols}x{wrows}"
    block = f"{wcols * bw}x{(8 // bw) * wrows}"
    tag = f"batched-256^3-384^2-pop100-{a.voxel}-{lname}-loop{unroll}{wshape}"
    l2_peak = xr.measure_l2_read_bandwidth(dev)
    roofline = _roofline(vt, layout, drr_ms, samples, loaded, l2_peak, tag)
    roofline["kernel"] = f"drr_kernel<{a.voxel},sum,{lname},unroll{unroll}> block {block}, warps {wcols}x{wrows}"

    extras = {}
    if not a.no_extras and rank == 0:
        extras = _extras(xr, w, fixed, dev, stream, pops[a.warmup], d_sims, a, flush, l2_peak)
        for key in ("batched_f32_skipping_off", "batched_f32_noisy_air"):
            if isinstance(extras.get(key), dict) and "drr_kernel" in extras[key]:
                roofline["dense" if key.endswith("off") else "noisy_air"] = extras[key]["drr_kernel"]

    res = {
        "metric": "poses/sec (DRR+grad-NCC pose evaluations, batched population)",
        "value": round(value, 2),
        "unit": "poses/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": round(t_total * 1e3 / a.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"f32": "f32", "f16": "f16-volume/f16x2-x-blend/f32-accum", "bf16": "bf16-volume/f32-accum"}[a.voxel],
        "data": "synthetic (seeded ellipsoid phantom, sampled poses, noisy fixed DRR)",
        "config": dict(_config(w, a.voxel), l2="flushed between timed steps (256 MB write)",
                       parallelism=f"replicas x{world}"),
        "e2e": {"value": round(e2e, 2), "unit": "poses/s", "h2d_bytes_per_step": POP * 16 * 8,
                "d2h_bytes_per_step": POP * 4},
        "gpu_launches": a.steps * (2 if a.path == "fused" else 5),
        "evaluation_paths_poses_per_s": paths,
        "roofline": roofline,
        "clocks": clk.summary(t_clk0, t_clk1 + 0.06),
    }
    if rank == 0:
        res["cpu_baseline"] = cpu_baseline(w, fixed, a.cpu_seconds)
        res.update(extras)
    return res


def _plain_small(xr, dev, cpu_budget_s: float):
    """The plain method's own configuration: 128^3 FP32 phantom at 1.5 mm, 256^2
    detector at 1.55 mm, 0.5 mm step, NCC, one pose per evaluation.  The GPU's
    plain path (pose upload, DRR launch, NCC launches, host read per pose) and
    the oracle's FP32 DRR + NCC on the host cores, on the same poses; the largest
    difference of the NCC values over the poses the oracle ran."""
    from oracle import oracle as O
    from tests.helpers import oracle_cams, oracle_geom
    from xreg_gb300 import synth
    w = synth.plain_small(0)
    rc0 = xr.RayCasterLineIntCUDA(dev)
    rc0.set_volume(w.vol)
    rc0.set_camera_model(w.cams[0])
    rc0.set_ray_step_size(w.step)
    rc0.set_num_projs(1)
    rc0.allocate_resources()
    rc0.distribute_xforms_among_cam_models(synth.fixed_pose(w)[None])
    rc0.compute()
    fixed = synth.add_noise(rc0.proj(0), 0.01, w.seed + 2)
    rc0.close()
    poses = synth.sample_poses(w.vol, w.gt, 200, w.rot_sigma, w.trans_sigma, seed=w.seed + 3)
    rc = xr.RayCasterLineIntCUDA(dev)
    rc.set_volume(w.vol)
    rc.set_camera_model(w.cams[0])
    rc.set_ray_step_size(w.step)
    rc.set_num_projs(1)
    rc.allocate_resources()
    m = xr.ImgSimMetric2DNCCCUDA(dev)
    m.set_fixed_image(fixed)
    m.set_num_moving_images(1)
    m.set_mov_imgs_buf_from_ray_caster(rc, 0)
    m.allocate_resources()
    for i in range(5):
        rc.distribute_xforms_among_cam_models(poses[i][None])
        rc.compute()
        m.compute()
        m.sim_vals()
    vals = []
    t0 = time.perf_counter()
    for p in poses:
        rc.distribute_xforms_among_cam_models(p[None])
        rc.compute()
        m.compute()
        vals.append(float(m.sim_vals()[0]))
    gpu = len(poses) / (time.perf_counter() - t0)
    rc.close()
    cores = O.set_threads(os.cpu_count() or 1)
    geom, cams = oracle_geom(w.vol), oracle_cams(w.cams)
    done, t_used, diff = 0, 0.0, 0.0
    while done < len(poses) and (done == 0 or t_used < cpu_budget_s):
        t1 = time.perf_counter()
        d = O.drr_f32(w.vol.voxels, geom, cams, poses[done][None], step=w.step)
        v = float(O.ncc(fixed, d)[0])
        t_used += time.perf_counter() - t1
        diff = max(diff, abs(v - vals[done]))
        done += 1
    return {"workload": "128^3 FP32 @1.5 mm, 256^2 @1.55 mm, step 0.5 mm, NCC, one pose per evaluation",
            "gpu_plain_poses_per_s": round(gpu, 1),
            "how": "per pose: pose upload, DRR launch, NCC launches, host read (200 poses)",
            "cpu_oracle_poses_per_s": round(done / t_used, 2), "cpu_cores": cores,
            "cpu_sample": f"{done} poses, {t_used:.1f} s",
            "max_abs_ncc_diff_vs_oracle": diff}


def _extras(xr, w, fixed, dev, stream, poses, d_sims, a, flush, l2_peak):
    """Plain single-pose path (one DRR + one metric launch per pose, host sync per
    pose as xReg's OpenCL path does), half-precision volumes, dense sampling,
    errors against the oracle, and the other workloads, for context."""
    import torch
    out = {}
    try:
        out["errors_vs_oracle"] = _errors_vs_oracle(xr, w, fixed, dev, poses[:2])
    except Exception as e:  # reported, never fatal to the headline line
        out["errors_vs_oracle"] = {"error": f"{type(e).__name__}: {e}"}
    rc = xr.RayCasterLineIntCUDA(dev)
    rc.set_volume(w.vol)
    rc.set_camera_model(w.cams[0])
    rc.set_ray_step_size(w.step)
    rc.set_num_projs(1)
    rc.allocate_resources()
    m = xr.ImgSimMetric2DGradNCCCUDA(dev)
    m.set_fixed_image(fixed)
    m.set_num_moving_images(1)
    m.set_mov_imgs_buf_from_ray_caster(rc, 0)
    m.allocate_resources()
    vals = []
    n = 20
    for i in range(3):
        rc.distribute_xforms_among_cam_models(poses[i][None])
        rc.compute()
        m.compute()
        m.sim_vals()
    t0 = time.perf_counter()
    for i in range(n):
        rc.distribute_xforms_among_cam_models(poses[i][None])
        rc.compute()
        m.compute()
        vals.append(m.sim_vals()[0])
    plain = n / (time.perf_counter() - t0)
    out["plain_single_pose_fp32"] = {"value": round(plain, 2), "unit": "poses/s",
                                     "how": "per pose: pose upload, DRR launch, grad-NCC launches, host read"}
    ref = d_sims[a.warmup][:n].cpu().numpy()
    out["plain_single_pose_fp32"]["max_abs_diff_vs_batched"] = float(np.max(np.abs(np.array(vals) - ref)))
    # the same volume in half precision; then float32 with empty-space skipping
    # off, and float32 with CT-like air (noise of 10 HU about -1000: about half
    # of the air voxels convert to small positive attenuations, so only the
    # clamped half can be skipped)
    from xreg_gb300 import synth
    v_air = w.vol.voxels.copy()
    air = v_air == 0.0
    v_air[air] = synth.hu_to_lin_att(-1000.0 + np.random.default_rng(17).standard_normal(
        int(air.sum()), dtype=np.float32) * 10.0)
    noisy_air = dataclasses.replace(w.vol, voxels=v_air)
    brick = (3, 1, 1, 4)  # the brick-staged layout: each slab's cells copied to shared memory
    for key, vol_k, vt, skipping, cfg in (("batched_f16_volume", w.vol, 1, True, None),
                                          ("batched_bf16_volume", w.vol, 2, True, None),
                                          ("batched_f32_skipping_off", w.vol, 0, False, None),
                                          ("batched_f32_noisy_air", noisy_air, 0, True, None),
                                          ("batched_f16_noisy_air", noisy_air, 1, True, None),
                                          ("batched_bf16_noisy_air", noisy_air, 2, True, None),
                                          ("batched_f32_brick_staged", w.vol, 0, True, brick),
                                          ("batched_f32_brick_staged_skipping_off", w.vol, 0, False, brick)):
        rch = xr.RayCasterLineIntCUDA(dev)
        if cfg:
            rch.set_launch_config(*cfg)
        rch.set_stream(stream.cuda_stream)
        rch.set_volume(vol_k, vt)
        rch.set_empty_space_skipping(skipping)
        rch.set_camera_model(w.cams[0])
        rch.set_ray_step_size(w.step)
        mh = xr.ImgSimMetric2DGradNCCCUDA(dev)
        mh.set_fixed_image(fixed)
        objh = xr.PopulationObjective(rch, [mh], POP)
        dp = torch.from_numpy(poses.reshape(POP, 16).copy()).to(f"cuda:{dev}")
        ds = torch.empty(POP, dtype=torch.float32, device=f"cuda:{dev}")
        with torch.cuda.stream(stream):
            for _ in range(3):
                objh.eval_device(POP, dp.data_ptr(), ds.data_ptr())
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
        with torch.cuda.stream(stream):
            for s, e in evs:
                s.record(stream)
                objh.eval_device(POP, dp.data_ptr(), ds.data_ptr())
                e.record(stream)
        torch.cuda.synchronize()
        t = np.mean([s.elapsed_time(e) for s, e in evs]) / 1e3
        out[key] = {"value": round(POP / t, 2), "unit": "poses/s",
                    "max_abs_sim_diff_vs_f32": float(
                        np.max(np.abs(ds.cpu().numpy() - d_sims[a.warmup].cpu().numpy())))}
        if key.endswith("noisy_air"):
            out[key]["air_voxels_nonzero_frac"] = round(float(np.mean(v_air[air] > 0)), 3)
        if vt == 2:
            out[key]["tolerance"] = "BF16 volume: DRRs held to 2^-8 of the float32 oracle, outside the 2e-3 " \
                                    "half-precision tolerance"
        if key in ("batched_f32_skipping_off", "batched_f32_noisy_air") or cfg:
            ms_k, smp, ld = _drr_kernel_stats(rch, dp.data_ptr(), 5, stream, flush)
            lay = rch.launch_config_ex()
            rf = _roofline(vt, lay[0], ms_k, smp, ld, l2_peak, "")
            out[key]["drr_kernel"] = {k: rf[k] for k in ("achieved", "peak", "unit", "frac", "kernel_ms",
                                                         "samples_per_launch", "loaded_samples_per_launch",
                                                         "loaded_frac")}
        objh.close()
    del v_air, noisy_air
    for key, fn in (("plain_small_config", lambda: _plain_small(xr, dev, min(3.0, a.cpu_seconds))),
                    ("precision_large", lambda: _precision(xr, dev, stream)),
                    ("uneven_multi_job", lambda: _multi_job(xr, dev)),
                    ("serving", lambda: _serving(dev, a.serving_requests, _rates(a.serving_rates)))):
        if key == "serving" and a.serving_requests <= 0:
            continue
        try:
            out[key] = fn()
        except Exception as e:  # reported, never fatal to the headline line
            out[key] = {"error": f"{type(e).__name__}: {e}"}
    return out


def _precision(xr, dev, stream, pop: int = 20, reps: int = 5):
    """The precision workload (512x512x400 phantom at 0.8x0.8x1 mm, 1536^2 detector
    downsampled 2x to 768^2, patch grad-NCC 11x11 stride 1): population throughput
    for float32, FP16 and BF16 volumes, and the FP16 / BF16 DRR and similarity
    differences against the float32-volume path (errors against the FP64 oracle
    are checked by the full-size GPU tests)."""
    import torch
    from xreg_gb300 import synth
    w = synth.precision_large(0)
    rc = xr.RayCasterLineIntCUDA(dev)
    rc.set_volume(w.vol)
    rc.set_camera_models(w.cams)
    rc.set_ray_step_size(w.step)
    rc.set_num_projs(1)
    rc.allocate_resources()
    rc.distribute_xforms_among_cam_models(w.gt[None])
    rc.compute()
    fixed = synth.add_noise(rc.proj(0), 0.01, 3)
    rc.close()
    poses = synth.sample_poses(w.vol, w.gt, pop, 5.0, 10.0, seed=5)
    dp = torch.from_numpy(poses.reshape(pop, 16).copy()).to(f"cuda:{dev}")
    out = {"volume": "512x512x400 @0.8x0.8x1 mm", "detector": "768x768", "metric": "patch grad-NCC 11x11 stride 1",
           "pop": pop}
    ref_drr = ref_sims = None
    from oracle import oracle as O
    from tests.helpers import oracle_cams, oracle_geom
    O.set_threads(os.cpu_count() or 1)
    o_geom, o_cams = oracle_geom(w.vol), oracle_cams(w.cams)
    o32 = O.drr_f32(w.vol.voxels, o_geom, o_cams, poses[:1], step=w.step)[0]
    o64 = O.drr_f64(w.vol.voxels, o_geom, o_cams, poses[:1], step=w.step)[0]
    o_body = o64 > 0.1 * o64.max()
    o_sim = float(O.patch_grad_ncc(fixed, o32[None], smooth_ksize=5, radius=5, stride=1)[0])
    for vname, vt in (("f32", 0), ("f16", 1), ("bf16", 2)):
        rcv = xr.RayCasterLineIntCUDA(dev)
        rcv.set_stream(stream.cuda_stream)
        rcv.set_volume(w.vol, vt)
        rcv.set_camera_models(w.cams)
        rcv.set_ray_step_size(w.step)
        m = xr.ImgSimMetric2DPatchGradNCCCUDA(dev)
        m.set_fixed_image(fixed)
        obj = xr.PopulationObjective(rcv, [m], pop)
        ds = torch.empty(pop, dtype=torch.float32, device=f"cuda:{dev}")
        with torch.cuda.stream(stream):
            for _ in range(2):
                obj.eval_device(pop, dp.data_ptr(), ds.data_ptr())
        stream.synchronize()
        drr = rcv.projs()[0].copy()
        sims = ds.cpu().numpy().copy()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        with torch.cuda.stream(stream):
            for s0, e0 in evs:
                s0.record(stream)
                obj.eval_device(pop, dp.data_ptr(), ds.data_ptr())
                e0.record(stream)
        torch.cuda.synchronize()
        t = float(np.mean([s0.elapsed_time(e0) for s0, e0 in evs])) / 1e3
        entry = {"poses_per_s": round(pop / t, 2)}
        nz = o32 != 0
        entry["errors_vs_oracle_pose0"] = {
            "drr_max_rel_vs_fp32_oracle": float(np.max(np.abs(drr[nz] - o32[nz]) / o32[nz])),
            "drr_max_rel_vs_fp64_oracle_body": float(np.max(np.abs(drr[o_body] - o64[o_body]) / o64[o_body])),
            "drr_median_rel_vs_fp64_oracle_body": float(np.median(np.abs(drr[o_body] - o64[o_body]) / o64[o_body])),
            "patch_grad_ncc_abs_vs_oracle_fp32_drr": abs(float(sims[0]) - o_sim)}
        if ref_drr is None:
            ref_drr, ref_sims = drr, sims
        else:
            body = ref_drr > 0.1 * ref_drr.max()
            entry["drr_max_rel_diff_vs_f32_over_body"] = float(np.max(np.abs(drr[body] - ref_drr[body]) / ref_drr[body]))
            entry["sim_max_abs_diff_vs_f32"] = float(np.max(np.abs(sims - ref_sims)))
        out[vname] = entry
        obj.close()
    return out


def _multi_job(xr, dev, steps: int = 5, njobs: int = 8):
    """8 concurrent registrations of uneven size (volumes 192^3 .. 512x512x300,
    1-3 views, detector 4x or 8x downsampled, lambda 20-100; FP16 volumes), one
    population per job per optimizer step: one job-set call per step (geometry,
    one DRR launch, one batched grad-NCC launch), the fused job-set
    step beside it, and the same populations evaluated job by job."""
    from xreg_gb300 import synth
    specs = synth.uneven_job_specs(njobs, seed=4)
    objs, poses_sets, total = [], [], 0
    for sp in specs:
        vol = synth.phantom_volume(sp.size, sp.spacing, sp.seed)
        cams = synth.view_cameras(sp.view_angles, sp.ds_first)
        gt = synth.gt_pose(vol)
        fixed = synth.render_fixed(vol, cams, gt, 0.5, sp.seed, dev)
        rc = xr.RayCasterLineIntCUDA(dev)
        rc.set_volume(vol, 1)
        rc.set_camera_models(cams)
        rc.set_ray_step_size(0.5)
        ms = []
        for f in fixed:
            m = xr.ImgSimMetric2DGradNCCCUDA(dev)
            m.set_fixed_image(f)
            ms.append(m)
        objs.append(xr.PopulationObjective(rc, ms, sp.pop))
        poses_sets.append([synth.sample_poses(vol, gt, sp.pop, 10.0, 20.0, seed=sp.seed + 100 + k)
                           for k in range(steps + 1)])
        total += sp.pop
    js = xr.JobSet(dev)
    js.eval(objs, [p[0] for p in poses_sets])  # warm-up
    for o, p in zip(objs, poses_sets):
        o.eval(p[0])
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        mixed = js.eval(objs, [p[k] for p in poses_sets])
    t_mixed = time.perf_counter() - t0
    launches = js.last_kernel_launches()
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        alone = [o.eval(p[k]) for o, p in zip(objs, poses_sets)]
    t_alone = time.perf_counter() - t0
    # the fused step: geometry, then one DRR + grad-NCC launch per voxel group
    js.set_fused(True)
    js.eval(objs, [p[0] for p in poses_sets])
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        fused = js.eval(objs, [p[k] for p in poses_sets])
    t_fused = time.perf_counter() - t0
    fused_launches = js.last_kernel_launches()
    js.set_fused(False)
    same = all(np.array_equal(x, y) for x, y in zip(mixed, alone)) and \
        all(np.array_equal(x, y) for x, y in zip(mixed, fused))
    # one pose of the largest job against the oracle (its DRRs from the last job-set call)
    errs = None
    try:
        from oracle import oracle as O
        from tests.helpers import oracle_cams, oracle_geom
        big = int(np.argmax([np.prod(sp.size) * len(sp.view_angles) for sp in specs]))
        sp, ob = specs[big], objs[big]
        jvol = synth.phantom_volume(sp.size, sp.spacing, sp.seed)
        jcams = synth.view_cameras(sp.view_angles, sp.ds_first)
        nv = len(jcams)
        p0 = poses_sets[big][steps][0]
        ref = O.drr_f32(jvol.voxels, oracle_geom(jvol), oracle_cams(jcams), np.stack([p0] * nv),
                        cam_idx=list(range(nv)), step=0.5)
        g = ob.rc.projs()
        got = np.stack([g[v * sp.pop] for v in range(nv)])
        nz = ref != 0
        errs = {"job": f"{sp.size[0]}x{sp.size[1]}x{sp.size[2]} v{nv} ds{int(round(1 / sp.ds_first))} FP16 volume",
                "drr_max_rel_vs_fp32_oracle": float(np.max(np.abs(got[nz] - ref[nz]) / ref[nz])),
                "background_equal": bool(np.all(got[~nz] == 0)), "drr_tolerance": 2e-3}
    except Exception as e:
        errs = {"error": f"{type(e).__name__}: {e}"}
    return {"value": round(steps * total / t_mixed, 2), "unit": "poses/s",
            "errors_vs_oracle_largest_job_pose0": errs,
            "one_job_at_a_time": round(steps * total / t_alone, 2),
            "fused_step": round(steps * total / t_fused, 2),
            "kernel_launches_per_step": launches, "fused_step_kernel_launches": fused_launches,
            "ms_per_step": round(1e3 * t_mixed / steps, 3), "jobs": njobs, "poses_per_step": total,
            "identical_to_alone": bool(same),
            "job_shapes": [f"{s.size[0]}x{s.size[1]}x{s.size[2]} v{len(s.view_angles)} "
                           f"ds{int(round(1 / s.ds_first))} pop{s.pop}" for s in specs],
            "how": "host poses in, host values out, one job-set call per step (wall clock)"}


SERVING_RATES = (2.0, 4.0, 8.0, 16.0, 32.0, 50.0)
SERVING_TOL = (0.05, 0.1)  # deg, mm: the registration tolerance the path is specified with


def _rates(text: str) -> tuple:
    return tuple(float(x) for x in text.split(",") if x.strip())


def _serving(dev, n_req: int, rates=SERVING_RATES):
    """Steady-state serving: at each arrival rate, n_req two-level registration
    requests arrive as a Poisson process (8x CMA-ES up to 150 iterations, then
    4x BOBYQA-style level of up to 100 evaluations after its 2n+1 initial ones;
    grad-NCC; FP16 volumes).  Requests are drawn from 12 patients of the uneven
    multi-job sizes (volumes 192^3 .. 512x512x300, 1-3 views), each request
    with its own start pose (N(0, 5 deg) / N(0, 10 mm) from the truth) and
    optimizer seed; CMA-ES state on the device.  Requests are prepared before
    the clock starts; latency runs from arrival to completion (queue wait =
    arrival to admission, service = admission, including the volume upload,
    to completion).  The saturation throughput is the highest completion rate
    measured."""
    from xreg_gb300 import synth
    from xreg_gb300.regi import pose_error
    from xreg_gb300.serving import RegistrationServer
    specs = synth.uneven_job_specs(12, seed=5)
    templates = []
    for sp in specs:
        sp.ds_first = 0.125
        templates.append(synth.job_registration(sp, iters=(150, 100), level2_pop=8, voxel_type=1, device=dev))
    reqs = []
    for i in range(n_req):
        t, gt = templates[i % len(templates)]
        reqs.append((synth.request_like(t, gt, 7000 + i), gt))
    jobs = [r for r, _ in reqs]

    def one_run(r):
        for j in jobs:
            j.reset()
        rng = np.random.default_rng(int(r * 1000) + 6)
        offsets = np.cumsum(rng.exponential(1.0 / r, n_req))
        srv = RegistrationServer(dev, hbm_budget_bytes=180e9)
        with ClockSampler(dev) as clk:
            clk.wait_started()
            t0 = time.perf_counter()
            st = srv.run(arrivals=list(zip(offsets.tolist(), jobs)))
            makespan = time.perf_counter() - t0
        srv.close()
        errs = np.array([pose_error(j.final_pose, gt, j.vol) for j, gt in reqs])
        within = int(np.sum((errs[:, 0] <= SERVING_TOL[0]) & (errs[:, 1] <= SERVING_TOL[1])))
        s = st.summary()
        return {"arrival_rate_per_s": r, "requests": n_req, "completed": s["completed"],
                "p50_latency_s": round(s["p50_s"], 3), "p99_latency_s": round(s["p99_s"], 3),
                "queue_wait_p50_s": round(s["queue_wait_p50_s"], 3), "queue_wait_p99_s": round(s["queue_wait_p99_s"], 3),
                "service_p50_s": round(s["service_p50_s"], 3), "service_p99_s": round(s["service_p99_s"], 3),
                "registrations_per_s": round(s["completed"] / makespan, 3), "makespan_s": round(makespan, 3),
                "poses_evaluated": s["poses_evaluated"], "server_steps": s["steps"], "max_active": s["max_active"],
                "step_s": round(s["busy_s"], 3), "max_footprint_gb": round(s["max_footprint_gb"], 2),
                "within_tolerance": within,
                "pose_error_deg_median": round(float(np.median(errs[:, 0])), 4),
                "pose_error_mm_median": round(float(np.median(errs[:, 1])), 4),
                "pose_error_deg_max": round(float(errs[:, 0].max()), 4),
                "pose_error_mm_max": round(float(errs[:, 1].max()), 4),
                "clocks": clk.summary()}

    runs = [one_run(r) for r in rates]
    return {"rates": runs, "requests_per_rate": n_req, "patients": len(templates),
            "saturation_registrations_per_s": max(d["registrations_per_s"] for d in runs),
            "all_within_tolerance": all(d["within_tolerance"] == n_req for d in runs),
            "tolerance_deg_mm": list(SERVING_TOL),
            "generation_step": "one xr_regi_jobset_step call per server step: device CMA-ES sampling in the "
                               "geometry launch, DRR launch, grad-NCC launch with the CMA-ES update"}


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    """Maximum of x over the ranks (the slowest replica sets the time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _config_fields(step_mm: float, voxel: str) -> dict:
    """The workload as both arms name it."""
    return {"workload": "batched population: 256^3 phantom @1 mm, 1536^2@0.194 mm detector ds 4x -> 384^2, "
                        "lambda=100, grad-NCC 5x5 Gaussian + Sobel",
            "volume": "256x256x256 " + voxel, "detector": "384x384", "pop": POP, "step_mm": step_mm}


def _config(w, voxel: str) -> dict:
    return _config_fields(w.step, voxel)


def run_reference(a, rank, world):
    """The reference's CPU path timed on the host cores, on the same workload:
    every step evaluates one full population of lambda = 100 poses (DRR +
    grad-NCC).  xReg's ray caster cannot be compiled here (ITK, Eigen, OpenCV,
    TBB absent), so its restatement in C (oracle/) runs, with all host threads.
    Nothing of the product is imported or loaded on this path; the inputs come
    from oracle/workload.py (the same seeded generators)."""
    if rank != 0:
        return None
    from oracle import oracle as O
    from oracle import workload as W
    w = W.Batched(0, POP)
    cores = O.set_threads(os.cpu_count() or 1)
    fixed = W.add_noise(O.drr_f32(w.voxels, w.geom, w.cams, w.fixed_pose()[None], step=w.step)[0], 0.01,
                        w.seed + 2)
    pops = w.populations(a.warmup + a.steps, 1234)

    def one_step(k):
        d = O.drr_f32(w.voxels, w.geom, w.cams, pops[k], step=w.step)
        O.grad_ncc(fixed, d)

    for k in range(a.warmup):
        one_step(k)
    t0 = time.perf_counter()
    for k in range(a.steps):
        one_step(a.warmup + k)
    t = time.perf_counter() - t0
    v = a.steps * POP / t
    cfg = _config_fields(w.step, "f32")
    return {
        "impl": "reference",
        "metric": "poses/sec (DRR+grad-NCC pose evaluations, batched population)",
        "value": round(v, 3), "unit": "poses/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": round(t * 1e3 / a.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, sampled poses, noisy fixed DRR)",
        "config": dict(cfg, parallelism="rank 0 on the host cores"),
        "cpu_baseline": {"value": round(v, 3), "unit": "poses/s", "cores": cores, "kind": "port",
                         "sample": f"{a.steps} full populations of {POP} poses; xReg's CPU ray caster + grad-NCC "
                                   "restated in C (the reference needs ITK/OpenCV/TBB, absent here)"},
        "e2e": {"value": round(v, 3), "unit": "poses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "product_loaded": _product_loaded(),
    }


def _product_loaded() -> bool:
    """Whether this process imported the product package or mapped its library."""
    if any(m == "xreg_gb300" or m.startswith("xreg_gb300.") for m in sys.modules):
        return True
    try:
        with open("/proc/self/maps") as f:
            return "libxreg_gb300" in f.read()
    except OSError:
        return False


def main():
    faulthandler.enable()
    a = _args()
    rank, world, local = _dist()
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "gloo" if a.impl == "reference" else "nccl"
        if a.impl != "reference":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    if a.only:
        import torch
        import xreg_gb300 as xr
        torch.cuda.set_device(local)
        xr.load()
        fn = {"plain-small": lambda: _plain_small(xr, local, min(3.0, a.cpu_seconds)),
              "precision": lambda: _precision(xr, local, torch.cuda.Stream(device=local)),
              "multi-job": lambda: _multi_job(xr, local),
              "serving": lambda: _serving(local, a.serving_requests, _rates(a.serving_rates))}[a.only]
        res = {"only": a.only, "result": fn()} if rank == 0 else None
    elif a.impl == "reference":
        res = run_reference(a, rank, world)
    else:
        res = run_ours(a, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
