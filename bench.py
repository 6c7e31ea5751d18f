"""Benchmark: closest-hit Mrays/s on the terrain ray-cast workload, 1 GB300 per rank.

Workload (one "step"): closest-hit traversal of 4,194,304 coherent primary rays (2048 x 2048
pinhole camera, pixel centres) and 4,194,304 incoherent rays (cosine-distributed about the
first-hit normals, hashed resampling of hit pixels) against a 1024 x 1024-cell fBm heightfield
(2,097,152 triangles, seed 7, world scale 8) in the reference's compact SBVH layout
(split alpha 1e-5, leaf <= 8). Inputs are resident in HBM; rays (256 MB) and the BVH (~330 MB)
are each larger than the 129 MB L2, and L2 is additionally flushed (a 256 MB write) between
timed steps, outside the timed region.

  value     Mrays/s over both ray sets, device-resident inputs, CUDA events on the stream
  e2e       the same through tt_trace_host (host buffers; H2D of the rays and D2H of the hits
            inside the timed region, page-locked host memory)
  cache     the metric's second half at a reduced size (multi-material scene, 960 x 540): time
            to relMSE levels for the plain tracer and the learned radiance cache, three seeds, against
            an FP64 reference whose own error is reported (--cache-seconds 0 skips it)
  ref_kernel  the reference's own CUDA intersect() on the same BVH and rays, Mrays/s per ray set
  roofline  the traversal kernel: algorithmic bytes per ray (ray 32 + hit 8 + 64 per inner
            node + 16 per leaf + 48 per triangle tested + 56 per accepted hit update, counts
            from the oracle's instrumented restatement on the same rays) over the
            measured kernel time, against the measured HBM copy bandwidth
  cpu_baseline  the reference's traversal restated in C (oracle/, plain float arithmetic like
            the reference's host build) under OpenMP on all host cores, on all 8,388,608 rays,
            repeated for at least 10 s (--impl reference: one pass of all rays per step)

Other workloads (--workload; one JSON line each, same keys):
  cornell        unit Cornell box + displaced subdivision-5 icosphere (20,492 tris), 512 x 512,
                 16 spp, depth 8, Russian roulette from 4: Msamples/s of the native path tracer
  multimaterial  400 displaced subdivision-5 icospheres (8,192,002 tris) with Lambert / GGX /
                 dielectric materials under a 2048 x 1024 sky with a 0.5 degree sun of 5e4,
                 1920 x 1080, 64 spp, depth 16: Msamples/s
  batch          64 orbit views of the terrain (sizes 256^2..1024^2, 4/16/64 spp) as one
                 graph-captured batch with an autotuned launch shape, against 64 sequential renders
  cache          time to relMSE 0.01 against a 16,384-spp FP64 render, plain tracer versus the
                 learned radiance cache (multimaterial scene; --cache-scene terrain for the terrain)
  mlp            the radiance cache's BF16 tensor-core kernels alone (inference on 2^21 records,
                 one frame's training): TFLOP/s against the measured BF16 peak

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload W]
Multi-GPU (torchrun): every rank is an independent replica tracing its own rays (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_CELLS = 1024
SCALE = 8.0
WIDTH = 2048
SHADOW_LIGHT = [8.0 * SCALE, 2.0 * SCALE, 0.0]  # the point (8, 2, 0) of the unit terrain
METRIC = "Mrays/s closest-hit; time to relMSE 0.01, cached vs plain tracer, 1 GB300"
UNIT = "Mrays/s"
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the trace kernel of
# this workload (the default, ray-ordered variant), the mean of the primary (293.1 MB) and
# incoherent (328.8 MB) launches ncu captured of `bench.py --steps 2 --warmup 3` on a GB300; the
# ordering kernels around them add 8 MB (primary: the probe only) and 523 MB (incoherent: probe,
# keys, scan, ordered copy, hit gather). bench.py cannot run ncu itself.
TRACE_DRAM_BYTES_PER_LAUNCH = 311_000_000
# L2 of the same GB300 from one ncu capture of the incoherent trace launch (1M rays, the current
# 10-block build): 74.89 sectors/ns were 6.59 % of the sustained peak, i.e. 1,136 sectors/ns x 32 B;
# the launch's own L2 traffic was that 6.6 % of it
TRACE_L2_PEAK_GBS = 36_370.0
TRACE_L2_TRAFFIC_PCT = 6.6


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# the SIMD efficiency and the L2 figures of the trace kernel from the same committed ncu capture
# (profiles/trace_kernel_terrain_closest.md, incoherent launch): threads per executed instruction
TRACE_THREADS_PER_INST = 9.06


def terrain_config(n_rays: int) -> dict:
    """The workload description both arms print (the same dict, so the lines compare)."""
    return {"workload": "terrain ray-cast: 1024x1024-cell fBm heightfield, 2,097,152 tris, world scale 8; "
                        f"{n_rays // 2:,} coherent primary + {n_rays // 2:,} incoherent rays, closest hit",
            "bvh": "compact SBVH, split alpha 1e-5, leaf <= 8", "rays_per_step": n_rays,
            "l2": "inputs larger than L2; L2 also flushed (256 MB write) between GPU steps, untimed"}


def reference_workload(width: int = WIDTH) -> dict:
    """The terrain workload built by the oracle alone (no libtt.so): the mesh from the numpy scene
    generators, the BVH by the oracle's restatement of the reference's single-threaded SBVH builder
    (timed), the incoherent rays spawned from the first hits of the oracle's traversal in the
    reference kernel's arithmetic (so the rays are those of the GPU arm, bit for bit)."""
    from oracle import oracle
    from trenchanttracer_gb300 import scenes  # numpy only; loads no library
    mesh = scenes.terrain(N_CELLS, SCALE)
    with tempfile.TemporaryDirectory() as d:
        build_s = oracle.sbvh_build(mesh.vertices, mesh.normals, mesh.vidx, mesh.nidx, mesh.mat,
                                    Path(d) / "bvh.cache", 1e-5, 1, 8)
        arr = oracle.read_cache(Path(d) / "bvh.cache")
    cam = scenes.terrain_camera(SCALE)
    primary = scenes.pinhole_rays(width, width, cam["eye"], cam["target"], cam["tan_half_fov"])
    first = oracle.intersect(arr, primary, True, arith=oracle.DEVICE, normals=True)
    secondary, _ = scenes.secondary_rays(primary, first["t"], first["normal"], primary.shape[0], 11, 1e-4 * SCALE)
    return {"arrays": arr, "primary": primary, "secondary": secondary, "build_s": build_s, "mesh": mesh}


def workload(trace_ext=None, width: int = WIDTH):
    """Scene, BVH and the two ray sets (width^2 rays each). trace_ext(rays) -> (t, normal) gives
    the first hits from which the incoherent rays are spawned (the product's own kernel on the
    GPU arm)."""
    from trenchanttracer_gb300 import BVHCompact, Scene, scenes
    mesh = scenes.terrain(N_CELLS, SCALE)
    bvh = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8)
    cam = scenes.terrain_camera(SCALE)
    primary = scenes.pinhole_rays(width, width, cam["eye"], cam["target"], cam["tan_half_fov"])
    t, normal = trace_ext(bvh, primary)
    secondary, _ = scenes.secondary_rays(primary, t, normal, primary.shape[0], 11, 1e-4 * SCALE)
    # shadow rays from first hits to the point (8, 2, 0) of the unit terrain, tmax = the distance
    shadow = scenes.shadow_rays(primary, t, SHADOW_LIGHT, primary.shape[0], 5, 1e-4 * SCALE)
    return mesh, bvh, primary, secondary, shadow


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = sorted(float(r[1]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


def trace_call_launches(dbvh) -> int:
    """Kernels one DeviceBVH.intersect call launches: with the ray-ordered variants the ordering
    probe, keys, scan and scatter, the trace and the hit gather (the ordering kernels return at
    once when the probe finds the rays coherent, but they are still launched); otherwise the
    trace alone."""
    return 6 if dbvh.variant in (dbvh.VARIANT_SORTED, dbvh.VARIANT_SORTED_OCC) else 1


def bytes_per_ray(counters: np.ndarray) -> float:
    """Algorithmic bytes per ray from the oracle's (node, leaf, tri, hit-update) counts."""
    c = counters.astype(np.float64).mean(axis=0)
    return 32.0 + 8.0 + 64.0 * c[0] + 16.0 * c[1] + 48.0 * c[2] + 56.0 * c[3]


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the architecture)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_baseline(bvh_arrays: dict, rays: np.ndarray, stride: int, want_counters: bool, min_seconds: float = 0.0) -> dict:
    """The oracle (plain arithmetic, OpenMP on all host cores) on every stride-th ray, repeated
    until at least min_seconds have passed (one pass at least); traversal counters from a
    separate untimed pass."""
    from oracle import oracle
    sub = np.ascontiguousarray(rays[::max(1, stride)])
    threads = oracle.max_threads()
    oracle.intersect(bvh_arrays, sub[:4096], True, arith=oracle.PLAIN, threads=threads)  # warm
    counters = None
    if want_counters:
        counters = oracle.intersect(bvh_arrays, sub, True, arith=oracle.PLAIN, threads=threads,
                                    counters=True)["counters"]
    passes = 0
    t0 = time.perf_counter()
    while True:
        oracle.intersect(bvh_arrays, sub, True, arith=oracle.PLAIN, threads=threads)
        passes += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    return {"mrays": passes * sub.shape[0] / dt / 1e6, "rays": int(sub.shape[0]), "passes": passes,
            "seconds": dt, "threads": threads, "counters": counters}


def rank_info() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time: every rank times its own replica; the job takes as long as the
    slowest one (all_reduce MAX over the default process group when world > 1)."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms: float, world: int) -> float:
    """The whole job's throughput in millions of units per second when each of `world`
    replicas processes `units_per_rank` units in `ms` milliseconds."""
    return world * units_per_rank / ms / 1e3


def host_sbvh_build_seconds(mesh) -> dict:
    """The terrain's SBVH build on the host: the oracle's single-threaded restatement of the
    reference's builder, and this project's builder (OpenMP subtrees, same bytes)."""
    from oracle import oracle
    from trenchanttracer_gb300 import BVHCompact, Scene
    with tempfile.TemporaryDirectory() as d:
        oracle_s = oracle.sbvh_build(mesh.vertices, mesh.normals, mesh.vidx, mesh.nidx, mesh.mat,
                                     Path(d) / "bvh.cache", 1e-5, 1, 8)
    sc = Scene.from_mesh(mesh)
    t0 = time.perf_counter()
    BVHCompact.build(sc, 1e-5, 1, 8)
    return {"oracle_s": round(oracle_s, 2), "ours_s": round(time.perf_counter() - t0, 3)}


def reference_kernel_rates(bvh_arrays: dict, sets: dict, reps: int = 7) -> dict:
    """The reference's own CUDA intersect() (oracle/_ref/ref_intersect.cubin: the reference source
    with its one-line ballot shim, one ray per thread, 256 threads per block) on this GB300, same
    BVH and rays: Mrays/s per ray set, closest and any hit, from the median of `reps` back-to-back
    launches (CUDA events)."""
    from oracle import refgpu
    if not refgpu.available():
        return {"unavailable": "oracle/_ref/ref_intersect.cubin was not built (the reference checkout is absent)"}
    out = {}
    for name, rays in sets.items():
        for closest in (True, False):
            r = refgpu.intersect(bvh_arrays, rays, closest, reps=reps)
            out[f"{name}_{'closest' if closest else 'any'}_mrays"] = round(rays.shape[0] / r["ms"] / 1e3, 1)
    out["kernel"] = "the reference's intersect() compiled for sm_103a from its own source, one ray per thread"
    return out


def run_reference(args) -> None:
    """--impl reference: the reference's host path on the host cores, built only from the oracle
    (no libtt.so): its SBVH build restated single-threaded as the reference runs it (timed once,
    reported in cpu_baseline) and its traversal with the reference's plain float arithmetic under
    OpenMP on all host threads (timed per step), on this arm's workload and metric."""
    _, rank, _ = rank_info()
    if rank != 0:
        return
    from oracle import oracle
    w = reference_workload()
    arr = w["arrays"]
    rays = np.concatenate([w["primary"], w["secondary"]])
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(arr, rays, 1, False)
        if i >= args.warmup:
            vals.append(r["mrays"])
            secs.append(r["seconds"])
    v = float(np.median(vals))
    cores = oracle.max_threads()
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.median(secs)) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm terrain, seed 7; rays seeded)",
            "config": terrain_config(rays.shape[0]),
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                             "sample": f"all {r['rays']:,} rays of both sets per step, "
                                       f"{float(np.median(secs)):.2f} s per step",
                             "sbvh_build_s": round(w["build_s"], 2),
                             "sbvh_build": "the reference's SBVH build + compact emission restated in C "
                                           "(oracle/tt_oracle_sbvh.c, byte-identical bvh.cache), 1 thread "
                                           "as the reference builds"},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    world, rank, local = rank_info()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from trenchanttracer_gb300 import DeviceBVH, hits_to_numpy

    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    state = {}

    def gpu_ext(bvh, rays):
        d = DeviceBVH(bvh)
        state["dbvh"] = d
        dr = torch.from_numpy(rays).to(dev)
        dh = torch.empty((rays.shape[0], 6), dtype=torch.int32, device=dev)
        d.intersect(dr, dh, closest=True, ext=True, stream=stream.cuda_stream)
        torch.cuda.synchronize(dev)
        d.check(stream.cuda_stream)
        h = dh.cpu().numpy()
        return h[:, 2].copy().view(np.float32), h[:, 3:6].copy().view(np.float32)

    mesh, bvh, primary, secondary, shadow = workload(gpu_ext, args.trace_width)
    dbvh = state["dbvh"]
    sets = [torch.from_numpy(primary).to(dev), torch.from_numpy(secondary).to(dev)]
    hits = [torch.empty((s.shape[0], 2), dtype=torch.int32, device=dev) for s in sets]
    n_rays = sum(s.shape[0] for s in sets)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    s = stream.cuda_stream

    def step(evs=None):
        for i, (r, h) in enumerate(zip(sets, hits)):
            if evs is not None:
                evs[2 * i].record(stream)
            dbvh.intersect(r, h, closest=True, stream=s)
            if evs is not None:
                evs[2 * i + 1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    dbvh.check(s)
    step_ms, launch_ms = [], [[], []]
    with Clocks(local) as clk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)
        for _ in range(args.steps):
            flush.fill_(1)  # L2 flush, outside the timed events
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            step(evs)
            torch.cuda.synchronize(dev)
            step_ms.append(evs[0].elapsed_time(evs[3]))
            launch_ms[0].append(evs[0].elapsed_time(evs[1]))
            launch_ms[1].append(evs[2].elapsed_time(evs[3]))
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()
    dbvh.check(s)
    clocks = clk.summary()
    ms = max_over_ranks(float(np.sum(step_ms)) / args.steps, world, dev)
    value = whole_job_rate(n_rays, ms, world)  # whole-job Mrays/s

    # any hit on both sets and on the shadow rays (not part of the closest-hit value)
    any_hit = {}
    for name, rr in (("primary", sets[0]), ("incoherent", sets[1]), ("shadow", torch.from_numpy(shadow).to(dev))):
        hh = torch.empty((rr.shape[0], 2), dtype=torch.int32, device=dev)
        for _ in range(3):
            dbvh.intersect(rr, hh, closest=False, stream=s)
        ts = []
        for _ in range(max(3, args.steps // 2)):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dbvh.intersect(rr, hh, closest=False, stream=s)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        any_hit[f"{name}_mrays"] = round(rr.shape[0] / float(np.median(ts)) / 1e3, 1)
        if name == "shadow":
            any_hit["shadow_occluded_fraction"] = round(float((hh[:, 0] >= 0).float().mean().item()), 4)
    dbvh.check(s)

    # end to end through the host-buffer entry point (pinned host memory)
    h_sets = [torch.from_numpy(primary).pin_memory(), torch.from_numpy(secondary).pin_memory()]
    h_hits = [torch.empty((x.shape[0], 2), dtype=torch.int32).pin_memory() for x in h_sets]
    from trenchanttracer_gb300 import _lib
    import ctypes as C

    def e2e_step():
        for hr, hh in zip(h_sets, h_hits):
            _lib.check(_lib.lib().tt_trace_host(dbvh._h, C.c_void_p(hr.data_ptr()), hr.shape[0],
                                                 C.c_void_p(hh.data_ptr()), 1, C.c_void_p(s)))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = whole_job_rate(n_rays, max_over_ranks(float(np.mean(e2e_ms)), world, dev), world)
    # device and host paths agree bit for bit
    ids_d, t_d = hits_to_numpy(hits[1].cpu().numpy())
    ids_h, t_h = hits_to_numpy(h_hits[1].numpy())
    assert np.array_equal(ids_d, ids_h) and np.array_equal(t_d.view(np.uint32), t_h.view(np.uint32))

    if rank != 0:
        return
    peaks = load_peaks()
    cpu = cpu_baseline(bvh.arrays(), np.concatenate([primary, secondary]), 1, True, min_seconds=10.0)
    host_build = host_sbvh_build_seconds(mesh)
    cache_line = cache_target(seconds=args.cache_seconds) if args.cache_seconds > 0 else None
    ref_kernel = reference_kernel_rates(bvh.arrays(), {"primary": primary, "incoherent": secondary, "shadow": shadow})
    bpr = bytes_per_ray(cpu["counters"])
    kernel_ms = (np.mean(launch_ms[0]) + np.mean(launch_ms[1])) / 2.0
    achieved = bpr * (n_rays / 2) / (kernel_ms * 1e-3) / 1e9
    hit_frac = float((ids_d >= 0).mean())
    ids_p, _ = hits_to_numpy(hits[0].cpu().numpy())
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm terrain, seed 7; rays seeded)",
        "config": terrain_config(n_rays), "parallelism": f"replicas x{world}",
        "per_set": {"primary_mrays": round(sets[0].shape[0] / np.mean(launch_ms[0]) / 1e3, 1),
                    "incoherent_mrays": round(sets[1].shape[0] / np.mean(launch_ms[1]) / 1e3, 1),
                    "primary_hit_fraction": round(float((ids_p >= 0).mean()), 4),
                    "incoherent_hit_fraction": round(hit_frac, 4)},
        "any_hit": dict(any_hit, light=SHADOW_LIGHT),
        "e2e": {"value": round(e2e_val, 2), "unit": UNIT, "h2d_bytes_per_step": int(n_rays * 32),
                "d2h_bytes_per_step": int(n_rays * 8)},
        "roofline": {"binding": "issue and latency of divergent traversal: DRAM at 4 % of its peak, real L2 traffic "
                                f"at {TRACE_L2_TRAFFIC_PCT} % of its peak, issue on 59 % of cycles with "
                                f"{TRACE_THREADS_PER_INST} of 32 lanes per instruction (ncu, incoherent launch)",
                     "l2": {"frac": round(achieved / TRACE_L2_PEAK_GBS, 4), "achieved": round(achieved, 1),
                            "peak": TRACE_L2_PEAK_GBS, "unit": "GB/s", "l2_traffic_pct_of_peak": TRACE_L2_TRAFFIC_PCT,
                            "peak_source": "ncu: lts__t_sectors.sum.per_second / lts__t_sectors.sum.pct_of_peak_"
                                           "sustained_elapsed x 32 B, incoherent trace launch"},
                     "simd_efficiency": {"frac": round(TRACE_THREADS_PER_INST / 32.0, 4),
                                         "threads_per_instruction": TRACE_THREADS_PER_INST,
                                         "source": "ncu smsp__thread_inst_executed_per_inst_executed, incoherent "
                                                   "trace launch (profiles/trace_kernel_terrain_closest.md)"},
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": TRACE_DRAM_BYTES_PER_LAUNCH,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per trace launch of this "
                                       "workload (mean of the primary and incoherent launches)",
                     "peak_source": f"{peaks['source']} hbm_gbs (MEASURED_PEAKS.json)" if peaks["source"] == "measured"
                     else "fallback 6.8 TB/s", "bytes_per_ray": round(bpr, 1),
                     "kernel": "tt_trace: ray ordering + trace_warp_kernel<closest> (avg per ray set)",
                     "avg_launch_ms": round(float(kernel_ms), 4)},
        "ref_kernel": ref_kernel,
        "cache": cache_line,
        "cpu_baseline": {"value": round(cpu["mrays"], 3), "unit": UNIT, "cores": cpu["threads"], "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"all {cpu['rays']:,} rays of both sets, {cpu['passes']} passes, "
                                   f"{cpu['seconds']:.1f} s",
                         "sbvh_build_s": host_build["oracle_s"],
                         "sbvh_build": "the reference's SBVH build + compact emission restated in C "
                                       "(oracle/tt_oracle_sbvh.c, byte-identical bvh.cache), 1 thread as the "
                                       "reference builds",
                         "sbvh_build_s_ours": host_build["ours_s"]},
        "clocks": clocks,
        "gpu_launches": 2 * args.steps * trace_call_launches(dbvh),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---- path-tracing workloads ----------------------------------------------------------------------
RENDER_CONFIGS = {
    "cornell": dict(desc="Cornell box (10 wall tris + 0.25 x 0.25 ceiling light 17,12,4) + subdivision-5 "
                         "icosphere r 0.3 (seed-42 noise 0.03, Lambert 0.8), 20,492 tris; 512 x 512, 16 spp, "
                         "depth 8, Russian roulette from 4, PCG32", width=512, height=512, spp=16, depth=8),
    "multimaterial": dict(desc="400 displaced subdivision-5 icospheres (8,192,002 tris incl. ground), Lambert / "
                               "GGX / dielectric 1.5; 2048 x 1024 sky with a 0.5-degree sun of 5e4, 2D-CDF light "
                               "sampling with MIS; 1920 x 1080, 64 spp, depth 16, Russian roulette from 4",
                          width=1920, height=1080, spp=64, depth=16),
}
# The launch shape of a render (threads, shared stack, wave or pool size, ordered queues, streamed)
# is picked by the batch autotuner on the view itself, outside the timed region, unless --launch
# or --ordered fixes it.


def render_scene(name: str, width: int, height: int):
    """(Scene, mesh, tt_camera_meta) of a path-tracing workload."""
    import math
    from trenchanttracer_gb300 import Scene, make_camera_meta, scenes
    if name == "cornell":
        mesh = scenes.cornell(5)
        sc = Scene.from_mesh(mesh)
        cam = make_camera_meta(width, height, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 45.0))
    elif name == "multimaterial":
        mesh = scenes.multi_material(400, 5)
        sc = Scene.from_mesh(mesh)
        sc.set_env(scenes.sky_env(2048, 1024, sun_radiance=5e4, sun_diameter_deg=0.5))
        fy = 2.0 * math.degrees(math.atan(math.tan(math.radians(30.0)) * height / width))
        cam = make_camera_meta(width, height, [0.0, 14.0, 34.0], [0.0, -12.0, -34.0], fov=(60.0, fy))
    elif name == "terrain":
        mesh = scenes.terrain(N_CELLS, SCALE)
        sc = Scene.from_mesh(mesh)
        sc.set_env(scenes.sky_env(2048, 1024, sun_radiance=5e4, sun_diameter_deg=0.5))
        c = scenes.terrain_camera(SCALE)
        eye, tgt = np.array(c["eye"]), np.array(c["target"])
        fx = 2.0 * math.degrees(math.atan(c["tan_half_fov"]))
        fy = 2.0 * math.degrees(math.atan(c["tan_half_fov"] * height / width))
        cam = make_camera_meta(width, height, list(eye), list(tgt - eye), fov=(fx, fy))
    else:
        raise ValueError(name)
    return sc, mesh, cam


def render_cpu_baseline(bvh, sc, cam, spp: int, depth: int, budget_s: float = 15.0, min_s: float = 10.0) -> dict:
    """The oracle's C restatement of the native path tracer (OpenMP, all host cores) on the same
    view, at the highest resolution (halving from the full one down to 1/16) whose render takes
    under a quarter of budget_s, repeated with further samples until min_s have passed: paths
    per second."""
    import ctypes as C
    from oracle import oracle
    from trenchanttracer_gb300 import _lib, make_camera_meta, render_params
    mats, geos = sc.materials_raw(), sc.geometries_raw()
    mats = (_lib.Material * len(mats))(*mats)
    geos = (_lib.Geometry * len(geos))(*geos)
    env = sc.env()
    arr = bvh.arrays()
    threads = oracle.max_threads()
    tx = float(np.float32(np.tan(np.radians(cam.fov[0]) / 2)))
    ty = float(np.float32(np.tan(np.radians(cam.fov[1]) / 2)))

    def render(scale: int, offset: int):
        w, h = max(8, cam.width // scale), max(8, cam.height // scale)
        small = make_camera_meta(w, h, list(cam.position), list(cam.view), list(cam.up), tuple(cam.fov))
        p = render_params(spp=spp, sample_offset=offset, max_depth=depth, rr_depth=4, seed=1)
        t0 = time.perf_counter()
        oracle.render_native(arr, mats, geos, env, small, p, tx, ty, threads=threads)
        return w, h, time.perf_counter() - t0

    scale = 16
    while True:
        w, h, dt = render(scale, 0)
        if dt > budget_s / 4 or scale == 1:
            break
        scale //= 2
    total, passes = dt, 1
    while total < min_s:
        total += render(scale, passes * spp)[2]
        passes += 1
    return {"paths_per_s": passes * w * h * spp / total, "seconds": total, "threads": threads,
            "sample": f"{w}x{h} x {spp} spp x {passes} passes"}


def run_render(args) -> None:
    """Native path tracer on one of RENDER_CONFIGS: a step = one render of the configured image
    and sample count."""
    import torch
    from trenchanttracer_gb300 import BVHCompact, DeviceBVH, Renderer, render_params
    cfg = RENDER_CONFIGS[args.workload]
    dev = torch.device("cuda", 0)
    sc, mesh, cam = render_scene(args.workload, cfg["width"], cfg["height"])
    t0 = time.perf_counter()
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    build_s = time.perf_counter() - t0
    r = Renderer(DeviceBVH(bvh), sc)
    params = lambda k: render_params(spp=cfg["spp"], sample_offset=k * cfg["spp"], max_depth=cfg["depth"], rr_depth=4,
                                     seed=1)
    tune_s, trials = 0.0, 0
    if args.launch:  # a given shape
        r.set_launch(*[int(x) for x in args.launch.split(",")])
    elif args.ordered >= 0:  # the fixed default shape, ordering as asked
        r.set_launch(128, 16, 1 << 22, args.ordered)
    else:  # the launch-shape autotuner on the view itself (a batch of one)
        from trenchanttracer_gb300 import Batch
        t0 = time.perf_counter()
        trials = len(Batch(r, [(cam, cfg["spp"], 0, 1)], render_params(max_depth=cfg["depth"], rr_depth=4)).autotune())
        tune_s = time.perf_counter() - t0
    npx = cfg["width"] * cfg["height"] * 3
    acc = torch.zeros(npx, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for k in range(args.warmup):
        r.render_native(cam, params(k), acc, stream=stream.cuda_stream)
    torch.cuda.synchronize(dev)
    r.check()
    r.stats(reset=True)
    r.launches(reset=True)
    ms = []
    with Clocks(0) as clk:
        for k in range(args.steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record(stream)
            r.render_native(cam, params(args.warmup + k), acc, stream=stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
    r.check()
    st = r.stats(reset=True)
    launches = r.launches(reset=True)
    mean_ms = float(np.mean(ms))
    paths = cfg["width"] * cfg["height"] * cfg["spp"]
    rays = (st["extension_rays"] + st["shadow_rays"]) / args.steps
    # end to end: the render call plus the read of the image into page-locked host memory
    host = torch.empty(npx, dtype=torch.float32).pin_memory()
    e2e = []
    for k in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r.render_native(cam, params(k), acc, stream=stream.cuda_stream)
        host.copy_(acc, non_blocking=True)
        torch.cuda.synchronize(dev)
        e2e.append((time.perf_counter() - t0) * 1e3)
    img = host.numpy()
    assert np.isfinite(img).all()
    cpu = render_cpu_baseline(bvh, sc, cam, cfg["spp"], cfg["depth"])
    line = {
        "metric": f"Msamples/s native path tracer ({args.workload})", "value": round(paths / mean_ms / 1e3, 2),
        "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mean_ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": cfg["desc"], "tris": int(mesh.num_tris), "bvh_build_s": round(build_s, 2),
                   "launch_shape": list(r.launch), "autotune_s": round(tune_s, 2), "autotune_trials": trials,
                   "l2": "L2 flushed (256 MB write) between steps, untimed"},
        "mrays_per_s": round(rays / mean_ms / 1e3, 1),
        "rays_per_step": {"extension": st["extension_rays"] // args.steps, "shadow": st["shadow_rays"] // args.steps},
        "e2e": {"value": round(paths / float(np.mean(e2e)) / 1e3, 2), "unit": "Msamples/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(npx * 4)},
        "cpu_baseline": {"value": round(cpu["paths_per_s"] / 1e6, 4), "unit": "Msamples/s", "cores": cpu["threads"],
                         "cpu": cpu_model(),
                         "kind": "port", "sample": cpu["sample"] + f", {cpu['seconds']:.1f} s (same view)"},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def run_batch(args) -> None:
    """64 uneven orbit views of the terrain: one graph-captured batch versus 64 sequential renders."""
    import torch
    from trenchanttracer_gb300 import Batch, BVHCompact, DeviceBVH, Renderer, render_params, scenes
    dev = torch.device("cuda", 0)
    sc, mesh, _ = render_scene("terrain", 64, 64)
    r = Renderer(DeviceBVH(BVHCompact.build(sc, 1e-5, 1, 8)), sc)
    views = scenes.orbit_views(64)[:args.views]
    P = dict(max_depth=8, rr_depth=4)
    b = Batch(r, views, render_params(**P))
    t0 = time.perf_counter()
    if args.launch:
        r.set_launch(*[int(x) for x in args.launch.split(",")])
        trials = []
    else:
        trials = b.autotune()
    tune_s = time.perf_counter() - t0
    acc = torch.zeros(b.accum_elems, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        b.render(acc, stream=stream.cuda_stream)
    torch.cuda.synchronize(dev)
    r.check()
    r.stats(reset=True)
    ms = []
    with Clocks(0) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record(stream)
            b.render(acc, stream=stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
    r.check()
    st = r.stats(reset=True)
    accs = [torch.zeros(c.width * c.height * 3, dtype=torch.float32, device=dev) for c, *_ in views]
    seq = []
    for k in range(max(1, args.steps // 2)):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
        e0.record(stream)
        for (cam, spp, off, seed), a in zip(views, accs):
            r.render_native(cam, render_params(spp=spp, sample_offset=off, seed=seed, **P), a,
                            stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        seq.append(e0.elapsed_time(e1))
    host = torch.empty(b.accum_elems, dtype=torch.float32).pin_memory()
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b.render(acc, stream=stream.cuda_stream)
        host.copy_(acc, non_blocking=True)
        torch.cuda.synchronize(dev)
        e2e.append((time.perf_counter() - t0) * 1e3)
    mean_ms = float(np.mean(ms))
    rays = (st["extension_rays"] + st["shadow_rays"]) / args.steps
    line = {
        "metric": f"Msamples/s batched uneven renders ({len(views)} views, one graph launch)",
        "value": round(b.total_paths / mean_ms / 1e3, 2), "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(mean_ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded terrain and orbit poses)",
        "config": {"workload": f"{len(views)} orbit views of the terrain (2,097,152 tris, sky + sun), sizes from "
                               "{256,512,768,1024}^2, spp from {4,16,64}, depth 8, RR from 4",
                   "paths_per_step": b.total_paths, "graph_kernels": b.graph_kernels,
                   "launch_shape": list(r.launch), "autotune_s": round(tune_s, 2), "autotune_trials": len(trials),
                   "l2": "L2 flushed (256 MB write) between steps, untimed"},
        "sequential": {"value": round(b.total_paths / float(np.mean(seq)) / 1e3, 2), "unit": "Msamples/s",
                       "ms_per_step": round(float(np.mean(seq)), 3), "how": f"{len(views)} tt_render_native calls"},
        "mrays_per_s": round(rays / mean_ms / 1e3, 1),
        "e2e": {"value": round(b.total_paths / float(np.mean(e2e)) / 1e3, 2), "unit": "Msamples/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(b.accum_elems * 4)},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * b.graph_kernels,
    }
    print(json.dumps(line), flush=True)


def run_cache(args) -> None:
    """Time to relMSE 0.01 against an FP64 reference of args.ref_spp samples (rendered as two
    independent halves, whose disagreement measures the reference's own error), plain native
    tracer versus the tracer with the learned radiance cache, both at 1 spp per frame, time from
    CUDA events around each frame (training included), error evaluated between frames."""
    import torch
    from trenchanttracer_gb300 import BVHCompact, Cache, DeviceBVH, Renderer, render_params
    dev = torch.device("cuda", 0)
    W, H = args.width, args.height
    sc, mesh, cam = render_scene(args.cache_scene, W, H)
    r = Renderer(DeviceBVH(BVHCompact.build(sc, 1e-5, 1, 8)), sc)
    npx = W * H * 3
    D = dict(max_depth=16, rr_depth=4)
    half = args.ref_spp // 2
    t0 = time.perf_counter()
    halves = []
    for hlf in range(2):
        a = torch.zeros(npx, dtype=torch.float64, device=dev)
        for k in range(0, half, 256):
            n = min(256, half - k)
            r.render_native(cam, render_params(spp=n, sample_offset=hlf * half + k, seed=777, flags=1, **D), a)
        halves.append(a.view(-1, 3) / half)
    torch.cuda.synchronize(dev)
    r.check()
    ref_s = time.perf_counter() - t0
    ref = (halves[0] + halves[1]) / 2
    den = ref * ref + 1e-2

    def relmse(x):
        return float((((x - ref) ** 2) / den).sum(1).mean().item())

    a_, b_ = halves
    floor = float((((a_ - b_) ** 2) / (0.5 * (a_ * a_ + b_ * b_) + 1e-2)).sum(1).mean().item()) / 4.0
    evals = sorted({1, 2, 4, 8, 16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096})

    def run(step_fn):
        acc = torch.zeros(npx, dtype=torch.float32, device=dev)
        total, curve, hit = 0.0, [], None
        for f in range(args.max_frames):
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record()
            step_fn(f, acc)
            e1.record()
            e1.synchronize()
            total += e0.elapsed_time(e1) / 1e3
            if f + 1 in evals or f + 1 == args.max_frames:
                v = relmse(acc.view(-1, 3).double() / (f + 1))
                curve.append([f + 1, round(total, 4), round(v, 5)])
                if hit is None and v <= 0.01:
                    hit = [f + 1, round(total, 4)]
            if total > args.max_seconds:
                v = relmse(acc.view(-1, 3).double() / (f + 1))
                curve.append([f + 1, round(total, 4), round(v, 5)])
                break
        r.check()
        return hit, curve

    with Clocks(0) as clk:
        plain = run(lambda f, acc: r.render_native(cam, render_params(spp=1, sample_offset=f, seed=1, **D), acc))
        lo, hi = mesh.vertices.min(0) - 0.5, mesh.vertices.max(0) + 0.5
        cache = Cache(lo, hi)
        cached = run(lambda f, acc: r.render_cached(cache, cam, render_params(spp=1, sample_offset=f, seed=1, **D),
                                                    acc, train=True))

    time_to = _time_to

    t_plain, t_cached = time_to(plain[1], 0.01), time_to(cached[1], 0.01)
    final_plain = plain[1][-1]
    t_equal = time_to(cached[1], final_plain[2])
    line = {
        "metric": "time to relMSE 0.01, cached vs plain tracer", "value": None if t_cached is None else round(t_cached, 3),
        "unit": "s", "n_gpus": 1, "steps": len(cached[1]), "warmup": 0, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (MLP bf16, fp32 accumulation)",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": f"{args.cache_scene} {W}x{H}, depth 16, RR from 4, 1 spp per frame; cache MLP "
                               "160-64x5-3, 65,536 training paths per frame, 4 Adam steps of 16,384, lr 1e-2",
                   "relmse": "mean over pixels of sum_c (x - r)^2 / (r^2 + 0.01)",
                   "reference": f"{args.ref_spp} spp FP64 accumulation ({ref_s:.1f} s)"},
        "plain": {"time_to_0.01_s": None if t_plain is None else round(t_plain, 3), "curve": plain[1]},
        "cached": {"time_to_0.01_s": None if t_cached is None else round(t_cached, 3), "curve": cached[1],
                   "adam_steps": cache.steps},
        "time_ratio_cached_over_plain": None if (t_plain is None or t_cached is None) else round(t_cached / t_plain, 3),
        "reference_error": {"relmse_vs_truth_estimate": round(floor, 5),
                            "how": "relMSE between the two independent halves / 4"},
        "equal_error": {"plain_error": final_plain[2], "plain_s": final_plain[1],
                        "cached_s_to_same_error": None if t_equal is None else round(float(t_equal), 3),
                        "ratio": None if t_equal is None else round(float(t_equal) / final_plain[1], 3)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def _time_to(curve, level):
    """Time after which an error curve [(frames, seconds, error), ...] stays at or below `level`:
    the last crossing from above, interpolated linearly in log error (None if it ends above)."""
    above = [i for i, c in enumerate(curve) if c[2] > level]
    if not above:
        return curve[0][1]
    i = above[-1]
    if i == len(curve) - 1:
        return None
    (_, t0_, e0), (_, t1, e1) = curve[i], curve[i + 1]
    return t0_ + (t1 - t0_) * (np.log(e0) - np.log(level)) / (np.log(e0) - np.log(e1))


CACHE_LEVELS = [3.0, 1.0, 0.3, 0.1, 0.03, 0.01]


def cache_target(width: int = 960, height: int = 540, ref_spp: int = 16384, seconds: float = 4.0,
                 seeds=(1, 2, 3)) -> dict:
    """The metric's second half on the multi-material scene at a reduced size: relMSE against an
    FP64 reference of ref_spp samples (two independent halves, whose disagreement estimates the
    reference's own error), plain native tracer versus the learned radiance cache, 1 spp per
    frame, each run for `seconds` of GPU time (CUDA events around every frame, training included),
    for each seed (render streams and cache initialisation). The cache's training paths are
    scaled to the same share of a frame's paths as 65,536 are at 1920 x 1080."""
    import torch
    from trenchanttracer_gb300 import BVHCompact, Cache, DeviceBVH, Renderer, render_params
    dev = torch.device("cuda", 0)
    W, H = width, height
    sc, mesh, cam = render_scene("multimaterial", W, H)
    r = Renderer(DeviceBVH(BVHCompact.build(sc, 1e-5, 1, 8)), sc)
    npx = W * H * 3
    D = dict(max_depth=16, rr_depth=4)
    t0 = time.perf_counter()
    halves = []
    for hlf in range(2):
        a = torch.zeros(npx, dtype=torch.float64, device=dev)
        for k in range(0, ref_spp // 2, 512):
            n = min(512, ref_spp // 2 - k)
            r.render_native(cam, render_params(spp=n, sample_offset=hlf * (ref_spp // 2) + k, seed=777, flags=1, **D), a)
        halves.append(a.view(-1, 3) / (ref_spp // 2))
    torch.cuda.synchronize(dev)
    ref_s = time.perf_counter() - t0
    ref = (halves[0] + halves[1]) / 2
    den = ref * ref + 1e-2
    a_, b_ = halves
    floor = float((((a_ - b_) ** 2) / (0.5 * (a_ * a_ + b_ * b_) + 1e-2)).sum(1).mean().item()) / 4.0
    evals = {2 ** k for k in range(0, 16)}

    def run(step_fn):
        acc = torch.zeros(npx, dtype=torch.float32, device=dev)
        total, curve, f = 0.0, [], 0
        while total < seconds:
            e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
            e0.record()
            step_fn(f, acc)
            e1.record()
            e1.synchronize()
            total += e0.elapsed_time(e1) / 1e3
            f += 1
            if f in evals or total >= seconds:
                err = float((((acc.view(-1, 3).double() / f - ref) ** 2) / den).sum(1).mean().item())
                curve.append([f, round(total, 4), round(err, 5)])
        r.check()
        return curve

    lo, hi = mesh.vertices.min(0) - 0.5, mesh.vertices.max(0) + 0.5
    train_paths = max(1024, int(round(65536 * (W * H) / (1920 * 1080))))
    runs = []
    for seed in seeds:
        plain = run(lambda f, acc: r.render_native(cam, render_params(spp=1, sample_offset=f, seed=seed, **D), acc))
        cache = Cache(lo, hi, seed=seed, train_paths=train_paths)
        cached = run(lambda f, acc: r.render_cached(cache, cam, render_params(spp=1, sample_offset=f, seed=seed, **D),
                                                    acc, train=True))
        level = max(plain[-1][2], cached[-1][2])  # the lowest error both reach and stay at
        tp, tc = _time_to(plain, level), _time_to(cached, level)
        runs.append({"seed": seed, "common_level": round(level, 4),
                     "plain_s": None if tp is None else round(float(tp), 3),
                     "cached_s": None if tc is None else round(float(tc), 3),
                     "ratio_cached_over_plain": None if (tp is None or tc is None or tp <= 0) else round(float(tc / tp), 3),
                     "time_to_level_s": {str(lv): [None if _time_to(plain, lv) is None else round(float(_time_to(plain, lv)), 3),
                                                   None if _time_to(cached, lv) is None else round(float(_time_to(cached, lv)), 3)]
                                         for lv in CACHE_LEVELS},
                     "plain_curve": plain, "cached_curve": cached})
    ratios = [x["ratio_cached_over_plain"] for x in runs if x["ratio_cached_over_plain"] is not None]
    return {"workload": f"multi-material scene (8,192,002 tris, 2048 x 1024 sky, 5e4 sun) at {W} x {H} (the target's "
                        "1920 x 1080 reduced to fit a bench run), depth 16, roulette from 4, 1 spp per frame; cache MLP "
                        f"160-64x5-3, {train_paths:,} training paths per frame (3.2 % of the paths, as 65,536 are at "
                        "1920 x 1080), 4 Adam steps of 16,384, lr 1e-2",
            "relmse": "mean over pixels of sum_c (x - r)^2 / (r^2 + 0.01)",
            "reference": {"spp": ref_spp, "seconds": round(ref_s, 1), "own_error": round(floor, 5),
                          "how": "FP64 accumulation in two independent halves; own error = their relMSE / 4"},
            "time_to_0.01": "not reached by either tracer: the sun (5e4, 0.5 degrees) seen through dielectric "
                            "spheres makes caustic fireflies that neither estimator averages out in seconds "
                            "(time_to_level_s lists 3 .. 0.01 as [plain, cached])",
            "seconds_per_run": seconds, "runs": runs,
            "ratio_at_common_level": {"median": None if not ratios else float(np.median(ratios)),
                                      "min": None if not ratios else min(ratios),
                                      "max": None if not ratios else max(ratios), "seeds": len(ratios)}}


MLP_MACS = 160 * 64 + 4 * 64 * 64 + 64 * 8  # multiply-adds per row of one forward pass (padded output)


def run_mlp(args) -> None:
    """The radiance cache's tensor-core kernels alone: inference on 2^21 records and one frame's
    training (steps x batch rows; forward, backward and weight gradients = 3 forward's worth of
    multiply-adds) on random records, in TFLOP/s against the measured dense BF16 peak."""
    import torch
    from trenchanttracer_gb300 import Cache
    dev = torch.device("cuda", 0)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    g = torch.Generator(device=dev).manual_seed(5)
    n = 1 << 21
    rec = torch.rand((n, 16), generator=g, device=dev) * 2 - 1
    rec[:, 9:13] = rec[:, 9:13].abs()
    tgt = torch.rand((n, 3), generator=g, device=dev) + 0.1
    cache = Cache([-1.0] * 3, [1.0] * 3, mma_kind=args.mma_kind)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        cache.infer(rec)
        cache.train(rec[:65536], tgt[:65536], steps=4)
    torch.cuda.synchronize(dev)
    inf_ms, tr_ms = [], []
    with Clocks(0) as clk:
        for _ in range(args.steps):
            e0, e1, e2 = (torch.cuda.Event(True) for _ in range(3))
            e0.record(stream)
            out = cache.infer(rec)
            e1.record(stream)
            cache.train(rec[:65536], tgt[:65536], steps=4)
            e2.record(stream)
            torch.cuda.synchronize(dev)
            inf_ms.append(e0.elapsed_time(e1))
            tr_ms.append(e1.elapsed_time(e2))
    assert torch.isfinite(out).all()
    # the same training at 2^18 rows per Adam step, where the batch fills the GPU
    big = Cache([-1.0] * 3, [1.0] * 3, batch=1 << 18, mma_kind=args.mma_kind)
    for _ in range(2):
        big.train(rec[:1 << 20], tgt[:1 << 20], steps=4)
    torch.cuda.synchronize(dev)
    big_ms = []
    for _ in range(max(3, args.steps // 2)):
        e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
        e0.record(stream)
        big.train(rec[:1 << 20], tgt[:1 << 20], steps=4)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        big_ms.append(e0.elapsed_time(e1))
    big_tr = float(np.median(big_ms))
    big.check()
    cache.check()
    inf = float(np.median(inf_ms))
    tr = float(np.median(tr_ms))
    inf_tf = 2.0 * MLP_MACS * n / (inf * 1e-3) / 1e12
    tr_tf = 3 * 2.0 * MLP_MACS * 65536 / (tr * 1e-3) / 1e12
    line = {
        "metric": "radiance-cache MLP inference TFLOP/s (BF16 tensor cores, FP32 accumulation)",
        "value": round(inf_tf, 2), "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(inf, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 (fp32 accumulation)", "data": "synthetic (random feature records)",
        "config": {"workload": f"MLP 160-64x5-3 (padded to 8 outputs), inference on {n} records incl. encoding; "
                               "training = 4 Adam steps of 16,384 rows", "macs_per_row": MLP_MACS,
                   "kernels": "tcgen05 + TMEM" if args.mma_kind == 0 else "mma.sync m16n8k16"},
        "training": {"ms_per_frame": round(tr, 4), "tflops": round(tr_tf, 2),
                     "at_2^18_rows_per_step": {"ms_per_4_steps": round(big_tr, 4),
                                               "tflops": round(3 * 2.0 * MLP_MACS * (1 << 20) / (big_tr * 1e-3) / 1e12, 2)}},
        "roofline": {"bound": "tensor", "achieved": round(inf_tf, 2), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(inf_tf / peak, 4), "traffic": None,
                     "peak_source": "measured bf16_tflops (MEASURED_PEAKS.json)" if peaks else "fallback"},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * (1 + 4 * 4),  # inference; per Adam step forward, backward, wgrad, Adam
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["terrain", "cornell", "multimaterial", "batch", "cache", "mlp"], default="terrain")
    ap.add_argument("--cache-scene", choices=["multimaterial", "terrain"], default="multimaterial")
    ap.add_argument("--views", type=int, default=64, help="batch: the first N of the 64 orbit views (profiling)")
    ap.add_argument("--mma-kind", type=int, choices=[0, 1], default=0,
                    help="mlp: the cache's tensor-core kernels, 0 tcgen05 + TMEM, 1 mma.sync (comparison)")
    ap.add_argument("--launch", default="",
                    help="batch / cornell / multimaterial: block,stack_shared,wave_paths,ordered,streamed instead "
                         "of autotuning (profiling)")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--ordered", type=int, choices=[-1, 0, 1], default=-1,
                    help="cornell / multimaterial: the default launch shape with ordered queues (1) or not (0) "
                         "instead of autotuning (-1)")
    ap.add_argument("--trace-width", type=int, default=WIDTH,
                    help="terrain workload: camera width; each ray set has width^2 rays (profiling a "
                         "smaller case of the same kernels)")
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--max-frames", type=int, default=4096)
    ap.add_argument("--max-seconds", type=float, default=60.0)
    ap.add_argument("--cache-seconds", type=float, default=4.0,
                    help="terrain line: GPU seconds per tracer and seed of its radiance-cache measurement (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from trenchanttracer_gb300 import build
    build.build()
    if args.impl == "reference":
        if args.workload != "terrain":
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference arm is defined for the terrain "
                                  "ray-cast workload; the path-tracing workloads report the oracle port as "
                                  "cpu_baseline"}), flush=True)
            return
        run_reference(args)
    elif args.workload == "terrain":
        run_ours(args)
    elif args.workload in RENDER_CONFIGS:
        run_render(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "mlp":
        run_mlp(args)
    else:
        run_cache(args)


if __name__ == "__main__":
    main()
