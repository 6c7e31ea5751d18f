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
  roofline  the traversal kernel: algorithmic bytes per ray (ray 32 + hit 8 + 64 per inner
            node + 16 per leaf + 48 per triangle tested + 56 per accepted hit update, counts
            from the oracle's instrumented restatement on a sample of the same rays) over the
            measured kernel time, against the measured HBM copy bandwidth
  cpu_baseline  the reference's traversal restated in C (oracle/, plain float arithmetic like
            the reference's host build) under OpenMP on all host cores, on a sample of the rays

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
METRIC = "Mrays/s closest-hit; time to relMSE 0.01, cached vs plain tracer, 1 GB300"
UNIT = "Mrays/s"
L2_FLUSH_BYTES = 256 << 20


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def workload(trace_ext=None):
    """Scene, BVH and the two ray sets. trace_ext(rays) -> (t, normal) gives the first hits
    from which the incoherent rays are spawned (the product's own kernel on the GPU arm)."""
    from trenchanttracer_gb300 import BVHCompact, Scene, scenes
    mesh = scenes.terrain(N_CELLS, SCALE)
    bvh = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8)
    cam = scenes.terrain_camera(SCALE)
    primary = scenes.pinhole_rays(WIDTH, WIDTH, cam["eye"], cam["target"], cam["tan_half_fov"])
    t, normal = trace_ext(bvh, primary)
    secondary, _ = scenes.secondary_rays(primary, t, normal, primary.shape[0], 11, 1e-4 * SCALE)
    return mesh, bvh, primary, secondary


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


def bytes_per_ray(counters: np.ndarray) -> float:
    """Algorithmic bytes per ray from the oracle's (node, leaf, tri, hit-update) counts."""
    c = counters.astype(np.float64).mean(axis=0)
    return 32.0 + 8.0 + 64.0 * c[0] + 16.0 * c[1] + 48.0 * c[2] + 56.0 * c[3]


def cpu_baseline(bvh_arrays: dict, rays: np.ndarray, sample: int, want_counters: bool) -> dict:
    """The oracle (plain arithmetic, OpenMP on all host cores) on every k-th ray."""
    from oracle import oracle
    stride = max(1, rays.shape[0] // sample)
    sub = np.ascontiguousarray(rays[::stride])
    threads = oracle.max_threads()
    oracle.intersect(bvh_arrays, sub[:4096], True, arith=oracle.PLAIN, threads=threads)  # warm
    t0 = time.perf_counter()
    o = oracle.intersect(bvh_arrays, sub, True, arith=oracle.PLAIN, threads=threads, counters=want_counters)
    dt = time.perf_counter() - t0
    return {"mrays": sub.shape[0] / dt / 1e6, "rays": int(sub.shape[0]), "seconds": dt, "threads": threads,
            "counters": o.get("counters")}


def run_reference(args) -> None:
    """--impl reference: the reference's traversal on the host cores (the oracle port with the
    reference's plain float arithmetic, OpenMP), on this arm's workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from trenchanttracer_gb300 import scenes
    from oracle import oracle

    def host_ext(bvh, rays):
        o = oracle.intersect(bvh.arrays(), rays, True, arith=oracle.PLAIN, normals=True)
        return o["t"], o["normal"]

    _, bvh, primary, secondary = workload(host_ext)
    arr = bvh.arrays()
    rays = np.concatenate([primary, secondary])
    sample = 1 << 20
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(arr, rays, sample, False)
        if i >= args.warmup:
            vals.append(r["mrays"])
            secs.append(r["seconds"])
    v = float(np.median(vals))
    cores = oracle.max_threads()
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.median(secs)) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm terrain, seed 7)",
            "config": {"workload": "terrain ray-cast: 2,097,152 tris, 4M coherent + 4M incoherent closest-hit rays",
                       "sample_rays_per_step": r["rays"]},
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"every {rays.shape[0] // r['rays']}th ray of the 8,388,608 (both sets)"},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
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

    mesh, bvh, primary, secondary = workload(gpu_ext)
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
    ms = float(np.sum(step_ms)) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n_rays / ms / 1e3  # whole-job Mrays/s

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
    e2e_val = world * n_rays / (float(np.mean(e2e_ms))) / 1e3
    # device and host paths agree bit for bit
    ids_d, t_d = hits_to_numpy(hits[1].cpu().numpy())
    ids_h, t_h = hits_to_numpy(h_hits[1].numpy())
    assert np.array_equal(ids_d, ids_h) and np.array_equal(t_d.view(np.uint32), t_h.view(np.uint32))

    if rank != 0:
        return
    peaks = load_peaks()
    cpu = cpu_baseline(bvh.arrays(), np.concatenate([primary, secondary]), 1 << 20, True)
    bpr = bytes_per_ray(cpu["counters"])
    kernel_ms = (np.mean(launch_ms[0]) + np.mean(launch_ms[1])) / 2.0
    achieved = bpr * (n_rays / 2) / (kernel_ms * 1e-3) / 1e9
    hit_frac = float((ids_d >= 0).mean())
    ids_p, _ = hits_to_numpy(hits[0].cpu().numpy())
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm terrain, seed 7; rays seeded)",
        "config": {"workload": "terrain ray-cast: 1024x1024-cell heightfield, 2,097,152 tris, world scale 8; "
                               "4,194,304 coherent primary + 4,194,304 incoherent rays, closest hit",
                   "bvh": "compact SBVH, split alpha 1e-5, leaf <= 8", "rays_per_step": n_rays,
                   "l2": "inputs larger than L2; L2 also flushed (256 MB write) between steps, untimed",
                   "parallelism": f"replicas x{world}"},
        "per_set": {"primary_mrays": round(sets[0].shape[0] / np.mean(launch_ms[0]) / 1e3, 1),
                    "incoherent_mrays": round(sets[1].shape[0] / np.mean(launch_ms[1]) / 1e3, 1),
                    "primary_hit_fraction": round(float((ids_p >= 0).mean()), 4),
                    "incoherent_hit_fraction": round(hit_frac, 4)},
        "e2e": {"value": round(e2e_val, 2), "unit": UNIT, "h2d_bytes_per_step": int(n_rays * 32),
                "d2h_bytes_per_step": int(n_rays * 8)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                     "peak_source": f"{peaks['source']} hbm_gbs (MEASURED_PEAKS.json)" if peaks["source"] == "measured"
                     else "fallback 6.8 TB/s", "bytes_per_ray": round(bpr, 1),
                     "kernel": "trace_kernel<closest> (avg launch)", "avg_launch_ms": round(float(kernel_ms), 4)},
        "cpu_baseline": {"value": round(cpu["mrays"], 3), "unit": UNIT, "cores": cpu["threads"], "kind": "port",
                         "sample": f"{cpu['rays']} rays (every {n_rays // cpu['rays']}th of both sets), "
                                   f"{cpu['seconds']:.1f} s"},
        "clocks": clocks,
        "gpu_launches": 2 * args.steps,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from trenchanttracer_gb300 import build
    build.build()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
