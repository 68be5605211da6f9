"""Benchmark of the kd-tree build + trace path on one GB300 (or N replicas).

Workload (one "step" = one frame of the 1M-triangle clustered scene):
  * rebuild the kd tree over 1,000,000 device-resident triangles
    (64 Gaussian clusters, 2 ground-plane triangles, 2000 thin triangles);
  * trace 1920x1080 primary rays with the short-stack tracer (depth 8) and,
    fused in the same kernel, one shadow ray per hit toward (0.5, 3, 0.5).
Metric: rays traced (primary + shadow) per second of the whole step, build
included, in Mrays/s; the build time and the trace-only throughput are
reported beside it.

Timing: CUDA events on the launching stream around each step, L2 flushed
(a 512 MB write) between steps outside the events; max over ranks.  Under
torchrun each rank runs an independent replica (weak scaling).

--impl reference times the reference's algorithms on the host cores: the CPU
restatement in oracle/ (the reference itself does not compile here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "extensions-photonmapping_gb300"))

N_TRIS = 1_000_000
WIDTH, HEIGHT = 1920, 1080
LIGHT = (0.5, 3.0, 0.5)
SCENE_SEED = 2
BUILD = dict(lower=1, traversal_cost=1.0, intersection_cost=1.5, min_leaf=8)
BUILD_DESC = "reference upper (median + empty space to <32 refs) + SAH lower Ct=1 Ci=1.5 min_leaf=8"
STACK_DEPTH = 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tris", type=int, default=N_TRIS)
    ap.add_argument("--width", type=int, default=WIDTH)
    ap.add_argument("--height", type=int, default=HEIGHT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() and args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def workload(args):
    from kdgb import scenes
    tris = scenes.clustered(args.tris, seed=SCENE_SEED)
    o, d = scenes.camera_rays(args.width, args.height)
    return tris, o, d


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
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
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per trace launch from the committed ncu summary, scaled by
    the units it covers; None when no capture has been committed."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def cpu_baseline(tris, o, d, sample_stride=16, threads=0):
    """The oracle (reference algorithms restated in C, OpenMP) on the host
    cores: full build + traced sample of every `sample_stride`-th ray."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from kdgb import scenes
    O.lib()
    t0 = time.perf_counter()
    tree = O.build(tris, **BUILD)
    t_build = time.perf_counter() - t0
    idx = np.arange(0, o.shape[0], sample_stride)
    t0 = time.perf_counter()
    h, t, _, _ = O.trace(tree, tris, o[idx], d[idx], tracer=O.TRACER_SHORTSTACK, stack_depth=STACK_DEPTH,
                         threads=threads)
    pts = scenes.hit_points(o[idx], d[idx], t, h)[h >= 0]
    O.trace_shadow(tree, tris, pts, LIGHT, threads=threads)
    t_trace = time.perf_counter() - t0
    n_sample = len(idx) + int((h >= 0).sum())
    scale = o.shape[0] / len(idx)
    step_s = t_build + t_trace * scale
    rays = n_sample * scale
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return {"value": rays / step_s / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
            "sample": f"full CPU build ({t_build * 1e3:.0f} ms) + every {sample_stride}th primary ray and its "
                      f"shadow ray ({t_trace * 1e3:.0f} ms), extrapolated to the frame",
            "build_ms": t_build * 1e3}


def run_reference(args, world, rank):
    """--impl reference: the oracle on all host cores, full frames."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from kdgb import scenes
    O.lib()
    tris, o, d = workload(args)
    cores = os.cpu_count() or 1

    def step():
        tree = O.build(tris, **BUILD)
        h, t, _, _ = O.trace(tree, tris, o, d, tracer=O.TRACER_SHORTSTACK, stack_depth=STACK_DEPTH)
        pts = scenes.hit_points(o, d, t, h)[h >= 0]
        O.trace_shadow(tree, tris, pts, LIGHT)
        return o.shape[0] + pts.shape[0]

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    rays = 0
    for _ in range(args.steps):
        rays += step()
    dt = time.perf_counter() - t0
    val = rays / dt / 1e6
    line = {"impl": "reference", "metric": "kd traversal Mrays/s per frame (1M-tri build + primary + shadow)",
            "value": val, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "clustered-1M-tris 1920x1080 primary + shadow, short-stack depth 8",
                       "tris": args.tris, "rays": args.width * args.height, "build": BUILD_DESC},
            "cpu_baseline": {"value": val, "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": "full frames: CPU restatement of the reference build + short-stack + "
                                       "shadow rays, OpenMP over all host cores"},
            "e2e": {"value": val, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    import torch
    import kdgb
    from kdgb import _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = kdgb.lib()
    tris, o, d = workload(args)
    n = o.shape[0]
    tris_d = torch.from_numpy(tris).to(dev)
    o_d = torch.from_numpy(o).to(dev)
    d_d = torch.from_numpy(d).to(dev)
    bp = kdgb.build_params(**BUILD)
    tp = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=STACK_DEPTH, tile_width=args.width)
    tree = kdgb.KDTree.build(tris_d, bp)
    outs = (torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.float32, device=dev),
            torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.float32, device=dev),
            torch.empty(n, dtype=torch.int32, device=dev))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def step(ev=None):
        tree.rebuild(tris_d, bp)
        if ev:
            ev[0].record(stream)
        tree.trace_primary_shadow(o_d, d_d, LIGHT, tp, out=outs)
        if ev:
            ev[1].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    n_hits = int((outs[0] >= 0).sum().item())
    rays_per_step = n + n_hits
    st = tree.stats()

    sampler = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches0 = L.kdgb_launch_count()
    sampler.start()
    step_ms, trace_ms = [], []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("kdgb_timed_step")
        e0.record(stream)
        step((t0, t1))
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        trace_ms.append(t0.elapsed_time(t1))
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = L.kdgb_launch_count() - launches0
    total_ms = float(sum(step_ms))
    if pg:
        t = torch.tensor([total_ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = rays_per_step * world / (ms_per_step / 1e3) / 1e6

    # Roofline of the dominant kernel (fused short-stack primary + shadow).
    T = tris.shape[0]
    scene_bytes = 36 * T + 16 * st.n_nodes + 4 * st.n_refs
    alg_bytes = 40 * n + 28 * n_hits + scene_bytes
    tr_ms = statistics.mean(trace_ms)
    peak, peak_kind = measured_peak_gbs()
    achieved = alg_bytes / (tr_ms / 1e3) / 1e9
    traffic = committed_traffic()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic.get("trace_dram_bytes_per_launch") if traffic else None,
            "kernel": "k_trace<SHORTSTACK,leaf-skip,shadow>", "algorithmic_bytes_per_launch": alg_bytes,
            "peak_source": f"{peak_kind} hbm_gbs"}

    # End to end through the public API with host buffers.
    e2e = None
    if not args.no_e2e:
        h_tris = torch.from_numpy(tris).pin_memory()
        h_o = torch.from_numpy(o).pin_memory()
        h_d = torch.from_numpy(d).pin_memory()
        h_out = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in outs]

        def e2e_step():
            tris_d.copy_(h_tris, non_blocking=True)
            o_d.copy_(h_o, non_blocking=True)
            d_d.copy_(h_d, non_blocking=True)
            step()
            for hb, db in zip(h_out, outs):
                hb.copy_(db, non_blocking=True)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        e1.synchronize()
        e2e_ms = e0.elapsed_time(e1) / args.steps
        if pg:
            t = torch.tensor([e2e_ms], device=dev)
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            e2e_ms = float(t.item())
        h2d = tris.nbytes + o.nbytes + d.nbytes
        d2h = sum(x.numel() * x.element_size() for x in outs)
        e2e = {"value": rays_per_step * world / (e2e_ms / 1e3) / 1e6, "unit": "Mrays/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(tris, o, d)

    if rank == 0:
        line = {"metric": "kd traversal Mrays/s per frame (1M-tri build + primary + shadow)", "value": value,
                "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded clustered scene, pinhole camera)",
                "config": {"workload": "clustered-1M-tris 1920x1080 primary + shadow, short-stack depth 8",
                           "tris": T, "rays_primary": n, "rays_shadow": n_hits, "build": BUILD_DESC,
                           "l2": "512 MB buffer written between timed steps",
                           "parallelism": f"replicas x{world}"},
                "build_ms": statistics.mean(s - t for s, t in zip(step_ms, trace_ms)),
                "trace_ms": tr_ms, "trace_mrays_s": rays_per_step / (tr_ms / 1e3) / 1e6,
                "tree": {"nodes": st.n_nodes, "refs": st.n_refs, "upper_levels": st.upper_levels,
                         "lower_levels": st.lower_levels},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clocks}
        print(json.dumps(line), flush=True)
    tree.close()
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
