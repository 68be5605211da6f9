"""Benchmark of the kd-tree build + trace path on one GB300 (or N replicas).

Default workload (one "step" = one frame of the 1M-triangle clustered scene):
  * rebuild the kd tree over 1,000,000 device-resident triangles
    (64 Gaussian clusters, 2 ground-plane triangles, 2000 thin triangles) by
    launching the tree's rebuild graph (kdgb_graph_launch: the whole level
    loop on the device, no host round trip);
  * trace 1920x1080 primary rays with the short-stack tracer (depth 8) and,
    fused in the same kernel, one shadow ray per hit toward (0.5, 3, 0.5).
Metric: rays traced (primary + shadow) per second of the whole step, build
included, in Mrays/s; the build time and the trace-only throughput are
reported beside it.  The same line carries the batched half of the metric
(512 meshes, one graph against a per-mesh loop of graph launches and one of
host-driven rebuilds), a parity record (the GPU tree and a ray sample against
the oracle, which the CPU baseline builds anyway) and the error of t, u, v
against an FP64 brute-force oracle on a ray sample.

Timing: CUDA events on the launching stream around each step, L2 flushed
(a 512 MB write) between steps outside the events; max over ranks.  Under
torchrun each rank runs an independent replica (weak scaling).

End to end (`e2e`): the same frames through the library's public calls with
host buffers: every frame uploads its triangles and rays from pinned host
memory, rebuilds its tree by one graph launch, traces and reads all its
outputs back.  Four frames are in flight: four tree handles take the frames
in turn, each rebuilt on its own stream, so the rebuilds of consecutive
frames overlap each other and the traces of earlier frames.  The
one-frame-in-flight figure is reported beside it.

--impl reference times the same frame (same build configuration, tracer and
rays) with the CPU restatement in oracle/ on all host cores; the reference
itself does not compile here.

--workload selects the other measured configurations (one JSON line each):
  small    4096-triangle height field, 256x256 rays: kd-restart and brute force
  photons  262,144-triangle clustered scene, 16M photons x 3 diffuse bounces,
           kd-restart vs short-stack, Msegments/s
  batched  512 clustered meshes (log-uniform 1k..200k triangles, ~22M total),
           64k rays per mesh: one graph (forest build + trace) vs per-mesh
           loops, parameters from the autotuner
  adjoint  100k-triangle height field (316x158), 512x512 rays: backward pass
  next     the rows after the hot path: a moving 1M-triangle surface updated,
           collected (vertices, normals, colours), rebuilt and shaded with
           reflections at 1920x1080; Woop's test against Moeller-Trumbore and
           the balanced lower creator and DIVIDE split method on the frame scene
"""
from __future__ import annotations

import argparse
import atexit
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

from kdgb import configs  # noqa: E402

METRIC = "kd traversal Mrays/s per frame (1M-tri build + primary + shadow)"
HEADROOM = 1.1
FLUSH_BYTES = 512 << 20
BUILDS = {"tuned": (configs.TUNED, configs.TUNED_DESC), "reference": (configs.SAH, configs.SAH_DESC)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="frame", choices=["frame", "small", "photons", "batched", "adjoint", "next"])
    ap.add_argument("--tris", type=int, default=configs.FRAME_TRIS)
    ap.add_argument("--width", type=int, default=configs.WIDTH)
    ap.add_argument("--height", type=int, default=configs.HEIGHT)
    ap.add_argument("--host-build", action="store_true", help="rebuild with the host-driven level loop")
    ap.add_argument("--build", default="tuned", choices=["tuned", "reference"],
                    help="tuned: the frame's configuration; reference: the reference's creators")
    ap.add_argument("--profile", action="store_true",
                    help="one build and two traces, nothing timed (for ncu captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--partition", type=int, default=0,
                    help="e2e with frames in flight: rebuilds on an SM partition of at least this many SMs, traces on "
                         "the rest (0: the whole device for both)")
    ap.add_argument("--no-batched", action="store_true", help="leave the batched record out of the frame line")
    ap.add_argument("--no-others", action="store_true",
                    help="leave the small, photon and adjoint records out of the frame line")
    ap.add_argument("--meshes", type=int, default=configs.BATCH_MESHES,
                    help="batched workload: number of meshes (the first of the 512-mesh mix)")
    return ap.parse_args()


def frame_config(args, build_desc, n_hits):
    """The frame's `config`, identical in both arms."""
    return {"workload": "clustered-1M-tris 1920x1080 primary + shadow, short-stack depth 8",
            "tris": args.tris, "rays_primary": args.width * args.height, "rays_shadow": int(n_hits),
            "light": list(configs.LIGHT), "build": build_desc,
            "l2": "GPU arm: 512 MB buffer written between timed steps; CPU arm: no GPU",
            "parallelism": f"replicas x{args.gpus}"}


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
    return configs.frame_scene(args.tris, args.width, args.height)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region.

    nvidia-smi needs a few hundred ms before its first sample, longer than a
    short timed region, so start() (called before the warm-up steps) returns
    only once the first sample has arrived; mark() opens the window at the
    start of the timed region, and stop() waits for one more sample taken
    after the region has ended."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 100

    def __init__(self, index: int, cmd: str = "nvidia-smi"):
        self.index = index
        self.cmd = cmd
        self.proc = None
        self.lines = []
        self.first = 0
        self.cv = threading.Condition()

    def start(self, wait_s: float = 5.0):
        try:
            self.proc = subprocess.Popen([self.cmd, f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            atexit.register(self._end)  # no sampler outlives the run, whatever happens before stop()
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        self._wait_for(1, wait_s)
        self.mark()

    def mark(self):
        with self.cv:
            self.first = len(self.lines)

    def _end(self):
        if self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def _read(self):
        for line in self.proc.stdout:
            with self.cv:
                self.lines.append(line.strip())
                self.cv.notify_all()

    def _wait_for(self, n: int, wait_s: float):
        with self.cv:
            self.cv.wait_for(lambda: len(self.lines) >= n, timeout=wait_s)

    def stop(self, wait_s: float = 2.0):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._wait_for(len(self.lines) + 1, wait_s)
        self._end()
        self.t.join(timeout=5)
        with self.cv:
            window = self.lines[self.first:]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in window:
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
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": self.INTERVAL_MS}


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes (read + write) per launch of the trace kernel from the
    committed ncu summary; None when no capture has been committed."""
    path = os.path.join(ROOT, "profiles", "k_trace_clustered1M_frame.md")
    if not os.path.exists(path):
        return None
    import re
    with open(path) as f:
        m = re.search(r"^traffic_bytes_per_launch = (\d+)$", f.read(), re.M)
    return {"trace_dram_bytes_per_launch": int(m.group(1)), "source": "profiles/k_trace_clustered1M_frame.md"} \
        if m else None


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.lib()
    return O




def oracle_kwargs(bp):
    """A library build-parameter struct as keyword arguments of the oracle."""
    return {name: getattr(bp, name) for name, _ in bp._fields_}


def cpu_frame(O, tris, o, d, build_kw, sample_stride=16, threads=0):
    """The oracle (the build and tracers restated in C, OpenMP) on the host
    cores: a full build with the GPU arm's parameters and the primary and
    shadow rays of every `sample_stride`-th pixel.  Returns the baseline
    record and, for the parity record, the tree and the sample's results."""
    from kdgb import scenes
    t0 = time.perf_counter()
    tree = O.build(tris, **build_kw)
    t_build = time.perf_counter() - t0
    idx = np.arange(0, o.shape[0], sample_stride)
    t0 = time.perf_counter()
    h, t, u, v = O.trace(tree, tris, o[idx], d[idx], tracer=O.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH,
                         threads=threads)
    hitm = h >= 0
    pts = scenes.hit_points(o[idx], d[idx], t, h)[hitm]
    occ_hits = O.trace_shadow(tree, tris, pts, configs.LIGHT, threads=threads)
    t_trace = time.perf_counter() - t0
    occ = np.zeros(idx.shape[0], np.int32)
    occ[hitm] = occ_hits
    n_sample = len(idx) + int(hitm.sum())
    scale = o.shape[0] / len(idx)
    step_s = t_build + t_trace * scale
    rays = n_sample * scale
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    rec = {"value": rays / step_s / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
           "sample": f"full CPU build, same parameters as the GPU arm ({t_build * 1e3:.0f} ms) + every "
                     f"{sample_stride}th primary ray and its shadow ray ({t_trace * 1e3:.0f} ms), extrapolated "
                     f"to the frame",
           "build_ms": t_build * 1e3,
           "compiler": "gcc -O3 -std=c11 -fopenmp -ffp-contract=off -fno-fast-math (oracle/Makefile, no -march)"}
    return rec, tree, idx, (h, t, u, v, occ)


TREE_FIELDS = ("info", "split", "children", "prim_index", "bitmap", "parent", "area", "aabb_min", "aabb_max",
               "prim_indices", "leaf_ids")


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return bool(np.array_equal(a.view(np.uint32), b.view(np.uint32)))
    return bool(np.array_equal(a, b))


def parity_record(gpu_tree, cpu_tree, idx, gpu_out, cpu_out):
    """The GPU tree and the GPU results on the sampled rays against the
    oracle's, bit for bit."""
    h, t, u, v, occ = gpu_out
    hr, tr, ur, vr, occr = cpu_out
    hit = hr >= 0
    tuv = all(same_bits(x[idx][hit], y[hit]) for x, y in ((t, tr), (u, ur), (v, vr)))
    return {"against": "oracle, same build parameters and tracer (CPU)",
            "tree_arrays_equal": all(same_bits(getattr(gpu_tree, f), getattr(cpu_tree, f)) for f in TREE_FIELDS),
            "rays_checked": int(idx.shape[0]), "hit_ids_equal": bool(np.array_equal(h[idx], hr)),
            "tuv_bits_equal": bool(tuv), "shadow_equal": bool(np.array_equal(occ[idx], occr))}


def fp64_error(O, tris, o, d, h, t, u, v, stride):
    """t, u, v of the fp32 tracer against an FP64 brute-force oracle on every
    `stride`-th ray (rays on which both find the same triangle)."""
    idx = np.arange(0, o.shape[0], stride)
    hf, tf, uf, vf = O.trace_brute_f64(tris, o[idx], d[idx])
    hs = h[idx]
    either = (hs >= 0) | (hf >= 0)
    agree = (hs == hf) & (hf >= 0)
    rel_t = np.abs(t[idx][agree].astype(np.float64) - tf[agree]) / np.abs(tf[agree])
    du = np.abs(u[idx][agree].astype(np.float64) - uf[agree])
    dv = np.abs(v[idx][agree].astype(np.float64) - vf[agree])
    return {"oracle": "FP64 brute force", "rays": int(idx.shape[0]), "hits_compared": int(agree.sum()),
            "id_agreement": float(agree.sum() / max(1, either.sum())),
            "t_max_rel": float(rel_t.max()) if rel_t.size else None,
            "t_median_rel": float(np.median(rel_t)) if rel_t.size else None,
            "u_max_abs": float(du.max()) if du.size else None, "v_max_abs": float(dv.max()) if dv.size else None}


def run_reference(args, world, rank):
    """--impl reference: the same frame (build configuration, tracer, rays)
    with the oracle on all host cores, full frames."""
    if rank != 0:
        return
    O = oracle_module()
    from kdgb import scenes
    tris, o, d = workload(args)
    cores = os.cpu_count() or 1
    build_kw, build_desc = BUILDS[args.build]

    def step(kw):
        tree = O.build(tris, **kw)
        h, t, _, _ = O.trace(tree, tris, o, d, tracer=O.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH)
        pts = scenes.hit_points(o, d, t, h)[h >= 0]
        O.trace_shadow(tree, tris, pts, configs.LIGHT)
        return o.shape[0] + pts.shape[0]

    for _ in range(args.warmup):
        rays = step(build_kw)
    t0 = time.perf_counter()
    rays = 0
    for _ in range(args.steps):
        rays += step(build_kw)
    dt = time.perf_counter() - t0
    val = rays / dt / 1e6
    n_hits = rays // args.steps - o.shape[0]
    # The other build configuration, one timed frame, for context.
    alt = "reference" if args.build == "tuned" else "tuned"
    alt_kw, alt_desc = BUILDS[alt]
    t0 = time.perf_counter()
    alt_rays = step(alt_kw)
    alt_s = time.perf_counter() - t0
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded clustered scene, pinhole camera)",
            "config": frame_config(args, build_desc, n_hits),
            "cpu_baseline": {"value": val, "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": "full frames: the oracle's restatement of the same build + short-stack + "
                                       "shadow rays, OpenMP over all host cores",
                             "compiler": "gcc -O3 -std=c11 -fopenmp -ffp-contract=off -fno-fast-math "
                                         "(oracle/Makefile, no -march)"},
            "e2e": {"value": val, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "other_build": {"build": alt_desc, "ms_per_step": alt_s * 1e3, "value": alt_rays / alt_s / 1e6}}
    print(json.dumps(line), flush=True)


def time_steps(step, steps, stream, flush=None):
    """Per-step device milliseconds (CUDA events on `stream`), L2 flushed
    between steps outside the events."""
    import torch
    out = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


FRAMES_IN_FLIGHT = 4
# Streams of the batched record's concurrent per-mesh comparator.
CONCURRENT_STREAMS = 16
# Bytes a traversal step reads: a node record, a leaf's box pair, a
# triangle record (the traversal layout's sizes).
TRACE_BYTES = {"node": 8, "box": 32, "tri": 48}


def e2e_frames_in_flight(args, dev, tree, graph, bp, tp, tris_d, o_d, d_d, outs, h_tris, h_o, h_d, stream,
                         n_slots=FRAMES_IN_FLIGHT, partition_sms=0):
    """End to end with n_slots frames in flight: as many tree handles (each
    with its own rebuild graph and its own input and output buffers) take the
    frames in turn.  Frame k is uploaded and rebuilt on slot k's own
    rebuild stream (high priority, so the rebuild's short kernels are
    scheduled ahead of the trace's blocks) while earlier frames are traced on
    the trace stream and read back on the read-back stream; the rebuilds of
    consecutive frames overlap each other and the traces.  Every frame still
    uploads its triangles and rays from pinned host memory, rebuilds its tree,
    traces all its rays and reads back all its outputs.  Returns the
    milliseconds per frame and the host copies of the last frames' outputs."""
    import torch
    import kdgb
    high = torch.cuda.Stream.priority_range()[1]
    part = kdgb.SmPartition(partition_sms) if partition_sms > 0 else None
    slots = [] if part else [dict(tree=tree, graph=graph, tris=tris_d, o=o_d, d=d_d, outs=outs)]
    while len(slots) < n_slots:
        t_ = tris_d.clone()
        tr = kdgb.KDTree.build(t_, bp)
        # With an SM partition each slot's rebuild graph is captured on a
        # stream of the rebuild partition, so its kernels keep to those SMs.
        sb = part.stream(0, priority=high) if part else torch.cuda.Stream(device=dev, priority=high)
        torch.cuda.synchronize()
        slots.append(dict(tree=tr, graph=kdgb.Graph(tr, t_, params=bp, headroom=HEADROOM, stream=sb), tris=t_,
                          o=o_d.clone(), d=d_d.clone(), outs=tuple(torch.empty_like(x) for x in outs), own=True,
                          build_stream=sb))
    for sl in slots:
        sl["h_out"] = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in sl["outs"]]
        if "build_stream" not in sl:
            sl["build_stream"] = torch.cuda.Stream(device=dev, priority=high)
        for name in ("built", "traced", "read"):
            sl[name] = torch.cuda.Event()
            sl[name].record(stream)
    st = part.stream(1) if part else torch.cuda.Stream(device=dev)
    up, back = torch.cuda.Stream(device=dev, priority=high), torch.cuda.Stream(device=dev)
    last_in = torch.cuda.Event()

    def frame(k):
        sl = slots[k % n_slots]
        sb = sl["build_stream"]
        up.wait_event(sl["built"])   # the slot's previous rebuild has read its triangles
        with torch.cuda.stream(up):
            sl["tris"].copy_(h_tris, non_blocking=True)
        tin = torch.cuda.Event()
        tin.record(up)
        up.wait_event(sl["traced"])  # the slot's previous trace has read its rays
        with torch.cuda.stream(up):
            sl["o"].copy_(h_o, non_blocking=True)
            sl["d"].copy_(h_d, non_blocking=True)
        rin = torch.cuda.Event()
        rin.record(up)
        last_in.record(up)
        sb.wait_event(tin)
        sb.wait_event(sl["traced"])  # the slot's previous trace is done with its tree
        sl["graph"].launch(stream=sb)
        sl["built"].record(sb)
        st.wait_event(sl["built"])
        st.wait_event(rin)
        st.wait_event(sl["read"])    # the slot's previous outputs have been read back
        sl["tree"].trace_primary_shadow(sl["o"], sl["d"], configs.LIGHT, tp, stream=st, out=sl["outs"])
        sl["traced"].record(st)
        back.wait_event(sl["traced"])
        with torch.cuda.stream(back):
            for hb, db in zip(sl["h_out"], sl["outs"]):
                hb.copy_(db, non_blocking=True)
        sl["read"].record(back)

    for k in range(2 * n_slots):
        frame(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s_ in [sl["build_stream"] for sl in slots] + [st, up, back]:
        s_.wait_event(e0)
    for k in range(args.steps):
        frame(k)
    for sl in slots:
        stream.wait_event(sl["read"])
    stream.wait_event(last_in)
    e1.record(stream)
    e1.synchronize()
    for sl in slots:
        kdgb.check(sl["graph"].status(stream=stream), "graph rebuild")
    ms = e0.elapsed_time(e1) / args.steps
    h_outs = [sl["h_out"] for sl in slots]
    for sl in slots:
        if sl.get("own"):
            sl["graph"].close()
            sl["tree"].close()
    if part:
        torch.cuda.synchronize()
        part.close()
    return ms, h_outs


def run_frame(args, world, rank, local, pg):
    import torch
    import kdgb

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = kdgb.lib()
    tris, o, d = workload(args)
    n = o.shape[0]
    tris_d = torch.from_numpy(tris).to(dev)
    o_d = torch.from_numpy(o).to(dev)
    d_d = torch.from_numpy(d).to(dev)
    build_kw, build_desc = BUILDS[args.build]
    bp = kdgb.build_params(**build_kw)
    tp = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH, tile_width=args.width)
    tree = kdgb.KDTree.build(tris_d, bp)
    graph = None if args.host_build else kdgb.Graph(tree, tris_d, params=bp, headroom=HEADROOM)
    outs = (torch.empty(n, dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.float32, device=dev),
            torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.float32, device=dev),
            torch.empty(n, dtype=torch.int32, device=dev))
    stream = torch.cuda.current_stream()

    def build():
        if graph is not None:
            graph.launch()
        else:
            tree.rebuild(tris_d, bp)

    def step(ev=None):
        build()
        if ev:
            ev[0].record(stream)
        tree.trace_primary_shadow(o_d, d_d, configs.LIGHT, tp, out=outs)
        if ev:
            ev[1].record(stream)

    if args.profile:
        build()
        tree.trace_primary_shadow(o_d, d_d, configs.LIGHT, tp, out=outs)
        tree.trace_primary_shadow(o_d, d_d, configs.LIGHT, tp, out=outs)
        torch.cuda.synchronize()
        if graph is not None and graph.status() != 0:
            raise RuntimeError("graph rebuild failed")
        return

    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if graph is not None:
        kdgb.check(graph.status(), "graph rebuild")
    n_hits = int((outs[0] >= 0).sum().item())
    rays_per_step = n + n_hits
    st = tree.stats()

    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches0 = L.kdgb_launch_count()
    sampler.mark()
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
    if graph is not None:
        kdgb.check(graph.status(), "graph rebuild")
    total_ms = float(sum(step_ms))
    if pg:
        t = torch.tensor([total_ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = rays_per_step * world / (ms_per_step / 1e3) / 1e6
    # The outputs of the last timed step, for the parity and error records.
    gpu_out = tuple(x.cpu().numpy() for x in outs)
    gpu_tree = tree.to_host()

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
            "peak_source": f"{peak_kind} hbm_gbs",
            # The traversal is bound by issue and latency, not by HBM: the
            # committed profile of this kernel gives the ncu figures.
            "limiter": "issue/latency (ncu figures in profiles/k_trace_clustered1M_frame.md)"}
    if traffic:
        roof["traffic_source"] = traffic.get("source")
    # Logical bytes of the same trace (what the traversal reads from L1, L2
    # or HBM), from device step counters in a separate counting run after the
    # timed region: node records 8 B, leaf boxes 32 B, triangle records 48 B.
    c_outs = tuple(torch.empty_like(x) for x in outs)
    _, steps = tree.count_steps(o_d, d_d, configs.LIGHT, tp, out=c_outs)
    logical = sum(TRACE_BYTES[k] * (steps["primary"][k] + steps["shadow"][k]) for k in TRACE_BYTES)
    roof["logical"] = {"bytes_per_launch": logical, "gbs": logical / (tr_ms / 1e3) / 1e9,
                       "bytes_per_step": TRACE_BYTES, "steps": steps,
                       "outputs_equal_timed": all(torch.equal(a.view(torch.int32), b.view(torch.int32))
                                                  for a, b in zip(c_outs, outs)),
                       "source": "device step counters (kdgb_trace_count_steps), separate counting run"}

    # End to end through the public API with host buffers.
    e2e = None
    if not args.no_e2e:
        h_tris = torch.from_numpy(tris).pin_memory()
        h_o = torch.from_numpy(o).pin_memory()
        h_d = torch.from_numpy(d).pin_memory()
        h_out = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in outs]
        # Three copy streams keep the copies off the critical path:
        #  * the triangles of the next step are uploaded while this step's
        #    trace runs: the build reads the input triangles only while it
        #    loads them into its own arrays, and the trace never reads them;
        #  * the rays are uploaded while the tree is rebuilt (after the
        #    previous step's trace has read them);
        #  * the outputs are read back while the next step uploads and
        #    rebuilds; the next trace waits for the read-back before it
        #    rewrites the output buffers.
        # Each step of the timed loop issues one triangle upload, one ray
        # upload and one read-back of all outputs; the region ends when the
        # last read-back has landed.
        up = torch.cuda.Stream(device=dev)
        side = torch.cuda.Stream(device=dev)
        back = torch.cuda.Stream(device=dev)
        traced = torch.cuda.Event()
        traced.record(stream)
        read_back = torch.cuda.Event()
        read_back.record(stream)
        tris_in = torch.cuda.Event()
        with torch.cuda.stream(up):
            tris_d.copy_(h_tris, non_blocking=True)
        tris_in.record(up)

        def e2e_step():
            side.wait_event(traced)
            with torch.cuda.stream(side):
                o_d.copy_(h_o, non_blocking=True)
                d_d.copy_(h_d, non_blocking=True)
            rays_in = torch.cuda.Event()
            rays_in.record(side)
            stream.wait_event(tris_in)
            build()
            built = torch.cuda.Event()
            built.record(stream)
            up.wait_event(built)
            with torch.cuda.stream(up):
                tris_d.copy_(h_tris, non_blocking=True)  # the next step's triangles
            tris_in.record(up)
            stream.wait_event(rays_in)
            stream.wait_event(read_back)
            tree.trace_primary_shadow(o_d, d_d, configs.LIGHT, tp, out=outs)
            traced.record(stream)
            back.wait_event(traced)
            with torch.cuda.stream(back):
                for hb, db in zip(h_out, outs):
                    hb.copy_(db, non_blocking=True)
            read_back.record(back)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        stream.wait_event(read_back)
        stream.wait_event(tris_in)
        e1.record(stream)
        e1.synchronize()
        e2e_ms = e0.elapsed_time(e1) / args.steps
        if pg:
            t = torch.tensor([e2e_ms], device=dev)
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            e2e_ms = float(t.item())
        h2d = tris.nbytes + o.nbytes + d.nbytes
        d2h = sum(x.numel() * x.element_size() for x in outs)
        if graph is not None:
            inflight = e2e_frames_in_flight(args, dev, tree, graph, bp, tp, tris_d, o_d, d_d, outs, h_tris, h_o, h_d,
                                            stream, partition_sms=args.partition)
        one = {"value": rays_per_step * world / (e2e_ms / 1e3) / 1e6, "ms_per_step": e2e_ms,
               # The host copy of the last step must equal the device-timed
               # step's outputs (same inputs, same tree).
               "outputs_equal_device_steps": all(np.array_equal(hb.numpy(), g) for hb, g in zip(h_out, gpu_out))}
        e2e = {"value": one["value"], "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms, "frames_in_flight": 1,
               "outputs_equal_device_steps": one["outputs_equal_device_steps"]}
        if graph is not None:
            ms2, h_outs2 = inflight
            ms2_all = ms2
            if pg:
                t = torch.tensor([ms2], device=dev)
                pg.all_reduce(t, op=pg.ReduceOp.MAX)
                ms2_all = float(t.item())
            e2e.update({"value": rays_per_step * world / (ms2_all / 1e3) / 1e6, "ms_per_step": ms2_all,
                        "frames_in_flight": FRAMES_IN_FLIGHT,
                        "outputs_equal_device_steps": all(np.array_equal(hb.numpy(), g) for ho in h_outs2
                                                          for hb, g in zip(ho, gpu_out)),
                        "one_frame_in_flight": one})

    # The other build configuration on the same inputs, for context.
    variant = None
    if graph is not None:
        alt_kw, alt_desc = BUILDS["reference" if args.build == "tuned" else "tuned"]
        alt_bp = kdgb.build_params(**alt_kw)
        alt_tree = kdgb.KDTree.build(tris_d, alt_bp)
        alt_graph = kdgb.Graph(alt_tree, tris_d, params=alt_bp, headroom=HEADROOM)

        def alt_step():
            alt_graph.launch()
            alt_tree.trace_primary_shadow(o_d, d_d, configs.LIGHT, tp, out=outs)

        time_steps(alt_step, 3, stream)
        alt_ms = statistics.median(time_steps(alt_step, args.steps, stream, flush))
        kdgb.check(alt_graph.status(), "graph rebuild")
        alt_rays = n + int((outs[0] >= 0).sum().item())  # primary + one shadow ray per hit
        alt_st = alt_tree.stats()
        variant = {"build": alt_desc, "ms_per_step": alt_ms, "value": alt_rays / (alt_ms / 1e3) / 1e6,
                   "tree": {"nodes": alt_st.n_nodes, "refs": alt_st.n_refs}}
        alt_graph.close()
        alt_tree.close()

    cpu = parity = fp64 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        O = oracle_module()
        cpu, cpu_tree, idx, cpu_out = cpu_frame(O, tris, o, d, build_kw)
        parity = parity_record(gpu_tree, cpu_tree, idx, gpu_out, cpu_out)
        fp64 = fp64_error(O, tris, o, d, *gpu_out[:4], stride=2048)

    batched = None
    if rank == 0 and world == 1 and not args.no_batched and graph is not None:
        batched = measure_batched(args, steps=max(3, args.steps // 4), host_loop_steps=1)

    # The other configurations, each a compact copy of its own workload's
    # line (4096-triangle height field, photons, adjoint, the rows after the
    # hot path).
    others = None
    if rank == 0 and world == 1 and not args.no_others and graph is not None:
        keep = {"metric", "value", "unit", "ms_per_step", "higher_is_better", "config"}
        common = set(line_common(args, "", 0, "", True, 0, "", {}))
        others = {}
        for name, fn in (("small", measure_small), ("photons", measure_photons), ("adjoint", measure_adjoint),
                         ("next", measure_next)):
            others[name] = {k: v for k, v in fn(args).items() if k in keep or k not in common}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded clustered scene, pinhole camera)",
                "config": frame_config(args, build_desc, n_hits),
                "rebuild": "one graph launch" if graph is not None else "host-driven level loop",
                "build_ms": statistics.mean(s - t for s, t in zip(step_ms, trace_ms)),
                "trace_ms": tr_ms, "trace_mrays_s": rays_per_step / (tr_ms / 1e3) / 1e6,
                "tree": {"nodes": st.n_nodes, "refs": st.n_refs, "upper_levels": st.upper_levels,
                         "lower_levels": st.lower_levels},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clocks, "parity": parity, "fp64_err": fp64, "other_build": variant,
                "batched": batched, "other_configs": others}
        print(json.dumps(line), flush=True)
    if graph is not None:
        graph.close()
    tree.close()


# ---------------------------------------------------------------------------
# Other configurations (single GPU, rank 0 only).
# ---------------------------------------------------------------------------


def line_common(args, metric, value, unit, higher, ms, workload_desc, extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
         "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": higher, "scaling": "weak",
         "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": workload_desc}}
    d.update(extra)
    return d


def measure_small(args):
    """4096-triangle height field, 256x256 pinhole rays: SAH build, kd-restart
    and brute force.  Returns the workload's line."""
    import torch
    import kdgb
    from kdgb import scenes
    tris = scenes.heightfield(64, 32, seed=1)[0]
    o, d = scenes.camera_rays(256, 256)
    n = o.shape[0]
    td, od, dd = (torch.from_numpy(x).cuda() for x in (tris, o, d))
    stream = torch.cuda.current_stream()
    bp = kdgb.build_params(**configs.SAH)
    tree = kdgb.KDTree.build(td, bp)
    graph = kdgb.Graph(tree, td, params=bp, headroom=HEADROOM)
    tp = kdgb.trace_params(tracer=kdgb.TRACER_RESTART)
    outs = tuple(torch.empty(n, dtype=dt, device="cuda") for dt in (torch.int32, torch.float32, torch.float32,
                                                                      torch.float32))
    W = max(args.warmup, 3)
    res = {}
    for name, fn in (("host_build", lambda: tree.rebuild(td, bp)), ("graph_build", graph.launch),
                     ("restart", lambda: tree.trace(od, dd, tp, out=outs)),
                     ("brute", lambda: kdgb.trace_brute(td, od, dd))):
        time_steps(fn, W, stream)
        res[name] = statistics.median(time_steps(fn, args.steps, stream))
    kdgb.check(graph.status(), "graph rebuild")
    step_ms = res["graph_build"] + res["restart"]
    cpu = fp64 = None
    if not args.no_cpu_baseline:
        O = oracle_module()
        t0 = time.perf_counter()
        for _ in range(5):
            ot = O.build(tris, **configs.SAH)
        tb = (time.perf_counter() - t0) / 5
        t0 = time.perf_counter()
        for _ in range(5):
            O.trace(ot, tris, o, d, tracer=O.TRACER_RESTART)
        tt = (time.perf_counter() - t0) / 5
        t0 = time.perf_counter()
        O.trace(None, tris, o[::16], d[::16], tracer=O.TRACER_BRUTE)
        tbr = (time.perf_counter() - t0) * 16
        cpu = {"value": n / (tb + tt) / 1e6, "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "oracle build + kd-restart over all 65,536 rays (5 runs); brute force over every 16th ray",
               "build_ms": tb * 1e3, "restart_mrays_s": n / tt / 1e6, "brute_mrays_s": n / tbr / 1e6}
        fp64 = fp64_error(O, tris, o, d, *(x.cpu().numpy() for x in outs), stride=1)
    line = line_common(
        args, "kd-restart Mrays/s per step (4096-tri SAH build + 256x256 primary rays)", n / (step_ms / 1e3) / 1e6,
        "Mrays/s", True, step_ms, "heightfield-64x32 (4096 tris) 256x256 rays, SAH Ct=1 Ci=1.5 leaf 8",
        {"build_ms_graph": res["graph_build"], "build_ms_host": res["host_build"],
         "restart_trace_ms": res["restart"], "restart_mrays_s": n / (res["restart"] / 1e3) / 1e6,
         "brute_trace_ms": res["brute"], "brute_mrays_s": n / (res["brute"] / 1e3) / 1e6, "cpu_baseline": cpu,
         "fp64_err": fp64})
    graph.close()
    tree.close()
    return line


def run_small(args):
    print(json.dumps(measure_small(args)), flush=True)


def measure_photons(args):
    """Incoherent load: 16M photons from the frame's point light, 3
    cosine-weighted bounces with Russian roulette (p = 0.7), Philox stream;
    kd-restart vs short-stack on a 262,144-triangle clustered scene.  Returns
    the workload's line."""
    import torch
    import kdgb
    from kdgb import scenes
    T, P = configs.PHOTON_TRIS, configs.PHOTONS
    tris = scenes.clustered(T, seed=configs.FRAME_SEED)
    td = torch.from_numpy(tris).cuda()
    stream = torch.cuda.current_stream()
    tree = kdgb.KDTree.build(td, **configs.SAH)
    pkw = dict(light=configs.LIGHT, seed=configs.PHOTON_SEED, bounces=configs.PHOTON_BOUNCES,
               survival=configs.PHOTON_SURVIVAL)
    ph = kdgb.photon_params(**pkw)
    S = configs.PHOTON_BOUNCES + 1
    out = (torch.empty((P, S), dtype=torch.int32, device="cuda"),
           torch.empty((P, S), dtype=torch.float32, device="cuda"))
    W = max(args.warmup, 3)
    res = {}
    for name, tp in (("restart", kdgb.trace_params(tracer=kdgb.TRACER_RESTART)),
                     ("shortstack", kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK,
                                                      stack_depth=configs.STACK_DEPTH))):
        fn = lambda tp=tp: tree.trace_photons(P, tp, photons=ph, out=out)
        time_steps(fn, W, stream)
        res[name] = statistics.median(time_steps(fn, args.steps, stream))
    segs = int((out[0] != -2).sum().item())
    best = min(res, key=res.get)
    cpu = None
    if not args.no_cpu_baseline:
        O = oracle_module()
        ot = O.build(tris, **configs.SAH)
        sample = 1 << 20
        t0 = time.perf_counter()
        h, _ = O.trace_photons(ot, tris, sample, tracer=O.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH, **pkw)
        dt = time.perf_counter() - t0
        cpu = {"value": int((h != -2).sum()) / dt / 1e6, "unit": "Msegments/s", "cores": os.cpu_count(),
               "kind": "port", "sample": f"first {sample} photons, short-stack, OpenMP over all host cores",
               "segments_equal_gpu": bool(np.array_equal(h, out[0][:sample].cpu().numpy()))}
    line = line_common(
        args, "photon segments Msegments/s (262k-tri clustered, 16M photons x 3 bounces)",
        segs / (res[best] / 1e3) / 1e6, "Msegments/s", True, res[best],
        "clustered-262144-tris, 16M photons from (0.5,3,0.5), 3 bounces, RR p=0.7",
        {"segments": segs, "ms": res, "msegments_s": {k: segs / (v / 1e3) / 1e6 for k, v in res.items()},
         "best": best, "cpu_baseline": cpu})
    tree.close()
    return line


def run_photons(args):
    print(json.dumps(measure_photons(args)), flush=True)


def profile_batched(args):
    """--workload batched --profile: one host-driven forest build and one
    batched trace under each schedule, nothing timed (for ncu captures)."""
    import torch
    import kdgb
    R = configs.BATCH_RAYS_PER_MESH
    meshes, off, o, d = configs.batch_scene(n_meshes=args.meshes)
    td, od, dd = (torch.from_numpy(x).cuda() for x in (np.concatenate(meshes), o, d))
    bp = kdgb.build_params(**dict(configs.TUNED, leaf_size=16))
    with kdgb.KDTree.build_batch(td, off, bp) as forest:
        for sch in (kdgb.SCHEDULE_GRID, kdgb.SCHEDULE_QUEUE):
            forest.trace_batch(od, dd, rays_per_mesh=R, tracer=kdgb.TRACER_SHORTSTACK, stack_depth=8,
                               block_size=64, schedule=sch)
        torch.cuda.synchronize()


def measure_batched(args, steps, host_loop_steps=2, check_meshes=8):
    """512 meshes, parameters from the autotuner:
      * one graph: forest build of all meshes + batched trace (one launch);
      * per-mesh graph loop: one graph per mesh (its rebuild + its rays),
        launched one after another on one stream, no host synchronisation;
      * the same per-mesh graphs over CONCURRENT_STREAMS streams, largest
        meshes first (independent meshes overlap);
      * per-mesh host loop: host-driven rebuild + trace per mesh.
    Returns the record; the hits of all four must be identical, and a few
    meshes are checked against the oracle."""
    import torch
    import kdgb
    R = configs.BATCH_RAYS_PER_MESH
    meshes, off, o, d = configs.batch_scene(n_meshes=args.meshes)
    M = len(meshes)
    tris = np.concatenate(meshes)
    td, od, dd = (torch.from_numpy(x).cuda() for x in (tris, o, d))
    stream = torch.cuda.current_stream()
    base_b = kdgb.build_params(**configs.TUNED)
    base_t = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH)
    t0 = time.perf_counter()
    tuned = kdgb.autotune(td, od, dd, mesh_offsets=off, rays_per_mesh=R, build=base_b, trace=base_t,
                          builds_per_trace=1.0, reps=2)
    tune_s = time.perf_counter() - t0
    bp, tp = tuned.build, tuned.trace
    tp.tile_width = 0
    forest = kdgb.KDTree.build_batch(td, off, bp)
    graph = kdgb.Graph(forest, td, mesh_offsets=off, params=bp, headroom=HEADROOM, o=od, d=dd, rays_per_mesh=R,
                       trace=tp)
    time_steps(graph.launch, 3, stream)
    g_ms = time_steps(graph.launch, steps, stream)
    kdgb.check(graph.status(), "graph rebuild")
    hits = int((graph.out[0] >= 0).sum().item())
    ghit = graph.out[0].cpu().numpy()
    # The forest's trace alone under both schedules (the autotuner picked
    # one): one thread per ray, or the persistent queue.
    sched_ms = {}
    for name, sch in (("grid", kdgb.SCHEDULE_GRID), ("queue", kdgb.SCHEDULE_QUEUE)):
        tps = kdgb.TraceParams.from_buffer_copy(tp)
        tps.schedule = sch
        fn = lambda tps=tps: forest.trace_batch(od, dd, rays_per_mesh=R, params=tps)
        time_steps(fn, 2, stream)
        sched_ms[name] = statistics.median(time_steps(fn, steps, stream))

    views = [td[off[m]:off[m + 1]] for m in range(M)]
    oviews = [(od[m * R:(m + 1) * R], dd[m * R:(m + 1) * R]) for m in range(M)]
    trees = [kdgb.KDTree.build(views[m], bp) for m in range(M)]
    louts = [tuple(torch.empty(R, dtype=dt, device="cuda") for dt in (torch.int32, torch.float32, torch.float32,
                                                                      torch.float32)) for _ in range(M)]
    mgraphs = [kdgb.Graph(trees[m], views[m], params=bp, headroom=HEADROOM, o=oviews[m][0], d=oviews[m][1],
                          trace=tp, out=louts[m]) for m in range(M)]

    def graph_loop():
        for g in mgraphs:
            g.launch()

    time_steps(graph_loop, 2, stream)
    gl_ms = time_steps(graph_loop, steps, stream)
    for g in mgraphs:
        kdgb.check(g.status(), "per-mesh graph rebuild")
    same_graph_loop = all(np.array_equal(louts[m][0].cpu().numpy(), ghit[m * R:(m + 1) * R]) for m in range(M))

    # The same per-mesh graphs spread over concurrent streams (largest meshes
    # first), so independent meshes overlap as independent work items would.
    streams = [torch.cuda.Stream() for _ in range(CONCURRENT_STREAMS)]
    by_size = np.argsort([-mt.shape[0] for mt in meshes], kind="stable")

    def streams_loop():
        start = torch.cuda.Event()
        start.record(stream)
        for s in streams:
            s.wait_event(start)
        for j, m in enumerate(by_size):
            mgraphs[m].launch(stream=streams[j % len(streams)])
        for s in streams:
            done = torch.cuda.Event()
            done.record(s)
            stream.wait_event(done)

    for g in louts:
        g[0].fill_(-2)
    time_steps(streams_loop, 2, stream)
    gs_ms = time_steps(streams_loop, steps, stream)
    for g in mgraphs:
        kdgb.check(g.status(), "per-mesh graph rebuild")
    same_streams = all(np.array_equal(louts[m][0].cpu().numpy(), ghit[m * R:(m + 1) * R]) for m in range(M))
    for g in mgraphs:
        g.close()

    def host_loop():
        for m in range(M):
            trees[m].rebuild(views[m], bp)
            trees[m].trace(oviews[m][0], oviews[m][1], tp, out=louts[m])

    time_steps(host_loop, 1, stream)
    hl_ms = time_steps(host_loop, host_loop_steps, stream)
    same_host_loop = all(np.array_equal(louts[m][0].cpu().numpy(), ghit[m * R:(m + 1) * R]) for m in range(M))

    # A few meshes (small to large) against the oracle's own tree and tracer.
    O = oracle_module()
    okw = oracle_kwargs(bp)
    order = np.argsort([mt.shape[0] for mt in meshes])
    picks = order[np.linspace(0, M - 1, check_meshes).astype(np.int64)]
    oracle_ok = True
    for m in picks:
        ot = O.build(meshes[m], **okw)
        hr, _, _, _ = O.trace(ot, meshes[m], o[m * R:(m + 1) * R], d[m * R:(m + 1) * R], tracer=tp.tracer,
                              stack_depth=tp.stack_depth)
        oracle_ok &= bool(np.array_equal(hr, ghit[m * R:(m + 1) * R]))

    g, gl, hl = statistics.median(g_ms), statistics.median(gl_ms), statistics.median(hl_ms)
    gs = statistics.median(gs_ms)
    rec = {"workload": "%d clustered meshes log-uniform [1k,200k] tris (%d total), 64k random rays each"
                       % (M, tris.shape[0]),
           "meshes": M, "tris": int(tris.shape[0]), "rays": M * R, "one_graph_ms": g, "meshes_per_s": M / (g / 1e3),
           "rays_mrays_s": M * R / (g / 1e3) / 1e6, "hits": hits,
           "per_mesh_graph_loop_ms": gl, "per_mesh_host_loop_ms": hl,
           "speedup_vs_per_mesh_graph_loop": gl / g, "speedup_vs_per_mesh_host_loop": hl / g,
           "per_mesh_graphs_concurrent_ms": gs, "concurrent_streams": CONCURRENT_STREAMS,
           "speedup_vs_per_mesh_graphs_concurrent": gs / g,
           "parity": {"graph_loop_hits_identical": bool(same_graph_loop),
                      "concurrent_graphs_hits_identical": bool(same_streams),
                      "host_loop_hits_identical": bool(same_host_loop),
                      "oracle_meshes_checked": int(check_meshes), "oracle_hit_ids_equal": bool(oracle_ok)},
           "trace_only_ms": sched_ms,
           "autotune": {"leaf_size": bp.leaf_size, "sah_bins": bp.sah_bins, "stack_depth": tp.stack_depth,
                        "block_size": tp.block_size,
                        "schedule": "queue" if tp.schedule == kdgb.SCHEDULE_QUEUE else "grid",
                        "objective_ms": tuned.objective, "baseline_ms": tuned.baseline,
                        "trials": tuned.trials, "seconds": tune_s, "scored_on": "graph rebuild + trace"}}
    graph.close()
    forest.close()
    for t in trees:
        t.close()
    return rec


def run_batched(args):
    if args.profile:
        profile_batched(args)
        return
    rec = measure_batched(args, steps=args.steps, host_loop_steps=max(2, args.steps // 3))
    print(json.dumps(line_common(
        args, "batched build+trace of %d meshes, meshes/s (one graph launch)" % rec["meshes"], rec["meshes_per_s"],
        "meshes/s",
        True, rec["one_graph_ms"], rec["workload"], {"batched": rec})), flush=True)


def measure_adjoint(args):
    """Backward pass of t and barycentrics w.r.t. the vertices of a 100k
    triangle height field for 512x512 rays with fixed forward hits.  Returns
    the workload's line."""
    import torch
    import kdgb
    from kdgb import scenes
    tris, verts, idx = scenes.heightfield(316, 158, seed=5)
    o, d = scenes.camera_rays(512, 512)
    n = o.shape[0]
    stream = torch.cuda.current_stream()
    td = torch.from_numpy(tris).cuda()
    vd = torch.from_numpy(np.ascontiguousarray(verts, dtype=np.float32)).cuda()
    idd = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).cuda()
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    tree = kdgb.KDTree.build(td, **configs.SAH)
    hit, t, u, v = tree.trace(od, dd)
    g = torch.Generator(device="cpu").manual_seed(7)
    w = torch.randn(n, generator=g).cuda()
    wv = torch.randn(n, generator=g).cuda()
    grad = torch.zeros_like(vd)
    fn = lambda: kdgb.backward(vd, idd, od, dd, hit, w, wv, wv, out=grad)
    W = max(args.warmup, 3)
    time_steps(fn, W, stream)
    b_ms = statistics.median(time_steps(fn, args.steps, stream))
    f_ms = statistics.median(time_steps(lambda: tree.trace(od, dd), args.steps, stream))
    line = line_common(
        args, "adjoint backward ms (100k-tri height field, 512x512 rays)", b_ms, "ms", False, b_ms,
        "heightfield-316x158 (%d tris), 512x512 rays, loss sum w*t + v*(u+v)" % tris.shape[0],
        {"forward_trace_ms": f_ms, "hits": int((hit >= 0).sum().item()),
         "backward_mrays_s": n / (b_ms / 1e3) / 1e6})
    tree.close()
    return line


def run_adjoint(args):
    print(json.dumps(measure_adjoint(args)), flush=True)


# The rows after the hot path, on frame-sized inputs: a moving surface
# collected and shaded each frame (GeometryList::AddMesh,
# OscCUDAMeshNode::UpdateSurface, the tracers' shading loop), Woop's test, and
# the balanced lower creator and DIVIDE split method of the build.
OSC_DETAIL = 724         # (724+1)^2 vertices, 1,048,352 triangles
OSC_HEIGHT = 0.0
OSC_TIME = 0.75


def osc_surface(detail=OSC_DETAIL):
    """The oscillating surface's grid (OscCUDAMeshNode.cu:27-67): vertices
    i * 0.1, height, j * 0.1, normals, colours and its index buffer."""
    from kdgb import scenes
    d = detail + 1
    i, j = np.meshgrid(np.arange(d), np.arange(d), indexing="xy")
    verts = np.stack([i.ravel() * 0.1, np.full(d * d, OSC_HEIGHT), j.ravel() * 0.1, np.ones(d * d)],
                     1).astype(np.float32)
    idx = scenes.grid_indices(detail, detail).astype(np.int32)
    normals = np.zeros_like(verts)
    normals[:, 1] = 1.0
    g = np.arange(d * d, dtype=np.int64) % 251
    cols = np.stack([g, 255 - g, (g * 3) % 256, np.where(g % 3 == 0, 128, 255)], 1).astype(np.uint8)
    return verts, normals, cols, idx


def measure_next(args):
    """The rows after the hot path.  A dynamic frame: the surface is moved
    (kdgb_osc_update_surface), collected into triangles and per-triangle
    attributes (kdgb_geometry_gather, kdgb_geometry_gather_attributes; a model
    matrix fits it into the unit cube), rebuilt by one graph launch (tuned
    build) and shaded (kdgb_trace_shaded, short-stack, 1920x1080, reflections
    until alpha 0.97).  On the 1M-triangle frame scene: primary rays with Woop's
    test against Moeller-Trumbore, and the balanced lower creator and the
    DIVIDE split method as graph rebuilds.  Parity: pixels, hit ids and trees
    against the oracle.  Returns the workload's line."""
    import ctypes as C
    import torch
    import kdgb
    from kdgb import scenes
    W = max(args.warmup, 3)
    stream = torch.cuda.current_stream()
    L = kdgb.lib()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    sp = lambda: C.c_void_p(stream.cuda_stream)
    verts, normals, cols, idx = osc_surface()
    T = idx.shape[0] // 3
    vd, nd = torch.from_numpy(verts).cuda(), torch.from_numpy(normals).cuda()
    cd, idd = torch.from_numpy(cols).cuda(), torch.from_numpy(idx).cuda()
    s = 1.0 / (0.1 * OSC_DETAIL)
    model = np.array([s, 0, 0, 0, 0, 1, 0, 0.3, 0, 0, s, 0, 0, 0, 0, 1], np.float32)
    tris = torch.empty((T, 9), dtype=torch.float32, device="cuda")
    n0, n1, n2 = (torch.empty((T, 4), dtype=torch.float32, device="cuda") for _ in range(3))
    c0 = torch.empty((T, 4), dtype=torch.uint8, device="cuda")
    o, d = scenes.camera_rays(configs.WIDTH, configs.HEIGHT)
    od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    n = o.shape[0]
    clock = [0.0]

    def update():
        clock[0] += 1.0 / 60.0
        kdgb.check(L.kdgb_osc_update_surface(ptr(vd), ptr(nd), OSC_DETAIL, OSC_HEIGHT, OSC_TIME + clock[0], sp()),
                   "kdgb_osc_update_surface")

    def gather():
        kdgb.check(L.kdgb_geometry_gather(ptr(vd), vd.shape[0], ptr(idd), idd.shape[0],
                                          model.ctypes.data_as(C.c_void_p), ptr(tris), sp()),
                   "kdgb_geometry_gather")
        kdgb.check(L.kdgb_geometry_gather_attributes(ptr(nd), ptr(cd), vd.shape[0], ptr(idd), idd.shape[0], None,
                                                     ptr(n0), ptr(n1), ptr(n2), ptr(c0), sp()),
                   "kdgb_geometry_gather_attributes")

    update()
    gather()
    bp = kdgb.build_params(**configs.TUNED)
    tree = kdgb.KDTree.build(tris, bp)
    graph = kdgb.Graph(tree, tris, params=bp, headroom=HEADROOM)
    tp = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH, tile_width=configs.WIDTH)
    rgba = torch.empty((n, 4), dtype=torch.uint8, device="cuda")
    shade = lambda: tree.trace_shaded(od, dd, n0, n1, n2, c0, tp, out=rgba)
    stages = (("update", update), ("gather", gather), ("rebuild", graph.launch), ("shade", shade))

    def frame():
        for _, fn in stages:
            fn()

    time_steps(frame, W, stream)
    frame_ms = statistics.median(time_steps(frame, args.steps, stream))
    stage_ms = {}
    for name, fn in stages:
        stage_ms[name] = statistics.median(time_steps(fn, args.steps, stream))
    kdgb.check(graph.status(), "graph rebuild")
    frame_ms_final = frame_ms
    # Parity of the last frame: the oracle builds the same triangles and
    # shades every 97th ray with the same attributes.
    update()
    gather()
    graph.launch()
    shade()
    torch.cuda.synchronize()
    kdgb.check(graph.status(), "graph rebuild")
    parity = cpu = None
    if not args.no_cpu_baseline:
        O = oracle_module()
        ht, h0, h1, h2, hc = (x.cpu().numpy() for x in (tris, n0, n1, n2, c0))
        t0 = time.perf_counter()
        ot = O.build(ht, **configs.TUNED)
        tb = time.perf_counter() - t0
        sel = np.arange(0, n, 97)
        t0 = time.perf_counter()
        want = O.trace_shaded(ot, ht, o[sel], d[sel], h0, h1, h2, hc, tracer=O.TRACER_SHORTSTACK,
                              stack_depth=configs.STACK_DEPTH)
        ts = (time.perf_counter() - t0) * n / sel.size
        got = rgba.cpu().numpy()[sel]
        parity = {"against": "oracle, same triangles, attributes and tracer (CPU)", "pixels_checked": int(sel.size),
                  "pixels_equal": bool(np.array_equal(got, want)),
                  "lit_pixels": int((want[:, 3] > 0).sum())}
        cpu = {"value": n / (tb + ts) / 1e6, "unit": "Mrays/s (primary rays shaded)", "cores": os.cpu_count(),
               "kind": "port", "sample": "oracle build of the frame's triangles + shaded trace of every 97th ray, "
                                         "extrapolated to the frame", "build_ms": tb * 1e3}
    graph.close()
    tree.close()

    # Woop's test against Moeller-Trumbore, and the other build options, on
    # the frame scene.
    ftris, fo, fd = configs.frame_scene()
    ftd, fod, fdd = (torch.from_numpy(x).cuda() for x in (ftris, fo, fd))
    fn_ = fo.shape[0]
    extra = {}
    with kdgb.KDTree.build(ftd, bp) as ft:
        out = tuple(torch.empty(fn_, dtype=dt, device="cuda") for dt in (torch.int32, torch.float32, torch.float32,
                                                                          torch.float32))
        res = {}
        for name, isect in (("moeller_trumbore", kdgb.ISECT_MOELLER), ("woop", kdgb.ISECT_WOOP)):
            ptp = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH,
                                    tile_width=configs.WIDTH, intersection=isect)
            fn = lambda ptp=ptp: ft.trace(fod, fdd, ptp, out=out)
            time_steps(fn, W, stream)
            res[name] = statistics.median(time_steps(fn, args.steps, stream))
        woop_hits = out[0].cpu().numpy()
        woop = {"trace_ms": res, "mrays_s": {k: fn_ / (v / 1e3) / 1e6 for k, v in res.items()},
                "note": "primary rays of the frame; Woop's rows are recomputed from the geometry at the first "
                        "trace after each rebuild"}
        if not args.no_cpu_baseline:
            O = oracle_module()
            oft = O.build(ftris, **configs.TUNED)
            sel = np.arange(0, fn_, 61)
            wh = O.trace(oft, ftris, fo[sel], fd[sel], tracer=O.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH,
                         intersection=O.ISECT_WOOP)[0]
            woop["parity"] = {"rays_checked": int(sel.size), "hit_ids_equal": bool(np.array_equal(wh, woop_hits[sel]))}
        extra["woop"] = woop
    builds = {}
    for name, kw in (("balanced", dict(configs.TUNED, lower=kdgb.LOWER_BALANCED, traversal_cost=16.0)),
                     ("divide", dict(configs.TUNED, split_method=kdgb.SPLIT_DIVIDE))):
        bp2 = kdgb.build_params(**kw)
        with kdgb.KDTree.build(ftd, bp2) as bt:
            g2 = kdgb.Graph(bt, ftd, params=bp2, headroom=HEADROOM)
            time_steps(g2.launch, W, stream)
            b_ms = statistics.median(time_steps(g2.launch, args.steps, stream))
            kdgb.check(g2.status(), "graph rebuild")
            ptp = kdgb.trace_params(tracer=kdgb.TRACER_SHORTSTACK, stack_depth=configs.STACK_DEPTH,
                                    tile_width=configs.WIDTH)
            fn = lambda: bt.trace(fod, fdd, ptp)
            time_steps(fn, W, stream)
            t_ms = statistics.median(time_steps(fn, args.steps, stream))
            st = bt.stats()
            rec = {"build": kw, "rebuild_ms_graph": b_ms, "primary_trace_ms": t_ms,
                   "tree": {"nodes": st.n_nodes, "refs": st.n_refs}}
            if not args.no_cpu_baseline:
                O = oracle_module()
                ref = O.build(ftris, **kw)
                h = bt.to_host()
                rec["parity"] = {"tree_arrays_equal": all(
                    np.array_equal(getattr(h, f).view(np.uint32) if getattr(h, f).dtype.kind == "f" else getattr(h, f),
                                   getattr(ref, f).view(np.uint32) if getattr(ref, f).dtype.kind == "f"
                                   else getattr(ref, f))
                    for f in ("info", "split", "children", "bitmap", "prim_indices", "leaf_ids", "aabb_min",
                              "aabb_max", "area"))}
            g2.close()
        builds[name] = rec
    extra["builds"] = builds
    line = line_common(
        args, "dynamic surface frame Mrays/s (surface update + collection + graph rebuild + shaded trace)",
        n / (frame_ms_final / 1e3) / 1e6, "Mrays/s", True, frame_ms_final,
        "oscillating surface %d^2 cells (%d tris), 1920x1080 shaded, short-stack depth 8; frame scene for Woop and "
        "the build options" % (OSC_DETAIL, T),
        {"stage_ms": stage_ms, "parity": parity, "cpu_baseline": cpu, **extra})
    return line


def run_next(args):
    print(json.dumps(measure_next(args)), flush=True)


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "frame":
        run_frame(args, world, rank, local, pg)
    elif rank == 0:
        import torch
        torch.cuda.set_device(local)
        {"small": run_small, "photons": run_photons, "batched": run_batched, "adjoint": run_adjoint,
         "next": run_next}[args.workload](args)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
