"""Benchmark of the CUDA renderer level on the 20,000-path 4K scene.

One step = one full frame of the compute rasterization path (bound, flatten,
bin, backdrop propagation, fill grouping, fill + composite) over the seeded
synthetic 4K scene (20,000 paths, ~2.1M segments) into an RGBA8 3840x2160
target.  `value` is input segments per second with the scene resident in HBM
(L2 flushed between steps); `e2e` is the same metric through the public API
with host buffers: scene upload from pinned host memory, render, and the
RGBA8 image read back, every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cuda|reference]

`--impl reference` times the CPU restatement of the reference's Rayon + SIMD
CPU tiling path (tiling, FP32 coverage, composite) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mseg/s"
WORKLOAD = "svg_4k_20000_paths"
W, H = 3840, 2160


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0])); mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# Stages that are one kernel each (the roofline names one kernel).
# Stages that are one kernel in a plain frame (the flattening is one pass there).
STAGE_KERNELS = {"bound": "k_bound", "flatten": "k_flatten_count", "bin_count": "k_bin_count",
                 "bin_emit": "k_bin_emit", "fill": "k_mask", "composite": "k_composite"}


def measured_traffic(kernel_stage: str, full_size: bool, variant: str = "plain"):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    capture of the full-size frame of the same workload
    (profiles/svg4k_dram_full.md, svg4k_paints_dram_full.md,
    svg4k_d3d11_dram_full.md), for full-size workloads only."""
    if not full_size:
        return None, None
    name = {"plain": "svg4k_dram_full.md", "paints": "svg4k_paints_dram_full.md",
            "d3d11": "svg4k_d3d11_dram_full.md"}[variant]
    rel = os.path.join("profiles", name)
    key = f"traffic_bytes_per_launch {kernel_stage}:"
    try:
        with open(os.path.join(ROOT, rel)) as f:
            for line in f:
                if line.startswith(key):
                    return int(line.split(":")[1]), rel
    except OSError:
        pass
    return None, None


def stage_bytes(st, npts: int, nseg: int) -> dict:
    """Bytes each stage must move in this design, from per-unit figures:
    8 B per point and per segment record, 20 B per flattened line (an
    intermediate: written once, read by both binning passes), 8 B per fill
    (LineSegmentU16) written by the emit pass, 16 B per path tile record;
    the fill pass reads the 8 B fills of the visible mask tiles and writes
    their coverage (512 B: 256 pixels of 16-bit unorm) and reads a 16 B work
    item each; the composite reads that coverage and a 24 B record and key
    per visible tile and writes 4 B per pixel.  `frame` is the path's own
    formula, 8P + 8S + 12F + 16T + 256A + 4WH (12 B Fill records and 1 B mask
    pixels, as the reference stores them)."""
    P, S, F, T, A, L = npts, nseg, st.fill_count, st.tile_count, st.alpha_tile_count, st.line_count
    V, Am, Fm = st.visible_tile_count, st.mask_tile_count, st.mask_fill_count
    return {
        "bound": 8 * P,
        "flatten": 8 * P + 8 * S + 20 * L,
        "bin_count": 20 * L + 4 * L,
        "scans": 4 * L + 8 * T,
        "bin_emit": 20 * L + 8 * F,
        "propagate": 16 * T,
        "visibility": 16 * T,
        "fill": 8 * Fm + 528 * Am,
        "composite": 512 * Am + 24 * V + 4 * W * H,
        "frame": 8 * P + 8 * S + 12 * F + 16 * T + 256 * A + 4 * W * H,
    }


def job_totals(dist, segments: float, times_ms):
    """Whole-job figures of replica ranks: the input segments summed over the
    ranks (each renders its own scene) and each time the maximum over the
    ranks (the job ends with its slowest rank).  With no process group, this
    rank's own figures."""
    if dist is None:
        return float(segments), [float(t) for t in times_ms]
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    s = torch.tensor([float(segments)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(v) for v in times_ms], dtype=torch.float64, device=dev)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(s.item()), [float(v) for v in t.tolist()]


def svg_config(scene, args, paints, world: int = 1) -> dict:
    """The `config` of a 4K-scene line, the same in both arms."""
    return {"workload": (WORKLOAD if args.scale == 1.0 else f"{WORKLOAD}_scale{args.scale}")
                        + ("_paints" if paints else ""),
            **({"paints": paints} if paints else {}),
            "paths": len(scene.draw_paths), "clip_paths": len(scene.clip_paths), "segments": scene.segment_count,
            "points": len(scene.points), "width": W, "height": H, "seed": args.seed,
            "l2": "GPU arm: flushed between steps (512 MiB write); CPU arm: frames far larger than the host caches",
            "parallelism": f"replicas{world}",
            "tiling": "d3d11 level (uniform dicing)" if args.d3d11 else "cpu tiler (bit-exact)"}


def run_reference(args) -> None:
    """The reference arm: the oracle's CPU restatement of the reference's
    Rayon + SIMD CPU tiling path on all host threads.  It loads only the
    oracle's library (which carries its own copy of the scene generator), not
    the CUDA renderer."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import pathfinder_gb300 as pf
    import oracle
    oracle.build()
    scene = oracle.generate_scene(pf.PF_SCENE_SVG_4K, seed=args.seed, scale=args.scale)
    paints = add_paints(scene, args.seed) if args.paints else None
    nseg = scene.segment_count
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.cpu_frame(scene, W, H, threads)
    times = []
    for _ in range(args.steps):
        secs, _, counts = oracle.cpu_frame(scene, W, H, threads)
        times.append(secs)
    ms = 1e3 * sum(times) / len(times)
    value = nseg / (ms / 1e3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded PF_SCENE_SVG_4K: 20,000 log-normal star paths, 40/30/30 line/quad/cubic)",
        "config": svg_config(scene, args, paints, world),
        "cpu_baseline": {"value": round(value, 4), "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full frames of the 4K scene (tiling + FP32 coverage + composite)"},
        "e2e": {"value": round(value, 4), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mpx_per_s": round(W * H / (ms / 1e3) / 1e6, 3),
    }
    print(json.dumps(line), flush=True)


def add_paints(scene, seed: int) -> str:
    """Seeded paint effects over the generated scene: a quarter of the draw
    paths take one of 64 gradients (linear and radial, clamp and repeat, four
    random stops), a twentieth of the rest one of 8 image patterns, a tenth
    take a blend mode other than SrcOver (uniform over the other 26).
    Returns the description for the JSON line."""
    import numpy as np
    import pathfinder_gb300 as pf
    rng = np.random.default_rng(seed + 7)
    w, h = scene.width, scene.height
    for k in range(64):
        if k % 2 == 0:
            g = pf.Gradient.linear((rng.uniform(0, w), rng.uniform(0, h)), (rng.uniform(0, w), rng.uniform(0, h)))
        else:
            g = pf.Gradient.radial((rng.uniform(0, w), rng.uniform(0, h)), (0.0, rng.uniform(50, 800)))
        g.set_wrap(pf.GradientWrap.REPEAT if k % 4 >= 2 else pf.GradientWrap.CLAMP)
        for _ in range(4):
            g.add_color_stop(pf.ColorU(*[int(v) for v in rng.integers(0, 256, 3)], int(rng.integers(96, 256))),
                             float(rng.uniform(0, 1)))
        scene.push_gradient(g)
    patterns = []
    for k in range(8):  # 64x64 images: repeat/clamp, linear/nearest, a blur, a colour matrix
        px = rng.integers(0, 256, (64, 64, 4)).astype(np.uint8)
        px[..., 3] = np.maximum(px[..., 3], 96)
        p = pf.Pattern.from_image(px)
        p.repeat_x, p.repeat_y, p.smoothing = k % 2 == 0, k % 4 < 2, k != 3
        s = float(rng.uniform(0.5, 4.0))
        p.apply_transform((s, 0.0, 0.0, s, rng.uniform(0, w), rng.uniform(0, h)))
        if k == 5:
            p.set_blur(2.0, "x")
        elif k == 6:
            p.set_color_matrix(np.array([[0.3, 0.3, 0.3, 0], [0.59, 0.59, 0.59, 0], [0.11, 0.11, 0.11, 0],
                                         [0, 0, 0, 1], [0, 0, 0, 0]], np.float32))
        patterns.append(p)
    n = len(scene.draw_paths)
    pick = rng.random(n) < 0.25
    scene.draw_paths["overlay"][pick] = rng.integers(1, 65, int(pick.sum()))
    patt = (~pick) & (rng.random(n) < 0.05)
    scene.draw_paths["overlay"][patt] = [scene.PATTERN_OVERLAY_BASE + scene.push_pattern(patterns[int(i)])
                                         for i in rng.integers(0, 8, int(patt.sum()))]
    bm = rng.random(n) < 0.10
    scene.draw_paths["blend_mode"][bm] = rng.integers(1, 27, int(bm.sum()))
    scene.epoch += 1
    return (f"{int(pick.sum())} paths with one of 64 gradients (linear/radial, clamp/repeat), "
            f"{int(patt.sum())} with one of 8 64x64 image patterns (repeat/clamp, linear/nearest, a blur, "
            f"a colour matrix), {int(bm.sum())} with a blend mode other than SrcOver")


def cpu_baseline(scene, nseg: int, budget_s: float = 12.0) -> dict:
    import oracle
    threads = os.cpu_count() or 1
    oracle.cpu_frame(scene, W, H, threads)  # warm
    times = []
    t0 = time.time()
    while time.time() - t0 < budget_s or len(times) < 2:
        secs, _, _ = oracle.cpu_frame(scene, W, H, threads)
        times.append(secs)
        if len(times) >= 50:
            break
    ms = 1e3 * sum(times) / len(times)
    return {"value": round(nseg / (ms / 1e3) / 1e6, 4), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(times)} full frames of the 4K scene, all host threads ({ms:.1f} ms/frame)"}


def run_atlas(args) -> None:
    """The 16,384-glyph 4096x4096 R8 atlas as its own bench line."""
    import torch
    from pathfinder_gb300 import build as pbuild
    pbuild.build()
    torch.cuda.set_device(0)
    line = atlas_measure(args.seed, args.scale, args.steps, args.warmup, args.autotune)
    print(json.dumps(line), flush=True)


def atlas_measure(seed: int, scale: float, steps: int, warmup: int, autotune: bool = False) -> dict:
    """The 16,384-glyph 4096x4096 R8 atlas: one batched frame (all glyph
    scenes in one set of launches, replayed from a CUDA graph) against plain
    per-glyph frames on the same GPU, with identical output."""
    import torch
    import pathfinder_gb300 as pf

    stream = torch.cuda.Stream()
    prev_stream = torch.cuda.current_stream()
    torch.cuda.set_stream(stream)
    atlas = pf.generate_scene(pf.PF_SCENE_GLYPH_ATLAS, seed=seed, scale=scale)
    batch = pf.SceneBatch.glyphs_of(atlas)
    n, W_, H_ = len(batch), atlas.width, atlas.height
    nseg = atlas.segment_count
    r = pf.Renderer(0)
    r.set_stream(stream.cuda_stream)
    batched = torch.zeros((H_, W_), dtype=torch.uint8, device="cuda")
    per_glyph = torch.zeros_like(batched)
    r.render_batch(batch, batched, pf.PF_CUDA_FORMAT_R8)
    tuning = r.autotune(batch, batched, pf.PF_CUDA_FORMAT_R8, repeats=3) if autotune else r.get_tuning()
    st = r.stats()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn, reps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / reps

    for _ in range(warmup):
        r.render_batch(batch, batched, pf.PF_CUDA_FORMAT_R8, sync=False)
    ms_batched = timed(lambda: r.render_batch(batch, batched, pf.PF_CUDA_FORMAT_R8, sync=False), steps)
    r.graph_capture(batch, batched, pf.PF_CUDA_FORMAT_R8)
    for _ in range(warmup):
        r.graph_launch()
    ms_graph = timed(r.graph_launch, steps)
    r.graph_release()
    code, _ = r.render_status()
    assert code == 0, code

    def all_glyphs():
        for g in range(n):
            r.render_batch(batch, per_glyph, pf.PF_CUDA_FORMAT_R8, first=g, count=1, sync=False)

    all_glyphs()  # warm
    t0 = time.perf_counter()
    ms_per_glyph = timed(all_glyphs, 1)
    wall_per_glyph = 1e3 * (time.perf_counter() - t0)
    code, _ = r.render_status()
    assert code == 0, code
    identical = bool(torch.equal(batched, per_glyph))
    line = {
        "metric": "glyphs/s", "value": round(n / (ms_graph / 1e3), 1), "unit": "glyphs/s", "n_gpus": 1,
        "steps": steps, "warmup": warmup, "ms_per_step": round(ms_graph, 4), "higher_is_better": True,
        "dtype": "f32", "data": "synthetic (seeded PF_SCENE_GLYPH_ATLAS: quadratic glyph outlines with holes)",
        "config": {"workload": "glyph_atlas_16384" if scale == 1.0 else f"glyph_atlas_scale{scale}",
                   "glyphs": n, "segments": nseg, "width": W_, "height": H_, "format": "R8",
                   "l2": "flushed between steps (512 MiB write)"},
        "batched_graph_ms": round(ms_graph, 4), "batched_ms": round(ms_batched, 4),
        "per_glyph_ms": round(ms_per_glyph, 3), "per_glyph_wall_ms": round(wall_per_glyph, 3),
        "speedup_vs_per_glyph": round(ms_per_glyph / ms_graph, 2), "identical_output": identical,
        "frame": {"fills": st.fill_count, "tiles": st.tile_count, "alpha_tiles": st.alpha_tile_count,
                  "lines": st.line_count, "screen_tiles": st.screen_tile_count},
        "tuning": tuning, "gpu_launches_per_batched_frame": st.kernel_launches,
    }
    r.close()
    torch.cuda.set_stream(prev_stream)
    return line


def stroke_workload(seed: int, scale: float = 1.0):
    """The 4K scene's outlines as strokes: every draw path's contours, half of
    them open, seeded widths 0.5-8 px with every cap and join (miter limit 4).
    Returns (StrokeBatch, input segments)."""
    import numpy as np
    import pathfinder_gb300 as pf
    from pathfinder_gb300.stroke import LineCap, LineJoin, StrokeBatch, StrokeStyle
    scene = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=seed, scale=scale)
    rng = np.random.default_rng(seed + 11)
    items, nseg = [], 0
    starts, pts, fl = scene.contour_starts, scene.points, scene.flags
    for rec in scene.draw_paths:
        fc, n = int(rec["first_contour"]), int(rec["contour_count"])
        ol = pf.Outline()
        for c in range(fc, fc + n):
            a, b = int(starts[c]), int(starts[c + 1])
            ct = pf.Contour()
            ct.points = pts[a:b].tolist()
            ct.flags = fl[a:b].tolist()
            ct.closed = bool(rng.integers(0, 2))
            ends = int(np.count_nonzero((fl[a + 1:b] & 3) == 0))
            nseg += (ends + 1 if ct.closed else ends) if b > a else 0
            ol.contours.append(ct)
        items.append((ol, StrokeStyle(float(rng.uniform(0.5, 8.0)), LineCap(int(rng.integers(0, 3))),
                                      LineJoin(int(rng.integers(0, 3))), 4.0)))
    return StrokeBatch(items), nseg


def run_strokes(args) -> None:
    """Stroke to fill of the 4K scene's 20,000 outlines (2.1M segments) on the
    GPU, inputs and outputs resident in device memory; e2e through the C ABI
    with host buffers; CPU baseline: the oracle's single-threaded stroker."""
    import ctypes as C
    import numpy as np
    import torch
    from pathfinder_gb300 import build as pbuild
    pbuild.build()
    import pathfinder_gb300 as pf
    from pathfinder_gb300 import _abi
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    batch, nseg = stroke_workload(args.seed, args.scale)
    r = pf.Renderer(0)
    r.set_stream(stream.cuda_stream)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(batch, k))).cuda()
           for k in ("points", "flags", "contour_starts", "contour_closed", "outline_starts")}
    styles = torch.frombuffer(bytearray(bytes(batch.styles)), dtype=torch.uint8).cuda()
    d = _abi.PFCUDAStrokeInput()
    d.points, d.point_flags = dev["points"].data_ptr(), dev["flags"].data_ptr()
    d.contour_starts, d.contour_closed = dev["contour_starts"].data_ptr(), dev["contour_closed"].data_ptr()
    d.outline_starts, d.styles = dev["outline_starts"].data_ptr(), styles.data_ptr()
    d.point_count, d.contour_count, d.outline_count = len(batch.points), batch.contour_count, batch.outline_count
    d.memory = _abi.PF_MEMORY_DEVICE
    o = _abi.PFCUDAStrokeOutput()
    o.memory = _abi.PF_MEMORY_DEVICE
    L = r._lib
    rc = L.PFCUDAStrokeToFill(r._h, C.byref(d), C.byref(o))
    assert rc == _abi.PF_CUDA_ERR_CAPACITY, rc
    npts, ncont = int(o.point_count), int(o.contour_count)
    out_pts = torch.empty((npts, 2), dtype=torch.float32, device="cuda")
    out_fl = torch.empty((npts,), dtype=torch.uint8, device="cuda")
    out_cs = torch.empty((ncont + 1,), dtype=torch.int32, device="cuda")
    out_os = torch.empty((batch.outline_count + 1,), dtype=torch.int32, device="cuda")
    o.points, o.point_flags = out_pts.data_ptr(), out_fl.data_ptr()
    o.contour_starts, o.outline_starts = out_cs.data_ptr(), out_os.data_ptr()
    o.point_capacity, o.contour_capacity = npts, ncont
    for _ in range(args.warmup):
        assert L.PFCUDAStrokeToFill(r._h, C.byref(d), C.byref(o)) == 0
    sampler = ClockSampler(0)
    sampler.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in evs:
        a.record(stream)
        L.PFCUDAStrokeToFill(r._h, C.byref(d), C.byref(o))
        b.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    # e2e: host arrays in, host arrays out, through the Python API
    e2e = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        _stroke_host(r, batch, npts, ncont)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(e2e) / len(e2e)
    line = {
        "metric": "Mseg/s stroked", "value": round(nseg / (ms / 1e3) / 1e6, 3), "unit": "Mseg/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the seeded PF_SCENE_SVG_4K outlines, half open, widths 0.5-8 px, every cap and join)",
        "config": {"workload": "stroke_4k_20000_paths" if args.scale == 1.0 else f"stroke_4k_scale{args.scale}",
                   "outlines": batch.outline_count, "contours": batch.contour_count, "segments": nseg,
                   "input_points": len(batch.points), "output_points": npts, "output_contours": ncont},
        "e2e": {"value": round(nseg / (e2e_ms / 1e3) / 1e6, 3), "unit": "Mseg/s",
                "h2d_bytes_per_step": int(batch.points.nbytes + batch.flags.nbytes + batch.contour_starts.nbytes),
                "d2h_bytes_per_step": int(npts * 9 + (ncont + 1) * 4), "ms_per_step": round(e2e_ms, 3)},
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        oracle.stroke(batch.desc())
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(nseg / cpu_s / 1e6, 4), "unit": "Mseg/s", "cores": 1, "kind": "port",
                                "sample": f"the whole workload once on one host thread ({cpu_s:.2f} s)"}
    print(json.dumps(line), flush=True)
    r.close()


def _stroke_host(r, batch, npts, ncont):
    """PFCUDAStrokeToFill with host input and output buffers (the e2e leg)."""
    import ctypes as C
    import numpy as np
    from pathfinder_gb300 import _abi
    pts = np.empty((npts, 2), np.float32)
    fl = np.empty((npts,), np.uint8)
    cs = np.empty((ncont + 1,), np.uint32)
    os_ = np.empty((batch.outline_count + 1,), np.uint32)
    o = _abi.PFCUDAStrokeOutput()
    o.points, o.point_flags, o.contour_starts, o.outline_starts = (pts.ctypes.data, fl.ctypes.data, cs.ctypes.data,
                                                                   os_.ctypes.data)
    o.point_capacity, o.contour_capacity, o.memory = npts, ncont, _abi.PF_MEMORY_HOST
    d = batch.desc()
    _abi.check(r._lib.PFCUDAStrokeToFill(r._h, C.byref(d), C.byref(o)), "PFCUDAStrokeToFill")
    return pts, fl, cs, os_


def _diff_common():
    import torch
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn, reps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        t = sorted(a.elapsed_time(b) for a, b in evs)
        return sum(t) / reps

    return torch, stream, timed


def run_diff(args) -> None:
    import torch
    from pathfinder_gb300 import build as pbuild
    pbuild.build()
    torch.cuda.set_device(0)
    line = diff_measure(args.seed, args.steps, args.warmup)
    print(json.dumps(line), flush=True)


def diff_measure(seed: int, steps: int, warmup: int) -> dict:
    """256 closed cubic paths (4,096 control points), 1024^2 single-channel
    FP32 coverage, L2 loss against the render of the points + N(0, 2 px):
    forward + adjoint (dL/dpoints, dL/dalpha) per step against the plain
    (non-differentiable) FP32 coverage frame of the same scene."""
    import torch
    prev_stream = torch.cuda.current_stream()
    _, stream, timed = _diff_common()
    import pathfinder_gb300 as pf
    from pathfinder_gb300.diff import DiffRenderer
    scene = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=seed)
    tscene = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=seed, jitter_sigma=2.0, jitter_seed=seed + 1)
    Wd, Hd = scene.width, scene.height
    tdr = DiffRenderer(tscene)
    target = tdr.forward(tdr.points0, tdr.alpha0).clone()
    dr = DiffRenderer(scene, sync=False)
    dr.renderer.set_stream(stream.cuda_stream)
    pts, alpha = dr.points0.clone(), dr.alpha0.clone()
    plain = pf.Renderer(0)
    plain.set_stream(stream.cuda_stream)
    pbatch = pf.SceneBatch.packed([scene])
    pout = torch.zeros((Hd, Wd), dtype=torch.float32, device="cuda")
    plain.render_batch(pbatch, pout, pf.PF_CUDA_FORMAT_F32)
    grads = {}

    def fwd():
        img = dr.forward(pts, alpha)
        grads["img"] = img

    def fwd_bwd():
        img = dr.forward(pts, alpha)
        gp, ga = dr.backward(2.0 * (img - target))
        grads["gp"], grads["ga"] = gp, ga

    for _ in range(warmup):
        fwd_bwd()
        plain.render_batch(pbatch, pout, pf.PF_CUDA_FORMAT_F32, sync=False)
    ms_plain = timed(lambda: plain.render_batch(pbatch, pout, pf.PF_CUDA_FORMAT_F32, sync=False), steps)
    ms_fwd = timed(fwd, steps)
    ms_fb = timed(fwd_bwd, steps)
    code, _ = dr.renderer.render_status()
    assert code == 0, code
    st = dr.renderer.stats()
    loss = float(((grads["img"] - target) ** 2).sum()) if "img" in grads else None
    line = {
        "metric": "fwd_bwd_ms", "value": round(ms_fb, 4), "unit": "ms", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": round(ms_fb, 4), "higher_is_better": False, "dtype": "f32",
        "data": "synthetic (seeded PF_SCENE_CUBIC_1K: 256 closed cubic paths; target = points + N(0, 2 px))",
        "config": {"workload": "diff_cubic_256_paths_1024", "paths": len(scene.draw_paths),
                   "control_points": len(scene.points), "width": Wd, "height": Hd, "seed": seed,
                   "l2": "flushed between steps (512 MiB write)"},
        "plain_forward_ms": round(ms_plain, 4), "diff_forward_ms": round(ms_fwd, 4),
        "fwd_bwd_over_plain_forward": round(ms_fb / ms_plain, 3),
        "frame": {"lines": st.line_count, "fills": st.fill_count, "alpha_tiles": st.alpha_tile_count,
                  "visible_tiles": st.visible_tile_count},
        "loss": loss, "grad_points_abs_max": float(grads["gp"].abs().max()),
        "grad_alpha_abs_max": float(grads["ga"].abs().max()),
    }
    dr.renderer.close()
    tdr.renderer.close()
    plain.close()
    torch.cuda.set_stream(prev_stream)
    return line


def run_fit(args) -> None:
    """64 independent scenes of uneven size (32-512 cubic paths, canvases
    256^2-1024^2, drawn from the seed) fitted jointly toward perturbed targets
    (points + N(0, 2 px)) with Adam (lr 0.5 px) on the control points: one
    batched differentiable frame and one batched adjoint per step."""
    import torch
    from pathfinder_gb300 import build as pbuild
    pbuild.build()
    torch.cuda.set_device(0)
    _, stream, timed = _diff_common()
    import numpy as np
    import pathfinder_gb300 as pf
    from pathfinder_gb300.diff import DiffRenderer
    rng = np.random.default_rng(args.seed)
    n_scenes = 64
    scenes, targets = [], []
    for i in range(n_scenes):
        n_paths = int(rng.integers(32, 513))
        side = int(rng.integers(256, 1025))
        sd = args.seed * 1000 + i
        scenes.append(pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=sd, scale=n_paths / 256, width=side, height=side))
        targets.append(pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=sd, scale=n_paths / 256, width=side, height=side,
                                         jitter_sigma=2.0, jitter_seed=sd + 7))
    batch, tbatch = pf.SceneBatch.packed(scenes), pf.SceneBatch.packed(targets)
    tdr = DiffRenderer(tbatch)
    target = tdr.forward(tdr.points0, tdr.alpha0).clone()
    goal = tdr.points0.clone()
    dr = DiffRenderer(batch, sync=False)
    dr.renderer.set_stream(stream.cuda_stream)
    plain = pf.Renderer(0)
    plain.set_stream(stream.cuda_stream)
    pout = torch.zeros((batch.total_pixels,), dtype=torch.float32, device="cuda")
    plain.render_batch(batch, pout, pf.PF_CUDA_FORMAT_F32)
    for _ in range(args.warmup):
        plain.render_batch(batch, pout, pf.PF_CUDA_FORMAT_F32, sync=False)
    ms_plain = timed(lambda: plain.render_batch(batch, pout, pf.PF_CUDA_FORMAT_F32, sync=False), 20)

    pts = dr.points0.clone().requires_grad_(True)
    opt = torch.optim.Adam([pts], lr=0.5)
    losses = []
    dist0 = float((dr.points0 - goal).norm(dim=1).mean())

    def step():
        opt.zero_grad(set_to_none=False)
        loss = ((dr(pts) - target) ** 2).sum()
        loss.backward()
        opt.step()
        losses.append(loss.detach())

    # the first step sizes the device buffers (synchronous frame, regrow);
    # the timed steps are the rest
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step()
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    n_timed = max(1, args.fit_steps - 1)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_timed)]
    t0 = time.perf_counter()
    for a, b in evs:
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    code, _ = dr.renderer.render_status()
    assert code == 0, code
    ms = [a.elapsed_time(b) for a, b in evs]
    ms_step = sum(ms) / len(ms)
    dist1 = float((pts.detach() - goal).norm(dim=1).mean())
    # the renderer's share of a step: differentiable frame + adjoint only
    grad_img = torch.ones_like(target)

    def fwd_bwd():
        dr.forward(pts.detach(), dr.alpha0)
        dr.backward(grad_img)

    ms_fb = timed(fwd_bwd, 20)
    code, _ = dr.renderer.render_status()
    assert code == 0, code
    line = {
        "metric": "fit_ms_per_step", "value": round(ms_step, 4), "unit": "ms", "n_gpus": 1,
        "steps": n_timed, "warmup": 1, "ms_per_step": round(ms_step, 4), "higher_is_better": False,
        "dtype": "f32", "data": "synthetic (seeded PF_SCENE_CUBIC_1K scenes of uneven size; targets = points + N(0, 2 px))",
        "config": {"workload": "fit_64_scenes_adam", "scenes": n_scenes, "paths": sum(len(s.draw_paths) for s in scenes),
                   "control_points": int(dr.n_points), "pixels": int(batch.total_pixels), "lr_px": 0.5,
                   "seed": args.seed},
        "plain_forward_ms": round(ms_plain, 4), "fwd_bwd_adam_over_plain_forward": round(ms_step / ms_plain, 3),
        "fwd_bwd_ms": round(ms_fb, 4), "fwd_bwd_over_plain_forward": round(ms_fb / ms_plain, 3),
        "first_step_s": round(first_s, 3), "wall_s_timed_steps": round(wall, 3),
        "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
        "mean_point_distance_px": {"start": round(dist0, 4), "end": round(dist1, 4)},
    }
    print(json.dumps(line), flush=True)


def side_workloads(args) -> dict:
    """The path's other targets, measured in the same run: the batched
    16,384-glyph atlas against per-glyph frames (speed-up and identical
    output) and the differentiable frame's forward + adjoint against the
    plain forward."""
    a = atlas_measure(args.seed, 1.0, 20, 3)
    d = diff_measure(args.seed, 20, 3)
    return {
        "glyph_atlas_16384": {k: a[k] for k in ("batched_graph_ms", "batched_ms", "per_glyph_ms",
                                                "speedup_vs_per_glyph", "identical_output")}
                             | {"glyphs": a["config"]["glyphs"], "segments": a["config"]["segments"],
                                "format": "R8 4096x4096", "target": "speed-up >= 5x, identical output"},
        "diff_cubic_256_paths_1024": {k: d[k] for k in ("value", "plain_forward_ms", "diff_forward_ms",
                                                        "fwd_bwd_over_plain_forward")}
                                     | {"unit": "ms (fwd+bwd)", "target": "fwd+bwd <= 3x plain forward"},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="svg4k", choices=["svg4k", "atlas", "diff", "fit", "strokes"],
                    help="svg4k: the 20,000-path 4K frame (default); atlas: the batched glyph atlas; "
                         "diff: forward + adjoint of 256 cubic paths at 1024^2; fit: 64-scene Adam fit; "
                         "strokes: stroke to fill of the 4K scene's outlines")
    ap.add_argument("--fit-steps", type=int, default=200)
    ap.add_argument("--d3d11", action="store_true",
                    help="tile with the D3D11 level's semantics (uniform dicing) instead of the CPU tiler's")
    ap.add_argument("--paints", action="store_true",
                    help="add seeded gradients and blend modes to the 4K scene's paths")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cuda", choices=["cuda", "reference"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-side", action="store_true", help="skip the atlas and differentiable side workloads")
    ap.add_argument("--clock-soak", type=float, default=1.5,
                    help="seconds of untimed replays sampled for clocks before the timed steps")
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--e2e-depth", type=int, default=6, help="frames in flight in the end-to-end leg")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the 20,000 paths (small cases for profiling only)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "atlas":
        run_atlas(args)
        return
    if args.workload == "diff":
        run_diff(args)
        return
    if args.workload == "fit":
        run_fit(args)
        return
    if args.workload == "strokes":
        run_strokes(args)
        return

    import numpy as np
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from pathfinder_gb300 import build as pbuild
    pbuild.build()
    import pathfinder_gb300 as pf

    # replicas only: each rank renders its own scene (seed + rank)
    scene = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=args.seed + rank, scale=args.scale)
    paints = add_paints(scene, args.seed + rank) if args.paints else None
    nseg = scene.segment_count
    npts = len(scene.points)
    r = pf.Renderer(local, pf.RendererOptions(d3d11_semantics=args.d3d11))
    # a dedicated stream: the renderer, the L2 flush and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r.set_stream(stream.cuda_stream)
    out = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
    r.render(scene, out=out)  # first frame: sizes the buffers
    st = r.stats()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        flush.zero_()
        r.render_async(scene, out)
    code, _ = r.render_status()
    if code != 0:
        raise RuntimeError(f"render failed with status {code}")

    # Timed region: the frame replayed from its CUDA graph (every kernel of the
    # frame runs on every step; the graph removes the launch gaps only).
    r.graph_capture(None, out, pf.PF_CUDA_FORMAT_RGBA8)
    for _ in range(args.warmup):
        flush.zero_()
        r.graph_launch()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    # The sampler reads every 100 ms, longer than the timed steps take: it runs
    # over ~1.5 s of untimed replays of the same frame that lead straight into
    # the timed steps, so the clocks are those of the GPU under this load.
    soak_end, soak = time.perf_counter() + args.clock_soak, 0
    while time.perf_counter() < soak_end:
        flush.zero_()
        r.graph_launch()
        soak += 1
        if soak % 32 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()  # inputs are below L2 size: flush between steps
        evs[k][0].record(stream)
        r.graph_launch()
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    r.graph_release()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps

    # Stage breakdown: a second timed region of enqueued frames with CUDA
    # events between the stages (the roofline of the dominant kernel).
    r.set_profiling(True)
    stage_sum = {}
    evs2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        evs2[k][0].record(stream)
        r.render_async(scene, out)
        evs2[k][1].record(stream)
        for n, v in r.stage_times().items():
            stage_sum[n] = stage_sum.get(n, 0.0) + v
    torch.cuda.synchronize()
    code, _ = r.render_status()
    if code != 0:
        raise RuntimeError(f"render failed with status {code}")
    st = r.stats()
    ms_enqueued = sum(a.elapsed_time(b) for a, b in evs2) / args.steps
    job_seg, (ms,) = job_totals(dist, nseg, [ms])
    value = job_seg / (ms / 1e3) / 1e6

    # roofline of the dominant stage
    stage_ms = {n: v / args.steps for n, v in stage_sum.items()}
    sb = stage_bytes(st, npts, nseg)
    # single-kernel stages (the D3D11 level's flattening is its dicing: three launches)
    stage_kernels = {k: v for k, v in STAGE_KERNELS.items() if not (args.d3d11 and k == "flatten")}
    dom = max((n for n in stage_ms if n in stage_kernels), key=stage_ms.get)
    peak, peak_kind = _peaks()
    achieved = sb[dom] / (stage_ms[dom] / 1e3) / 1e9
    frame_gbs = sb["frame"] / (ms / 1e3) / 1e9
    # the committed capture is of the plain full-size frame only
    variant = "paints" if args.paints else ("d3d11" if args.d3d11 else "plain")
    traffic, traffic_src = measured_traffic(dom, args.scale == 1.0 and not (args.paints and args.d3d11), variant)

    # e2e through the public API with host buffers
    # about 0.4 s of pipelined steps at the default: runs of 200 steps spread
    # by up to 20% with host-side jitter, runs of 1000 by about 1%
    e2e_steps = args.e2e_steps or max(3, min(10 * args.steps, 1000))
    depth = max(1, args.e2e_depth)
    pinned = {}
    for name in ("points", "flags", "contour_starts", "clip_paths", "draw_paths"):
        a = getattr(scene, name)
        t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).pin_memory()  # path records as bytes
        pinned[name] = t
        setattr(scene, name, t.numpy().view(a.dtype).reshape(a.shape))
    host_out = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory()
    host_np = host_out.numpy()
    h2d = sum(getattr(scene, n).nbytes for n in ("points", "flags", "contour_starts", "clip_paths", "draw_paths"))
    d2h = host_np.nbytes
    r.set_profiling(False)
    for _ in range(2):
        r.upload_scene(scene, force=True)
        r.render(scene, out=host_np)
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        r.upload_scene(scene, force=True)
        r.render(scene, out=host_np)
        e2e_times.append(time.perf_counter() - t0)
    serial_ms = 1e3 * sum(e2e_times) / len(e2e_times)
    # The same steps with `depth` frames in flight (RenderPipeline: one
    # renderer, stream and host thread per frame in flight), so one frame's
    # upload and image copy overlap another's kernels.  Step i is submitted
    # once step i - depth is done, into that step's host buffer; every step
    # uploads its scene and copies its image to host memory.
    pipe = pf.RenderPipeline(local, depth=depth, options=pf.RendererOptions(d3d11_semantics=args.d3d11))
    pouts = [torch.empty((H, W, 4), dtype=torch.uint8).pin_memory().numpy() for _ in range(depth)]
    for f in [pipe.submit(scene, pouts[i % depth]) for i in range(3 * depth)]:
        f.result()
    for o in pouts:
        if not np.array_equal(o, host_np):
            raise RuntimeError("pipelined frame differs from the serial frame")
    futs = []
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        if i >= depth:
            futs[i - depth].result()
        futs.append(pipe.submit(scene, pouts[i % depth]))
    for f in futs[-depth:]:
        f.result()
    e2e_ms = 1e3 * (time.perf_counter() - t0) / e2e_steps
    pipe.close()
    _, (e2e_ms, serial_ms) = job_totals(dist, nseg, [e2e_ms, serial_ms])
    e2e_value = job_seg / (e2e_ms / 1e3) / 1e6

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded PF_SCENE_SVG_4K: 20,000 log-normal star paths, 40/30/30 line/quad/cubic)",
            "config": svg_config(scene, args, paints, world),
            "mpx_per_s": round(world * W * H / (ms / 1e3) / 1e6, 3),
            "timing": "CUDA graph replay of the whole frame; ms_per_step_enqueued: the same frame enqueued "
                      "kernel by kernel with stage events",
            "ms_per_step_enqueued": round(ms_enqueued, 4),
            "frame": {"fills": st.fill_count, "tiles": st.tile_count, "alpha_tiles": st.alpha_tile_count,
                      "visible_tiles": st.visible_tile_count, "lines": st.line_count,
                      "algorithmic_bytes": sb["frame"], "achieved_gbs": round(frame_gbs, 1),
                      "frac_of_" + peak_kind: round(frame_gbs / peak, 4)},
            "stages_ms": {n: round(v, 4) for n, v in stage_ms.items()},
            "roofline": {"bound": "hbm", "kernel": stage_kernels[dom], "stage": dom, "achieved": round(achieved, 1),
                         "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": sb[dom], "traffic": traffic,
                         "traffic_source": traffic_src},
            "e2e": {"value": round(e2e_value, 4), "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3), "steps": e2e_steps,
                    "frames_in_flight": depth,
                    "mode": f"RenderPipeline (PFCUDAPipeline), {depth} renderers on their own streams and "
                            "worker threads; every "
                            "step uploads the scene from pinned host memory and copies its RGBA8 image to "
                            "pinned host memory (one device-to-host copy after the composite)",
                    "serial_ms_per_step": round(serial_ms, 3),
                    "serial_value": round(job_seg / (serial_ms / 1e3) / 1e6, 4)},
            "gpu_launches": int(st.kernel_launches * args.steps),
            "clocks": {**clocks, "window": f"{soak} untimed replays (~{args.clock_soak:.1f} s) then the timed steps"},
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(scene, nseg)
    r.close()
    if rank == 0:
        if world == 1 and not args.no_side and args.scale == 1.0 and not args.paints and not args.d3d11:
            line["side_workloads"] = side_workloads(args)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
