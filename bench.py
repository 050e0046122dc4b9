"""Benchmark of the lucid_gb300 raster pipeline (one JSON line on rank 0).

Workload: 1920x1080, 1M random triangles with heavy overdraw (Gaussian centres, sigma 0.2*W;
log-normal area, median 60 px^2, sigma 2; 5% of triangles log-uniform in [10k, 50k] px^2;
RGBA8, alpha U[0.1, 0.9]), exact per-pixel order, FP32 RGBA output. A step is one full frame
(quad setup, bin count, categorize, dispatch, raster).

value      fragments/s with the scene resident in device memory (CUDA events around each step
           on the launching stream; L2 flushed by a 256 MB write between steps).
e2e        same metric through lucid_render with host buffers: every step copies the scene from
           pinned host memory and reads the FP32 image back, as a serving loop (uploads and
           read-backs on copy streams overlap the neighbouring frames' renders).
roofline   raster kernel (the dominant kernel): algorithmic bytes per launch / its measured time.
cpu_baseline  the CPU oracle (port of the reference passes): one whole frame of the workload on
           all host threads (measured), and the 1280x720 / 100k-triangle frame on 1 core and on
           all cores.
parity     (not timed) the benchmark frame against the oracle on 16 seeded bins: fragment order
           bit-exact, image error, and the FP32 image's error against the FP64 blend.
workloads  the 3840x2160 / 5M-triangle mesh frame and the 1280x720 / 100k-triangle frame: frame
           time, fragments/s and the time of each pass.

--impl reference runs the CPU oracle only (the reference itself runs only as Vulkan GLSL).
Multi-GPU (torchrun): independent replicas, one frame per rank per step ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "heavy1080"
WORKLOAD_DESC = ("1920x1080, 1M random triangles: Gaussian centres (sigma 0.2*W), log-normal area "
                 "(median 60 px^2, sigma 2) with 5% log-uniform in [10k,50k] px^2, view depth "
                 "U[0.1,100], RGBA8 vertex colours, alpha U[0.1,0.9]; exact per-pixel order, FP32 RGBA")
METRIC = "fragments_blended_per_s_1080p_1M_tris"
UNIT = "fragments/s"
KERNELS_PER_FRAME = 8  # setupPrep, setupClassify, setupScan, setupStore, binCount, binCategorize, binDispatch, raster


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lucid_gb300", choices=["lucid_gb300", "reference"])
    ap.add_argument("--cpu-sample-bins", type=int, default=0, help="bins in the CPU sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the forward+backward and batched-view measurements (profiling runs)")
    ap.add_argument("--workload", default=WORKLOAD,
                    help="scenes.workload name (the default is the benchmark workload; smaller "
                         "ones exist for profiler captures)")
    ap.add_argument("--frames-only", type=int, default=0,
                    help="profiler captures: render this many frames of --workload (or, with "
                         "--workload batch64, of the 64-view batch) through the public API and "
                         "exit, with no timing")
    return ap.parse_args()


def workload_name(name):
    return name + ": " + WORKLOAD_DESC if name == WORKLOAD else name


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_fragment():
    """DRAM bytes per fragment of the raster kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "raster_heavy1080.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_fragment:"):
                return float(line.split(":", 1)[1].split()[0])
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="lucid_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_frame(scene, threads):
    """One whole frame of the CPU oracle (setup, binning, raster of every bin, FP32 blend that
    stops at T == 0): wall time in seconds and the frame's fragments."""
    from oracle import binding
    mvq = max(1024, scene.num_quads)
    t0 = time.perf_counter()
    o = binding.run(scene, max_visible_quads=mvq, raster=True, threads=threads, setup_outputs=False)
    return time.perf_counter() - t0, int(o["num_fragments"])


def cpu_sample(scene, sample_bins, threads, seed=0):
    """The CPU oracle on a seeded sample of bins (setup and binning of the whole frame, raster of
    `sample_bins` random bins); the raster time is extrapolated to the frame by fragments."""
    from oracle import binding
    mvq = max(1024, scene.num_quads)
    t0 = time.perf_counter()
    full = binding.run(scene, max_visible_quads=mvq, raster=False, setup_outputs=False)
    t_bin = time.perf_counter() - t0
    n = full["bin_count"]
    rng = np.random.default_rng(seed)
    k = min(n, sample_bins)
    subset = np.sort(rng.choice(n, size=k, replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    part = binding.run(scene, max_visible_quads=mvq, raster=True, bin_subset=subset, threads=threads,
                       setup_outputs=False)
    t_raster = max(time.perf_counter() - t0 - t_bin, 1e-9)  # the sampled run repeats setup + binning
    return dict(t_bin=t_bin, t_raster_sample=t_raster, frag_sample=int(part["num_fragments"]), bins=k,
                bin_count=n)


def host_cores():
    return os.cpu_count() or 1


def cpu_baselines(scene, fragments):
    """Rank 0 at N=1: the oracle's whole benchmark frame on all host cores (measured, not
    extrapolated) and the 1280x720 / 100k-triangle frame on 1 core and on all cores."""
    from lucid_gb300 import scenes
    cores = host_cores()
    t_frame, frags = cpu_frame(scene, cores)
    assert frags == fragments, (frags, fragments)
    c0 = scenes.workload("cpu720")
    t1, f0 = cpu_frame(c0, 1)
    tn, _ = cpu_frame(c0, cores)
    return {"value": frags / t_frame, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"one whole frame of the workload by the oracle (setup, binning, every bin's raster; "
                       f"FP32 blend stopping at T == 0) on {cores} host threads"),
            "ms_per_frame": t_frame * 1e3,
            "cpu720": {"workload": "1280x720, 100k random triangles", "fragments": f0,
                       "ms_per_frame_1_core": t1 * 1e3, "ms_per_frame_all_cores": tn * 1e3, "cores": cores}}


def parity_sample(r, frame, scene, num_bins=16, max_per_pixel=64, seed=0):
    """Checks the benchmark frame against the oracle on a seeded sample of bins (not timed):
    per-pixel fragment counts and first fragments in blend order bit-exact, image within 1e-5,
    and the FP32 image's error against the oracle's FP64 blend."""
    from oracle import binding
    mvq = max(1024, scene.num_quads)
    rng = np.random.default_rng(seed)
    bins = np.sort(rng.choice(r.num_bins, size=min(num_bins, r.num_bins), replace=False)).astype(np.int32)
    img, counts, prims = r.raster_dump_bins(frame, bins, max_per_pixel)
    o = binding.run(scene, max_visible_quads=mvq, bin_subset=bins, threads=host_cores(), image64=True,
                    max_per_pixel=max_per_pixel, dump_by_subset=True, setup_outputs=False)
    g = img.cpu().numpy()
    bcx = r.bin_count_x
    e32 = e64 = 0.0
    for b in bins:
        by, bx = divmod(int(b), bcx)
        ys = slice(by * 32, min(by * 32 + 32, scene.height))
        xs = slice(bx * 32, min(bx * 32 + 32, scene.width))
        e32 = max(e32, float(np.abs(g[ys, xs] - o["image"][ys, xs]).max()))
        e64 = max(e64, float(np.abs(g[ys, xs].astype(np.float64) - o["image64"][ys, xs]).max()))
    order_ok = bool(np.array_equal(counts, o["frag_counts"]) and np.array_equal(prims, o["frag_prims"]))
    return {"bins": int(len(bins)), "fragments": int(counts.sum()), "order_bit_exact": order_ok,
            "max_abs_err_vs_oracle": e32, "max_abs_err_vs_fp64_blend": e64,
            "first_fragments_compared_per_pixel": max_per_pixel}


def workload_config(name, scene, info=None):
    cfg = {"workload": workload_name(name), "width": scene.width, "height": scene.height,
           "triangles": scene.num_tris}
    if info is not None:
        w, h = scene.width, scene.height
        cfg.update({"fragments_per_frame": int(info.num_fragments),
                    "blended_fragments_per_frame": int(info.raster_blended_fragments),
                    "max_fragments_per_pixel": int(info.max_pixel_fragments),
                    "mean_layers_per_pixel": int(info.num_fragments) / (w * h),
                    "visible_quads": list(info.num_visible_quads),
                    "bin_levels": {"low": info.bin_level_counts[2], "high": info.bin_level_counts[4]},
                    "light_bins": int(info.raster_light_bins)})
    return cfg


def run_reference(args, rank):
    """--impl reference: the CPU oracle (port of the reference passes) on all host cores, on a
    bounded sample of the workload per step."""
    if rank != 0:
        return
    from lucid_gb300 import scenes
    scene = scenes.workload(args.workload)
    bins = args.cpu_sample_bins or 48
    cores = host_cores()
    vals = []
    times = []
    last = None
    for i in range(args.warmup + args.steps):
        r = cpu_sample(scene, bins, cores, seed=i)
        # extrapolated whole-frame rate: total fragments / (binning + raster of all bins)
        rate = r["frag_sample"] / r["t_raster_sample"]
        frame_frags = r["frag_sample"] * r["bin_count"] / r["bins"]
        frame_time = r["t_bin"] + frame_frags / rate
        if i >= args.warmup:
            vals.append(frame_frags / frame_time)
            times.append(frame_time)
        last = r
    value = float(np.mean(vals))
    ms_per_step = float(np.mean(times)) * 1e3
    sample = (f"setup+binning of the full scene, raster of {last['bins']} seeded random bins "
              f"of {last['bin_count']} per step; frame time extrapolated by fragments")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.workload, scene), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def grad_bench(steps, warmup, flush_buf):
    """Forward+backward on grad512 (512x512, 200k triangles, FP32 vertex RGBA, per-triangle
    opacity): L2 loss to a target rendered from perturbed colours, gradients with respect to
    vertex RGBA and triangle opacity. Times the plain forward (lucid_render), the differentiable
    forward (lucid_render_forward_grad), and forward_grad + loss gradient + lucid_render_backward."""
    import torch
    from lucid_gb300 import scenes
    from lucid_gb300._lib import check
    from lucid_gb300.renderer import FrameInputs, LucidRenderer, _dptr, _stream_ptr
    import ctypes
    sc = scenes.workload("grad512")
    r = LucidRenderer(sc.width, sc.height, max_input_quads=sc.num_quads, max_visible_quads=sc.num_quads,
                      max_bin_refs=8 * sc.num_quads)
    frame = FrameInputs.from_scene(sc)
    rng = np.random.default_rng(104)
    pert = sc.colors.copy()
    pert[:, :3] = np.clip(pert[:, :3] + rng.normal(0, 0.1, size=pert[:, :3].shape), 0, 1)
    tframe = FrameInputs.from_scene(scenes.Scene(**{**sc.__dict__, "colors": pert.astype(np.float32)}))
    target = r.render(tframe)
    img = r.new_image()
    dvc = torch.zeros_like(frame.colors)
    dop = torch.zeros_like(frame.tri_opacity)
    stream = torch.cuda.current_stream()
    fi = frame.c_struct()

    def fwd_plain():
        r.render(frame, img)

    def fwd_grad():
        check(r.lib.lucid_render_forward_grad(r.handle, ctypes.byref(fi), _dptr(img), _stream_ptr()),
              "lucid_render_forward_grad")

    def fwd_bwd():
        fwd_grad()
        g = 2.0 * (img - target)
        g[..., 3] = 0.0
        check(r.lib.lucid_render_backward(r.handle, ctypes.byref(fi), _dptr(g), _dptr(dvc), _dptr(dop),
                                          _stream_ptr()), "lucid_render_backward")

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for i in range(steps):
            flush_buf.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    t_plain, t_fgrad, t_fb = timed(fwd_plain), timed(fwd_grad), timed(fwd_bwd)
    info, _ = r.info()
    r.close()
    return {"workload": "grad512: 512x512, 200k random triangles (cpu720 distributions), FP32 vertex "
                        "RGBA, triangle opacity U[0.1,0.9], L2 loss to a perturbed-colour target",
            "fwd_ms": t_plain, "fwd_grad_ms": t_fgrad, "fwd_bwd_ms": t_fb, "ratio": t_fb / t_plain,
            "fragments": int(info.num_fragments), "median_of": steps}


def batch_bench(steps, warmup, flush_buf, num_views=64):
    """Batched multi-view frames: num_views random-triangle views (cpu720 distributions) with
    resolutions drawn from {256^2, 512^2, 1280x720, 1920x1080} and log-uniform [10k, 500k]
    triangles, rendered by one lucid_render_batch (replay of its recorded graph) against
    num_views sequential lucid_render calls (one renderer per resolution) on the same GPU."""
    import torch
    from lucid_gb300 import scenes
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    views = scenes.batch_views(num_views)
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    outs = [torch.empty((v.height, v.width, 4), dtype=torch.float32, device="cuda") for v in views]
    total_quads = sum(max(1, v.num_quads) for v in views)
    plain = {}
    for v in views:
        key = (v.width, v.height)
        if key not in plain:
            nq = max(x.num_quads for x in views if (x.width, x.height) == key)
            plain[key] = LucidRenderer(v.width, v.height, max_input_quads=nq, max_visible_quads=nq,
                                       max_bin_refs=8 * nq)
    br = LucidRenderer(max(v.width for v in views), max(v.height for v in views), max_input_quads=total_quads,
                       max_visible_quads=total_quads, max_bin_refs=4 * total_quads, max_views=num_views)
    # the batch's options (bin size, per-bin raster path, LOW/HIGH threshold, binning CTAs) tuned
    # on the batch itself by lucid_autotune_batch (the plain arm keeps the defaults)
    tuned = br.autotune_batch(frames, outs=outs)
    stream = torch.cuda.current_stream()

    def run_plain():
        for (f, w, h), o in zip(frames, outs):
            plain[(w, h)].render(f, o)

    def run_batch():
        br.render_batch(frames, outs=outs)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for i in range(steps):
            flush_buf.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    t_plain = timed(run_plain)
    t_batch = timed(run_batch)
    frags = sum(int(br.batch_info(i).num_fragments) for i in range(num_views))
    errors = [i for i in range(num_views) if br.batch_info(i).error_code != 0]
    for r in list(plain.values()) + [br]:
        r.close()
    return {"workload": f"{num_views} views, resolutions from {{256^2, 512^2, 1280x720, 1920x1080}}, "
                        "log-uniform [10k, 500k] random triangles each (cpu720 distributions)",
            "views": num_views, "triangles": int(sum(v.num_tris for v in views)), "fragments": frags,
            "plain_ms": t_plain, "batch_ms": t_batch, "plain_frames_per_s": num_views / (t_plain / 1e3),
            "batch_frames_per_s": num_views / (t_batch / 1e3), "speedup": t_plain / t_batch,
            "view_errors": errors, "median_of": steps, "tuning": tuned}


def quadgen_bench(steps, warmup):
    """Quad generation (lucid_quad_generate) on a 500k-triangle jittered grid mesh in random
    triangle order, against the oracle's restatement of the reference's sequential greedy
    (src/quad_generator.cpp) on one host core."""
    import time
    import torch
    from lucid_gb300 import scenes
    from lucid_gb300.renderer import quad_generate
    from oracle import binding as oracle
    pos, tris = scenes.tri_mesh("plane", 500, 500, seed=21)
    pos_d, tris_d = torch.from_numpy(pos).cuda(), torch.from_numpy(tris).cuda()
    for _ in range(warmup):
        quad_generate(pos_d, tris_d)
    ms = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q, nd = quad_generate(pos_d, tris_d)
        torch.cuda.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
    t0 = time.perf_counter()
    ref, ref_nd = oracle.quadgen(pos, tris, 1.0, 0)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    return {"workload": "500x500 grid, 500k triangles in random order, square_weight 1.0",
            "triangles": int(tris.shape[0]), "gpu_ms": float(np.median(ms)), "quads": int(q.shape[0]),
            "degenerate": int(nd), "cpu_reference_greedy_ms": cpu_ms, "cpu_quads": int(ref.shape[0]),
            "cpu_degenerate": int(ref_nd), "cpu_cores": 1, "median_of": steps}


def workload_bench(name, steps, warmup, flush_buf):
    """One named workload on its own renderer: median frame time (CUDA events, L2 flushed between
    frames), Mtri/s, fragments/s, realised depth complexity and the median time of each pass
    (pass-level entry points, one event pair per pass)."""
    import torch
    from lucid_gb300 import scenes
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.workload(name)
    r = LucidRenderer(sc.width, sc.height, max_input_quads=sc.num_quads, max_visible_quads=sc.num_quads,
                      max_bin_refs=8 * sc.num_quads)
    frame = FrameInputs.from_scene(sc)
    out = r.new_image()
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        r.render(frame, out)
    torch.cuda.synchronize()
    passes = [("setup", lambda: r.quad_setup(frame)), ("bin_count", r.bin_count),
              ("bin_categorize", r.bin_categorize), ("bin_dispatch", r.bin_dispatch),
              ("raster", lambda: r.raster(frame, out))]
    frame_ms, pass_ms = [], {n: [] for n, _ in passes}
    for i in range(steps):
        flush_buf.fill_(i & 0xFF)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(passes) + 1)]
        ev[0].record(stream)
        for k, (_, fn) in enumerate(passes):
            fn()
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
        for k, (n, _) in enumerate(passes):
            pass_ms[n].append(ev[k].elapsed_time(ev[k + 1]))
        frame_ms.append(ev[0].elapsed_time(ev[-1]))
    info, _ = r.info()
    if info.error_code != 0:
        raise RuntimeError(f"{name}: device error {info.error_code}")
    t = float(np.median(frame_ms))
    med = {n: float(np.median(v)) for n, v in pass_ms.items()}
    frags = int(info.num_fragments)
    res = {"config": workload_config(name, sc, info), "ms_per_frame": t,
           "mtri_per_s": sc.num_tris / (t / 1e3) / 1e6, "fragments_per_s": frags / (t / 1e3),
           "blended_fragments_per_s": int(info.raster_blended_fragments) / (t / 1e3),
           "pass_ms": med, "pass_share": {n: v / sum(med.values()) for n, v in med.items()},
           "median_of": steps}
    r.close()
    return res


def profile_figures():
    """Issue-slot figures of the raster kernel from the committed ncu summary (one launch)."""
    path = os.path.join(ROOT, "profiles", "raster_heavy1080.md")
    res = {}
    if os.path.exists(path):
        with open(path) as f:
            for line in f:
                for key in ("issue_active_frac", "warp_instructions_per_fragment"):
                    if line.startswith(key + ":"):
                        res[key] = float(line.split(":", 1)[1].split()[0])
    return res


def frames_only(args):
    """Renders args.frames_only frames and returns (for ncu captures of a known launch list)."""
    import torch
    from lucid_gb300 import build as lucid_build
    lucid_build.build()
    from lucid_gb300 import scenes
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    if args.workload == "batch64":
        views = scenes.batch_views(64)
        frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
        nq = sum(max(1, v.num_quads) for v in views)
        r = LucidRenderer(max(v.width for v in views), max(v.height for v in views), max_input_quads=nq,
                          max_visible_quads=nq, max_bin_refs=4 * nq, max_views=64)
        for _ in range(args.frames_only):
            r.render_batch(frames)
    else:
        sc = scenes.workload(args.workload)
        r = LucidRenderer(sc.width, sc.height, max_input_quads=sc.num_quads, max_visible_quads=sc.num_quads,
                          max_bin_refs=8 * sc.num_quads)
        frame, out = FrameInputs.from_scene(sc), r.new_image()
        for _ in range(args.frames_only):
            r.render(frame, out)
    torch.cuda.synchronize()
    r.close()


def main():
    args = parse_args()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.frames_only > 0:
        frames_only(args)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from lucid_gb300 import build as lucid_build
    if rank == 0:
        lucid_build.build()
    if dist is not None:
        dist.barrier()
    from lucid_gb300 import replicas, scenes, _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer

    # replicas: each rank renders its own seeded frame of the same workload
    scene = scenes.workload(args.workload, seed=replicas.rank_seed(1, rank))
    r = LucidRenderer(scene.width, scene.height, max_input_quads=scene.num_quads,
                      max_visible_quads=scene.num_quads, max_bin_refs=8 * scene.num_quads)
    frame = FrameInputs.from_scene(scene)
    out = r.new_image()
    stream = torch.cuda.current_stream()
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # correctness of the frame and its counts
    r.render(frame, out)
    info, counters = r.info()
    if info.error_code != 0:
        raise RuntimeError(f"device error {_lib.ERR_NAMES.get(info.error_code)} {tuple(info.error_detail)}")
    fragments = int(info.num_fragments)
    blended = int(info.raster_blended_fragments)
    hblock_tris = int(info.num_hblock_tris)
    qrefs, trefs = int(info.num_bin_quad_refs), int(info.num_bin_tri_refs)
    bq = r.download(_lib.BUF_BIN_QUADS, count=qrefs)
    culled = int(np.count_nonzero((bq >> 30) & 1) + np.count_nonzero((bq >> 31) & 1))
    bin_tris = 2 * qrefs - culled + trefs

    for _ in range(args.warmup):
        flush_buf.fill_(1)
        r.render(frame, out)
    torch.cuda.synchronize()

    # ---- timed region: K frames, device-resident inputs
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush_buf.fill_(i & 0xFF)
            starts[i].record(stream)
            r.render(frame, out)
            ends[i].record(stream)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # replicas: every rank's fragments over the slowest rank's time
    value, total_ms, _ = replicas.aggregate(float(sum(step_ms)), fragments * args.steps, dist, "cuda")
    ms_per_step = total_ms / args.steps

    # ---- raster kernel alone (roofline): pass-level API, events around lucid_raster
    r.quad_setup(frame)
    r.bin_count()
    r.bin_categorize()
    r.bin_dispatch()
    ras_ms = []
    for i in range(max(3, args.steps)):
        flush_buf.fill_(i & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.raster(frame, out)
        e1.record(stream)
        torch.cuda.synchronize()
        ras_ms.append(e0.elapsed_time(e1))
    raster_ms = float(np.median(ras_ms))
    w, h = scene.width, scene.height
    alg_bytes = 4 * (qrefs + trefs) + 32 * bin_tris + 68 * hblock_tris + 16 * w * h
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (raster_ms / 1e3) / 1e9
    tpf = profile_traffic_per_fragment()
    # frac is the HBM roofline fraction; the kernel keeps fragments on chip and is limited by
    # issue slots and latency (issue_active_frac, warp instructions per fragment: ncu, one launch)
    roofline = {"kernel": "rasterKernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": None if tpf is None else tpf * fragments,
                "algorithmic_bytes": alg_bytes, "kernel_ms": raster_ms,
                "limiter": "issue slots and latency (fragments stay in shared memory)", **profile_figures()}

    # ---- e2e: host buffers through lucid_render, as a serving loop: every step uploads its
    # inputs from pinned host memory and reads its image back; uploads run on one copy stream and
    # read-backs on another, so they overlap the neighbouring frames' renders (two input and two
    # image buffers)
    keys = ("positions", "colors", "quads", "instances", "instance_colors")
    host = {k: getattr(frame, k).cpu().pin_memory() for k in keys}
    fbuf = [frame, FrameInputs.from_scene(scene)]
    obuf = [out, r.new_image()]
    host_out = [torch.empty(out.shape, dtype=out.dtype).pin_memory() for _ in range(2)]
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = host_out[0].numel() * host_out[0].element_size()
    up_stream, down_stream = torch.cuda.Stream(), torch.cuda.Stream()
    up_done = [torch.cuda.Event() for _ in range(2)]
    rendered = [torch.cuda.Event() for _ in range(2)]
    read_back = [torch.cuda.Event() for _ in range(2)]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(args.warmup + args.steps):
        b = i % 2
        if i == args.warmup:
            torch.cuda.synchronize()
            e0.record(stream)
        up_stream.wait_event(rendered[b])  # frame i-2 has finished reading buffer b
        with torch.cuda.stream(up_stream):
            for k in keys:
                getattr(fbuf[b], k).copy_(host[k], non_blocking=True)
        up_done[b].record(up_stream)
        stream.wait_event(up_done[b])
        stream.wait_event(read_back[b])  # frame i-2's image has been read back
        r.render(fbuf[b], obuf[b], stream=stream)
        rendered[b].record(stream)
        down_stream.wait_event(rendered[b])
        with torch.cuda.stream(down_stream):
            host_out[b].copy_(obuf[b], non_blocking=True)
        read_back[b].record(down_stream)
    for ev in read_back:
        stream.wait_event(ev)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_value, e2e_total_ms, _ = replicas.aggregate(e0.elapsed_time(e1), fragments * args.steps, dist, "cuda")
    e2e_ms = e2e_total_ms / args.steps

    # ---- forward+backward workload (rank 0 only)
    extras = rank == 0 and not args.no_extras
    fwd_bwd = grad_bench(max(5, args.steps), max(3, args.warmup), flush_buf) if extras else None
    batch = batch_bench(max(5, args.steps), max(3, args.warmup), flush_buf) if extras else None
    quadgen = quadgen_bench(max(3, min(args.steps, 5)), 1) if extras else None
    workloads = {n: workload_bench(n, max(5, args.steps), max(3, args.warmup), flush_buf)
                 for n in ("meshes4k", "cpu720")} if extras else None

    # ---- CPU baseline and a parity check of the benchmark frame (rank 0, N=1 only; not timed)
    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baselines(scene, fragments)
        parity = parity_sample(r, frame, scene)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {**workload_config(args.workload, scene, info),
                       "l2": "flushed between steps (256 MB write, outside the step events)",
                       "parallelism": f"replicas x{world}"},
            "blended_fragments_per_s": blended * args.steps * world / (total_ms / 1e3),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                    "pipelining": "uploads and read-backs on two copy streams overlap the "
                                  "neighbouring frames' renders (two input and image buffers)"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": KERNELS_PER_FRAME * args.steps,
            "mtri_per_s": scene.num_tris * args.steps * world / (total_ms / 1e3) / 1e6,  # equal tris per rank
            "fwd_bwd": fwd_bwd,
            "batch": batch,
            "quadgen": quadgen,
            "workloads": workloads,
            "parity": parity,
        }
        print(json.dumps(line), flush=True)
    r.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
