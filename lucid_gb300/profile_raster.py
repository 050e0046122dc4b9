"""Phase timers and work counters of the raster pass on one of the benchmark workloads.

    python -m lucid_gb300.build --counters          # liblucid_gb300_counters.so
    python -m lucid_gb300.profile_raster heavy1080   # one frame, JSON on stdout

The frame is rendered with LUCID_OPT_TIMERS by the counters build of the library (the product
library is not loaded). Phase times are SM time per SM (clock64 deltas of thread 0 between the
raster kernel's CTA barriers, summed over the persistent CTAs and divided by the SM count)
at the SM clock given by --mhz; the counters are the ones listed at the top of
csrc/lucid_raster.cu. ms_frame is a frame of the same workload by the counters build, timed
with CUDA events without timers (the counters cost a few spilled registers: it is slower than
the product library's frame).
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np
import torch

from lucid_gb300 import _lib, build, scenes
from lucid_gb300.renderer import FrameInputs, LucidRenderer

PHASES = ["row spans", "counts, equal-key runs", "key ranges, slabs", "window selection, generation",
          "sorts", "shading", "blending", "output, bin fetch"]
COUNTERS = ["key_range_entry_visits", "slab_hist_evaluated", "slab_hist_counted", "window_gen_evaluated",
            "window_gen_kept", "slab_entries_broadcast", "window_entries_broadcast", "slabs", "window_groups",
            "direct_slab_fallbacks", "fragments_shaded", "windows", "selection_cycles", "generation_cycles",
            "key_range_cycles", "walk_cycles", "append_warp_cycles", "append_wall_cycles", "walk_warp_cycles",
            "walk_wall_cycles"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", nargs="?", default="heavy1080")
    ap.add_argument("--mhz", type=float, default=2070.0, help="SM clock of the cycle counts")
    args = ap.parse_args()
    if not os.path.exists(build.COUNTERS_LIB):
        raise SystemExit("run `python -m lucid_gb300.build --counters` first")
    _lib.LIB_PATH = build.COUNTERS_LIB
    sc = scenes.workload(args.workload)
    nq = sc.num_quads
    frame = FrameInputs.from_scene(sc)
    plain = LucidRenderer(sc.width, sc.height, max_input_quads=nq, max_visible_quads=nq)
    out = plain.new_image()
    for _ in range(3):
        plain.render(frame, out)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    times = []
    for _ in range(5):
        torch.cuda.synchronize()
        ev[0].record()
        plain.render(frame, out)
        ev[1].record()
        torch.cuda.synchronize()
        times.append(ev[0].elapsed_time(ev[1]))
    timed = LucidRenderer(sc.width, sc.height, max_input_quads=nq, max_visible_quads=nq, flags=_lib.OPT_TIMERS)
    timed.render(frame, out)
    torch.cuda.synchronize()
    info, _ = timed.info()
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    per_sm_ms = np.array(info.raster_timers, np.float64) * 256 / nsm / (args.mhz * 1e3)
    counts = np.frombuffer(bytes(info.temp), dtype=np.uint64)
    res = {
        "workload": args.workload,
        "ms_frame": sorted(times)[len(times) // 2],
        "fragments": int(info.num_fragments),
        "blended": int(info.raster_blended_fragments),
        "windows": int(info.raster_windows),
        "window_fragments": int(info.raster_window_fragments),
        "light_bins": int(info.raster_light_bins),
        "phase_ms_per_sm": {n: round(float(v), 3) for n, v in zip(PHASES, per_sm_ms)},
        "counters": {n: int(v) for n, v in zip(COUNTERS, counts)},
    }
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
