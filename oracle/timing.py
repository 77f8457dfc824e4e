"""Per-pass timing of the CPU oracle.  TEST INFRASTRUCTURE ONLY (the timed CPU
baseline of bench.py and of the baseline table).

One warm-up frame, then the median of `runs` frames, each pass timed on its
own with all host threads (OpenMP inside the oracle).
"""
from __future__ import annotations

import os
import statistics
import time

import numpy as np

import oracle


def frame_passes(mesh, camera, dom_params, lights, env=None) -> tuple[dict, dict]:
    """One oracle frame with per-pass seconds; returns (seconds, counts)."""
    t: dict = {}
    w, h = int(camera["screen"][0]), int(camera["screen"][1])
    capacity = max(mesh.strand_count(), 1)

    def timed(name, fn):
        s = time.perf_counter()
        r = fn()
        t[name] = time.perf_counter() - s
        return r

    center, cons, beta = timed("clear", lambda: oracle.clear_targets(w, h))
    lod_c = timed("lod_camera", lambda: oracle.lod(camera, mesh))
    refs_c, total_c = timed("scan_camera", lambda: oracle.scan(camera, lod_c, capacity))
    counts = {"camera": timed("raster_camera",
                              lambda: oracle.raster(camera, mesh, refs_c, total_c, center, cons, beta, None))}
    dmap = None
    if int(camera["flags"][3]):
        dw, dh = int(dom_params["screen"][0]), int(dom_params["screen"][1])
        dmap = timed("clear_dom", lambda: oracle.clear_dom(dw, dh))
        lod_d = timed("lod_dom", lambda: oracle.lod(dom_params, mesh))
        refs_d, total_d = timed("scan_dom", lambda: oracle.scan(dom_params, lod_d, capacity))
        counts["dom_depth"] = timed("raster_dom_depth", lambda: oracle.raster(dom_params, mesh, refs_d, total_d,
                                                                              center, cons, beta, dmap))
        layers = dom_params.copy()
        layers["pass_mode"][0] = 2
        counts["dom_layers"] = timed("raster_dom_layers", lambda: oracle.raster(layers, mesh, refs_d, total_d,
                                                                                center, cons, beta, dmap))
    shaded, sdepth = timed("shade", lambda: oracle.shade(camera, center, beta, dmap, lights, env=env))
    src, srcd = shaded, sdepth
    if int(camera["flags"][1]):
        src, srcd = timed("filter", lambda: oracle.filter_(camera, center, cons, shaded, sdepth))
    color = np.zeros(w * h * 4, dtype=np.float32)
    depth = np.full(w * h, 0.0 if int(camera["pass_mode"][2]) == 1 else 1.0, dtype=np.float32)
    timed("composite", lambda: oracle.composite(camera, src, srcd, color, depth))
    return t, counts


def per_pass(mesh, camera, dom_params, lights, env=None, runs: int = 5, threads: int | None = None) -> dict:
    """Median milliseconds per pass and per frame over `runs` frames after one warm-up."""
    threads = threads or os.cpu_count() or 1
    oracle.set_threads(threads)
    frame_passes(mesh, camera, dom_params, lights, env)
    samples = [frame_passes(mesh, camera, dom_params, lights, env) for _ in range(max(runs, 1))]
    names = list(samples[0][0])
    med = {n: round(1e3 * statistics.median(s[0][n] for s in samples), 3) for n in names}
    frame = statistics.median(sum(s[0].values()) for s in samples)
    counts = samples[0][1]
    segs = int(counts["camera"]["segments"])
    return {"per_pass_ms": med, "frame_ms": round(frame * 1e3, 3), "camera_segments": segs,
            "gseg_per_s": round(segs / frame / 1e9, 6), "threads": threads, "runs": runs,
            "counts_camera": counts["camera"], "counts_dom": {k: counts[k] for k in ("dom_depth", "dom_layers")
                                                               if k in counts}}
