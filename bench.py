#!/usr/bin/env python3
"""Benchmark of the plain forward scanline fill path.

Workload: the large plain-path scene -- 2048x2048 RGBA8, 32 samples per
pixel, multisample sRGB resolve, 15,000 glyph-like paths (10-40 quadratic /
cubic segments, 8-64 px box, per-path affine scale 0.5-4 and rotation) and
5,000 large paths (50-500 mixed segments spanning up to the viewport),
painter's-order alpha blending, from one seed (synthetic: the reference's
MPVG documents are not available).  One step = one frame through the C ABI
(spr_render) with the scene resident on the device.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The line also carries, unless --no-extras: "batched" (256 uneven scenes:
one batched render against one launch sequence per scene, scenes/s),
"differentiable" (1024x1024, 256 cubic paths, 16 spp: forward, forward + L2
gradient + backward, and the plain RGBA8 frame, ms), "batched_differentiable"
(64 scenes of 512^2-1024^2 fitted by gradient descent: forward and forward +
backward per scene) and "samples_256" (the 1024x1024 scene at 256 samples
per pixel beside 32).

The line's "cpu_baseline" is the CPU oracle -- the C++ restatement of the
reference pipeline (its own GPU code needs OpenGL, unavailable on this machine)
-- rendering the whole 2048x2048 frame once on all host threads.

--impl reference times the same CPU oracle on the same frame with all host
threads, one 2048x256 row band per step: step k renders rows
256 (k mod 8) .. 256 (k mod 8) + 255, so every 8 consecutive steps render
the whole frame once, and the value is the pixels of the timed steps over
their time.  Multi-GPU runs are independent replicas (the path has no
exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
for p in (ROOT / "gpu-scanline-path-rendering_gb300", ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "Mpix/s & ms/frame vs CPU oracle; batched scenes/s and fwd+bwd ms vs plain GPU path"
UNIT = "Mpix/s"
WORKLOAD = dict(kind=1, seed=20261203, width=2048, height=2048, n_paths=15000, n_large=5000,
                seg_min=10, seg_max=40, with_rational=False, with_affine=True)
SAMPLES, MS_OUTPUT, SRGB = 32, True, True
BAND_ROWS = 256  # rows per step of the reference arm (the frame in 8 bands)
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def workload_config(extra=None):
    c = {"workload": f"plain forward, large scene: {WORKLOAD['width']}x{WORKLOAD['height']} RGBA8, 32 spp ms "
                     f"sRGB, {WORKLOAD['n_paths']} glyph-like + {WORKLOAD['n_large']} large paths",
         "width": WORKLOAD["width"], "height": WORKLOAD["height"], "samples": SAMPLES,
         "ms_output": MS_OUTPUT, "srgb": SRGB, "glyph_paths": WORKLOAD["n_paths"],
         "large_paths": WORKLOAD["n_large"], "seed": WORKLOAD["seed"],
         "l2": "flushed (512 MB write) before every timed step; per-frame buffers exceed L2"}
    if extra:
        c.update(extra)
    return c


def scale_workload(scale):
    """Scales the workload's size by `scale` (path counts by scale^2); used to
    profile the same scene family on a case small enough for full captures."""
    if scale != 1.0:
        WORKLOAD.update(width=int(round(2048 * scale)), height=int(round(2048 * scale)),
                        n_paths=int(round(15000 * scale * scale)), n_large=int(round(5000 * scale * scale)))


def make_scene():
    import spr

    w = WORKLOAD
    return spr.Scene.generate(w["kind"], seed=w["seed"], width=w["width"], height=w["height"],
                              n_paths=w["n_paths"], n_large=w["n_large"], seg_min=w["seg_min"],
                              seg_max=w["seg_max"], with_rational=w["with_rational"],
                              with_affine=w["with_affine"])


def band_transform(y0):
    import numpy as np

    m = np.eye(4, dtype=np.float32)
    m[1, 3] = -float(y0)
    return m


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
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
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------- byte accounting --
def step_bytes(counts, npairs, V, C, P, W, H, S, affine):
    """Algorithmic bytes of each timed step (one read of every input, one
    write of every output, per frame)."""
    nf, nm, ns = counts["curve_fragment"], counts["merged_fragment"], counts["span"]
    mb = S // 2  # mask bytes per 2x2 cell
    nbins = ((W + 31) // 32) * ((H + 1) // 2)
    return {
        "transform": V * 20 + P * 5 + (24 * P if affine else 0),
        "intersect_count": C * 16 + V * 8 + P + C * 12,
        "intersect_emit_fragment": C * 16 + V * 8 + nf * 16 + nf * (4 + 4 + 1 + mb + 8 + 4),
        "sort": nf * 12 * 2,
        "scan_mark": nf * 15 + (nm + ns) * 16 + nm * 4,
        "stencil": nm * 13 + nf * (16 + mb) + nm * mb,
        "resolve_bin": (nm + ns) * 24 + npairs * 32,
        "resolve": npairs * 20 + nm * mb + nbins * 8 + W * H * 4,
    }


def frame_alg_bytes(counts, V, C, P, W, H, S):
    """Frame-level algorithmic bytes B_alg of the plain path."""
    nf, nm, ns = counts["curve_fragment"], counts["merged_fragment"], counts["span"]
    return (8 * V + 14 * C + 5 * P + nf * (2 * 8 + 2 * (9 + S // 2) + 2 * 8) + nm * (2 * (S // 2))
            + (nm + ns) * 2 * 16 + 4 * W * H)


def read_traffic(kernel):
    """Per-unit DRAM traffic of `kernel` from the committed ncu summary
    (profiles/roofline.md, rows `| kernel | dram bytes per unit | unit |`)."""
    f = ROOT / "profiles" / "roofline.md"
    if not f.exists():
        return None, None
    for line in f.read_text().splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) >= 3 and cells[0] == kernel:
            try:
                return float(cells[1]), cells[2]
            except ValueError:
                return None, None
    return None, None


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------- CPU arm --
def cpu_frame(scene, threads=0):
    """The oracle on the whole frame, once; returns (Mpix/s, ms, cores)."""
    import oracle

    cores = threads or os.cpu_count()
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    t, _ = oracle.time_run(scene, W, H, SAMPLES, MS_OUTPUT, SRGB, threads=cores)
    return W * H / (t / 1e3) / 1e6, t, cores


def cpu_bands(scene, steps, warmup, threads=0):
    """The oracle one row band per step, cycling through the frame's bands
    (step k: band k mod n_bands, counted from the first warm-up step);
    returns (Mpix/s over the timed steps, mean ms per step, cores)."""
    import oracle

    cores = threads or os.cpu_count()
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    nb = (H + BAND_ROWS - 1) // BAND_ROWS
    pix, ms = 0, []
    for k in range(warmup + steps):
        y0 = (k % nb) * BAND_ROWS
        bh = min(BAND_ROWS, H - y0)
        t, _ = oracle.time_run(scene, W, bh, SAMPLES, MS_OUTPUT, SRGB, threads=cores,
                               transform=band_transform(y0))
        if k >= warmup:
            ms.append(t)
            pix += W * bh
    return pix / (sum(ms) / 1e3) / 1e6, sum(ms) / len(ms), cores


SMALL = dict(kind=0, seed=20261203, width=512, height=512, n_paths=64, seg_min=8, seg_max=32, samples=8)


def crossing_accuracy(r, scene, W, H):
    """The FP64 check of the GPU's crossing points: the TVERTEX and
    INTERSECTION stages of the frame just rendered by handle `r`, measured by
    the CPU oracle against exact FP64 crossings (errors along the cut line,
    px)."""
    import oracle

    e = oracle.intersection_error(scene, r.dump("TVERTEX"), r.dump("INTERSECTION"), W, H)
    return {"max_intersection_x_err_px": e["max_err_px"], "mean_err_px": e["mean_err_px"],
            "crossings": e["n_crossings"], "over_1px": e["n_over_1px"], "not_bracketed": e["n_unbracketed"],
            "entries_not_matching_walk": e["n_mismatched"]}


def small_scene_accuracy(dev):
    """The small plain-path workload (512x512, 8 spp, 64 paths of 8-32
    segments) rendered on the GPU, its crossings checked in FP64."""
    import spr

    w = SMALL
    sc = spr.Scene.generate(w["kind"], seed=w["seed"], width=w["width"], height=w["height"],
                            n_paths=w["n_paths"], seg_min=w["seg_min"], seg_max=w["seg_max"])
    with spr.VGRasterizer(w["width"], w["height"], samples=w["samples"], device=dev.index) as r:
        r.add_vg(sc)
        r.rasterize()
        return crossing_accuracy(r, sc, w["width"], w["height"])


def run_reference(args, rank, world):
    if rank != 0:
        return
    scene = make_scene()
    value, mean_ms, cores = cpu_bands(scene, args.steps, args.warmup)
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    sample = (f"the {W}x{H} frame in {W}x{BAND_ROWS} row bands, one band per step in order (every "
              f"{(H + BAND_ROWS - 1) // BAND_ROWS} steps render the whole frame), all stages, {cores} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- added rows --
BATCH = dict(n_scenes=256, seed=20261203, sizes=(256, 512, 1024, 2048), samples=(8, 32), paths=(10, 5000),
             seg_min=8, seg_max=32)
DIFF = dict(width=1024, height=1024, n_paths=256, seg_min=16, seg_max=64, samples=16, seed=20261203,
            jitter_px=2.0, color_sigma=0.05)


def batch_items():
    """The batched workload: 256 scenes, path count log-uniform in 10-5000,
    square resolution from {256, 512, 1024, 2048}, 8 or 32 spp, paths of
    8-32 mixed segments with control points uniform in a per-path box (side
    U[d/32, d/4])."""
    import numpy as np

    import spr

    rng = np.random.default_rng(BATCH["seed"])
    items = []
    for i in range(BATCH["n_scenes"]):
        d = int(rng.choice(BATCH["sizes"]))
        smp = int(rng.choice(BATCH["samples"]))
        n = int(np.exp(rng.uniform(np.log(BATCH["paths"][0]), np.log(BATCH["paths"][1]))))
        sc = spr.Scene.generate(spr.SCENE_LOCAL, seed=BATCH["seed"] + 1 + i, width=d, height=d, n_paths=n,
                                seg_min=BATCH["seg_min"], seg_max=BATCH["seg_max"])
        items.append((sc, d, d, smp))
    return items


def _timed(dev, stream, fn, n):
    import torch

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    fn()
    torch.cuda.synchronize(dev)
    ts = []
    for _ in range(n):
        ev[0].record(stream)
        fn()
        ev[1].record(stream)
        ev[1].synchronize()
        ts.append(ev[0].elapsed_time(ev[1]))
    return sum(ts) / len(ts)


def run_batched(dev, stream, steps=3):
    """Scenes/s of one batched render of the whole set against one launch
    sequence (spr_render) per scene, both from device-resident scenes."""
    import spr

    items = batch_items()
    sp = stream.cuda_stream
    with spr.Batch(device=dev.index) as b:
        b.set_scenes(items)
        batch_ms = _timed(dev, stream, lambda: b.render(sp), steps)
        counts = b.element_number()
        st = b.frame_stats()
        b.enable_step_timing(True)
        b.render(sp)
        step_ms = b.step_timing()
        b.enable_step_timing(False)
        b.set_graph_replay(True)  # unchanged scenes: the captured launch sequence, no host reads
        for _ in range(2):
            b.render(sp)
        graph_ms = _timed(dev, stream, lambda: b.render(sp), steps)
        graph_syncs = b.frame_stats()["host_syncs"]
    hs = []
    for sc, W, H, smp in items:
        r = spr.VGRasterizer(W, H, samples=smp, device=dev.index)
        r.add_vg(sc)
        hs.append(r)

    def each():
        for r in hs:
            r.rasterize(sp)

    single_ms = _timed(dev, stream, each, max(1, steps - 1))
    launches = sum(r.frame_stats()["kernel_launches"] for r in hs)
    for r in hs:
        r.close()
    n = len(items)
    return {"workload": "256 scenes, paths log-uniform 10-5000, 256^2-2048^2, 8/32 spp ms sRGB, "
                        "8-32 mixed segments per path in a per-path box",
            "scenes": n, "pixels": int(sum(W * H for _, W, H, _ in items)), "counts": counts,
            "scenes_per_s": n / (batch_ms / 1e3), "ms_per_batch": batch_ms,
            "per_scene_scenes_per_s": n / (single_ms / 1e3), "per_scene_ms": single_ms,
            "speedup": single_ms / batch_ms, "launches_batched": st["kernel_launches"],
            "launches_per_scene_total": launches, "host_syncs_batched": st["host_syncs"],
            "device_bytes_batched": st["device_bytes"], "step_ms_batched": step_ms,
            "graph_replay": {"ms_per_batch": graph_ms, "scenes_per_s": n / (graph_ms / 1e3),
                             "speedup": single_ms / graph_ms, "host_syncs": graph_syncs}}


def run_diff(dev, stream, steps=5):
    """Differentiable render: forward (float composite), L2-loss gradient and
    backward (edge-sampled adjoint) against a target rendered with control
    points perturbed by N(0, 2 px) and colours by N(0, 0.05); the plain
    RGBA8 frame of the same scene beside it."""
    import numpy as np
    import torch

    import spr

    W, H = DIFF["width"], DIFF["height"]
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=DIFF["seed"], width=W, height=H, n_paths=DIFF["n_paths"],
                            seg_min=DIFF["seg_min"], seg_max=DIFF["seg_max"])
    rng = np.random.default_rng(DIFF["seed"])
    P = sc.n_paths
    fill0 = np.c_[rng.uniform(0, 1, (P, 3)), rng.uniform(0.5, 1, (P, 1))].astype(np.float32)
    tgt = sc.copy()
    tgt.vertex = tgt.vertex + rng.normal(0, DIFF["jitter_px"], tgt.vertex.shape).astype(np.float32)
    fill_t = np.clip(fill0 + rng.normal(0, DIFF["color_sigma"], fill0.shape), 0, 1).astype(np.float32)
    sp = stream.cuda_stream
    fill = torch.tensor(fill0, device=dev)
    img = torch.empty((H, W, 4), device=dev)
    target = torch.empty((H, W, 4), device=dev)
    gf = torch.empty_like(fill)
    gv = torch.empty((sc.n_vertices, 2), device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with spr.VGRasterizer(W, H, samples=DIFF["samples"], device=dev.index) as r:
        r.add_vg(tgt)
        ft = torch.tensor(fill_t, device=dev)
        r.diff_render(ft.data_ptr(), target.data_ptr(), sp)
        r.add_vg(sc)
        loss = torch.zeros((), device=dev)

        def step():
            r.diff_render(fill.data_ptr(), img.data_ptr(), sp)
            ev[1].record(stream)
            diff = img - target
            loss.copy_((diff * diff).sum())
            g = (2.0 * diff).contiguous()
            r.diff_backward(fill.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr(), None, sp)

        for _ in range(2):
            step()
        torch.cuda.synchronize(dev)
        fwd, tot = [], []
        for _ in range(steps):
            ev[0].record(stream)
            step()
            ev[2].record(stream)
            ev[2].synchronize()
            fwd.append(ev[0].elapsed_time(ev[1]))
            tot.append(ev[0].elapsed_time(ev[2]))
        dev_bytes = r.frame_stats()["device_bytes"]
        plain = _timed(dev, stream, lambda: r.rasterize(sp), steps)
        counts = r.element_number()
    f, t = sum(fwd) / len(fwd), sum(tot) / len(tot)
    return {"workload": f"{W}x{H}, {P} closed paths of 16-64 cubic segments, 16 spp, L2 loss vs a target with "
                        "control points + N(0, 2 px) and colours + N(0, 0.05)",
            "counts": counts, "fwd_ms": f, "fwd_bwd_ms": t, "fwd_bwd_over_fwd": t / f,
            "plain_rgba8_ms": plain, "fwd_bwd_over_plain": t / plain, "loss": float(loss),
            "device_bytes": dev_bytes}


BDIFF = dict(n_scenes=64, seed=20261204, sizes=(512, 640, 768, 896, 1024), paths=(128, 512), seg_min=16,
             seg_max=64, samples=16, steps=100, lr_fill=0.5, lr_point=4.0)


def run_batched_diff(dev, stream, steps=None):
    """Batched forward + backward: 64 scenes of uneven size fitted by plain
    gradient descent on contour points and fill colours (L2 loss against
    targets rendered with points + N(0, 2 px) and colours + N(0, 0.05)); each
    step moves the vertices on the device (spr_batch_update_vertices),
    renders, takes the loss gradient and runs the backward, which recomputes
    every stage."""
    import numpy as np
    import torch

    import spr

    steps = steps or BDIFF["steps"]
    rng = np.random.default_rng(BDIFF["seed"])
    items, fills, tgt_v, tgt_f, keys = [], [], [], [], []
    for i in range(BDIFF["n_scenes"]):
        d = int(rng.choice(BDIFF["sizes"]))
        n = int(rng.integers(BDIFF["paths"][0], BDIFF["paths"][1] + 1))
        sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=BDIFF["seed"] + 1 + i, width=d, height=d, n_paths=n,
                                seg_min=BDIFF["seg_min"], seg_max=BDIFF["seg_max"])
        items.append((sc, d, d, BDIFF["samples"]))
        f = np.c_[rng.uniform(0, 1, (n, 3)), rng.uniform(0.5, 1, (n, 1))].astype(np.float32)
        fills.append(f)
        tgt_v.append(sc.vertex + rng.normal(0, 2.0, sc.vertex.shape).astype(np.float32))
        tgt_f.append(np.clip(f + rng.normal(0, 0.05, f.shape), 0, 1).astype(np.float32))
    # contour points: the coincident end points of consecutive curves are one parameter
    vert = np.concatenate([it[0].vertex for it in items])
    pid = np.concatenate([it[0].vertex_path_id + sum(x[0].n_paths for x in items[:k]) for k, it in enumerate(items)])
    key = np.c_[pid.astype(np.float64), vert.astype(np.float64)]
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    idx = torch.tensor(inv.reshape(-1), device=dev)
    sp = stream.cuda_stream
    pts = torch.tensor(uniq[:, 1:].astype(np.float32), device=dev)
    fill = torch.tensor(np.concatenate(fills), device=dev)
    V, P = vert.shape[0], fill.shape[0]
    gf = torch.empty((P, 4), device=dev)
    gv = torch.empty((V, 2), device=dev)
    torch.cuda.reset_peak_memory_stats(dev)
    with spr.Batch(device=dev.index) as b:
        b.set_scenes(items)
        npix = int(b.image_offsets()[-1])
        img = torch.empty((npix, 4), device=dev)
        target = torch.empty((npix, 4), device=dev)
        b.update_vertices(torch.tensor(np.concatenate(tgt_v), device=dev).data_ptr(), sp)
        b.diff_render(torch.tensor(np.concatenate(tgt_f), device=dev).data_ptr(), target.data_ptr(), sp)
        losses = []
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        fwd_ms, bwd_ms, tot_ms = [], [], []
        for k in range(steps):
            ev[0].record(stream)
            v = pts[idx].contiguous()
            b.update_vertices(v.data_ptr(), sp)
            ev[1].record(stream)
            b.diff_render(fill.data_ptr(), img.data_ptr(), sp)
            ev[2].record(stream)
            diff = img - target
            g = (2.0 * diff).contiguous()
            ev[3].record(stream)
            b.diff_backward(fill.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr(), None, sp)
            ev[4].record(stream)
            with torch.no_grad():
                gpt = torch.zeros_like(pts).index_add_(0, idx, gv)
                fill -= BDIFF["lr_fill"] * gf / npix * 1e3
                fill.clamp_(0.0, 1.0)
                pts -= BDIFF["lr_point"] * gpt / (gpt.abs().max() + 1e-12)
            ev[5].record(stream)
            ev[5].synchronize()
            fwd_ms.append(ev[1].elapsed_time(ev[2]))
            bwd_ms.append(ev[3].elapsed_time(ev[4]))
            tot_ms.append(ev[0].elapsed_time(ev[5]))
            if k in (0, steps - 1):
                losses.append(float((diff * diff).sum()))
        dev_bytes = b.frame_stats()["device_bytes"]
    peak = torch.cuda.max_memory_allocated(dev) + dev_bytes
    n = len(items)
    def mean(x):
        return sum(x[1:]) / (len(x) - 1)

    f_ms, b_ms, t_ms = mean(fwd_ms), mean(bwd_ms), mean(tot_ms)
    return {"workload": f"{n} scenes of 128-512 closed cubic paths (16-64 segments), 512^2-1024^2, 16 spp; "
                        f"{steps} descent steps on contour points and fills (L2 to perturbed targets)",
            "pixels": npix, "paths": P, "vertices": V, "steps": steps,
            "fwd_ms_per_scene": f_ms / n, "fwd_bwd_ms_per_scene": (f_ms + b_ms) / n,
            "fwd_bwd_over_fwd": (f_ms + b_ms) / f_ms,
            "step_ms": t_ms, "step": "vertex update + forward + loss gradient + backward + descent update",
            "loss_first": losses[0], "loss_last": losses[-1],
            "peak_hbm_bytes": int(peak), "graph": "no: sizes change as the geometry moves (read back per step)"}


def run_spp256(dev, stream, steps=5):
    """256 samples per pixel (8 passes of 32, exact mean of all samples)
    beside 32 on the differentiable workload's scene: plain RGBA8 frames, and
    the differentiable forward + backward."""
    import numpy as np
    import torch

    import spr

    W, H = DIFF["width"], DIFF["height"]
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=DIFF["seed"], width=W, height=H, n_paths=DIFF["n_paths"],
                            seg_min=DIFF["seg_min"], seg_max=DIFF["seg_max"])
    sp = stream.cuda_stream
    fill = torch.tensor(np.random.default_rng(DIFF["seed"]).uniform(0.2, 1.0, (sc.n_paths, 4)).astype(np.float32),
                        device=dev)
    img = torch.empty((H, W, 4), device=dev)
    g = torch.ones_like(img)
    gf = torch.empty_like(fill)
    gv = torch.empty((sc.n_vertices, 2), device=dev)
    out = {"workload": f"{W}x{H}, {DIFF['n_paths']} closed paths of 16-64 cubic segments"}
    for smp in (32, 256):
        with spr.VGRasterizer(W, H, samples=smp, device=dev.index) as r:
            r.add_vg(sc)
            plain = _timed(dev, stream, lambda: r.rasterize(sp), steps)

            def fb():
                r.diff_render(fill.data_ptr(), img.data_ptr(), sp)
                r.diff_backward(fill.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr(), None, sp)

            out[f"spp{smp}"] = {"plain_ms": plain, "fwd_bwd_ms": _timed(dev, stream, fb, steps)}
    out["plain_256_over_32"] = out["spp256"]["plain_ms"] / out["spp32"]["plain_ms"]
    return out


# ------------------------------------------------------------- GPU arm --
def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import spr

    if not spr.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    scene = make_scene()
    r = spr.VGRasterizer(W, H, samples=SAMPLES, ms_output=MS_OUTPUT, srgb=SRGB, device=local_rank)
    r.add_vg(scene)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    for _ in range(args.warmup):
        r.rasterize(sp)
    torch.cuda.synchronize(dev)
    counts = r.element_number()
    stats = r.frame_stats()
    launches = stats["kernel_launches"]

    # ---- timed region: device-resident scene, one frame per step
    r.enable_step_timing(True)
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize(dev)
    frame_ms, steps = [], {}
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.rasterize(sp)
        e1.record(stream)
        e1.synchronize()
        frame_ms.append(e0.elapsed_time(e1))
        for k, v in r.step_timing().items():
            steps.setdefault(k, []).append(v)
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop()
    r.enable_step_timing(False)
    ms = sum(frame_ms) / len(frame_ms)
    ms_max = allreduce_max(ms, world)
    value = world * W * H / (ms_max / 1e3) / 1e6

    if args.profile:
        if rank == 0:
            print(json.dumps({"profile": True, "ms_per_step": ms_max, "step_ms": {
                k: sum(v) / len(v) for k, v in steps.items()}, "counts": counts}), flush=True)
        return
    # ---- end to end through the C ABI with host buffers: scene H2D (pinned),
    #      render, image D2H (pinned), every step
    pinned = [torch.from_numpy(getattr(scene, f)).pin_memory() if getattr(scene, f) is not None else None
              for f in spr.Scene.FIELDS]
    host_scene = spr.Scene(*[p.numpy() if p is not None else None for p in pinned])
    img = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory()
    bi = sum(getattr(host_scene, f).nbytes for f in spr.Scene.FIELDS if getattr(host_scene, f) is not None)
    bo = img.numel()
    for _ in range(1):
        r.add_vg(host_scene)
        r.rasterize(sp)
        r.read_image(img.numpy(), sp)
    e2e_ms = []
    barrier(world)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r.add_vg(host_scene)
        r.rasterize(sp)
        r.read_image(img.numpy(), sp)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = sum(e2e_ms) / len(e2e_ms)
    e2e_max = allreduce_max(e2e, world)
    e2e_value = world * W * H / (e2e_max / 1e3) / 1e6

    if rank != 0:
        return
    # ---- roofline of the dominant step
    step_mean = {k: sum(v) / len(v) for k, v in steps.items()}
    dom = max(step_mean, key=step_mean.get)
    npairs = stats["resolve_pairs"]
    sb = step_bytes(counts, npairs, scene.n_vertices, scene.n_curves, scene.n_paths, W, H, SAMPLES,
                    scene.path_affine is not None)
    peak, peak_kind = peaks()
    achieved = sb[dom] / (step_mean[dom] / 1e3) / 1e9
    per_unit, unit_name = read_traffic(dom)
    units = {"fragment": counts["curve_fragment"], "pixel": W * H}.get(unit_name or "", None)
    traffic = per_unit * units if (per_unit is not None and units) else None
    frame_bytes = frame_alg_bytes(counts, scene.n_vertices, scene.n_curves, scene.n_paths, W, H, SAMPLES)
    # the dominant step's instruction-issue roofline: warp instructions per
    # unit from the committed ncu capture (scaled by the frame's units) over
    # the step's time, against one instruction per scheduler per cycle
    inst_unit, inst_unit_name = read_traffic(dom + "_warp_instructions")
    issue = None
    if inst_unit is not None and clk.get("sm_mhz"):
        n_units = {"pixel": W * H}.get(inst_unit_name, 0)
        inst = inst_unit * n_units
        peak_inst = torch.cuda.get_device_properties(dev).multi_processor_count * 4 * clk["sm_mhz"] * 1e6
        issue = {"bound": "issue", "warp_instructions": inst, "achieved": inst / (step_mean[dom] / 1e3),
                 "peak": peak_inst, "unit": "warp instructions/s", "frac": inst / (step_mean[dom] / 1e3) / peak_inst,
                 "source": f"ncu warp instructions per {inst_unit_name} (profiles/roofline.md) x the frame's units; "
                           "peak = SMs x 4 schedulers x median SM clock"}

    cpu_value, cpu_ms, cores = cpu_frame(scene)
    accuracy = {"large_frame": crossing_accuracy(r, scene, W, H), "small_frame": small_scene_accuracy(dev),
                "what": "GPU crossing points (FP32) vs exact FP64 crossings of the same curves and cut lines, "
                        "error along the cut line in px, checked by the CPU oracle"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(),
        "frame": {"counts": counts, "resolve_pairs": npairs, "host_syncs_per_frame": stats["host_syncs"],
                  "device_bytes": stats["device_bytes"]},
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_max, "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo},
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "alg_bytes": sb[dom], "ms": step_mean[dom], "issue": issue},
        "frame_roofline": {"alg_bytes": frame_bytes, "achieved": frame_bytes / (ms_max / 1e3) / 1e9,
                           "frac": frame_bytes / (ms_max / 1e3) / 1e9 / peak, "unit": "GB/s"},
        "step_ms": step_mean,
        "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the whole {W}x{H} frame once, all stages, {cores} threads",
                         "ms": cpu_ms},
        "intersection_accuracy": accuracy,
    }
    if not args.no_extras:  # the batched and differentiable rows, on this GPU after the plain frames
        del flush
        line["batched"] = run_batched(dev, stream)
        line["differentiable"] = run_diff(dev, stream)
        line["batched_differentiable"] = run_batched_diff(dev, stream)
        line["samples_256"] = run_spp256(dev, stream)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------- distributed --
def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="linear size scale of the workload (profiling of smaller cases)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-scenes and differentiable-render measurements")
    ap.add_argument("--profile", action="store_true",
                    help="timed GPU frames only (no end-to-end or CPU legs), for profiler runs")
    ap.add_argument("--part", choices=["all", "batched", "diff", "batched_diff", "spp256"], default="all",
                    help="run only the batched or the differentiable measurement (one JSON object), "
                         "for profiler runs")
    ap.add_argument("--bd-scenes", type=int, default=BDIFF["n_scenes"],
                    help="scenes of the batched differentiable measurement (smaller cases for profiling)")
    args = ap.parse_args()
    BDIFF["n_scenes"] = args.bd_scenes
    scale_workload(args.scale)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.part != "all":
        import torch

        dev = torch.device("cuda", local_rank)
        torch.cuda.set_device(dev)
        stream = torch.cuda.current_stream(dev)
        fn = {"batched": run_batched, "diff": run_diff, "batched_diff": run_batched_diff,
              "spp256": run_spp256}[args.part]
        print(json.dumps({args.part: fn(dev, stream, steps=max(2, args.steps))}), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group(backend="nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
