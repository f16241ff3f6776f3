"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference tree is mounted (it builds oracle/_ref/libref.so from
the reference sources in place, see oracle/build_oracle.py):

    python tests/golden/make_goldens.py

Fixtures:
  sample_positions.json  pixel sample patterns (8, 32 spp) from the
                         reference's vg_sample_position, as float bit patterns
  mask_tables.json       SHA-256 of the reference's makeTable output (8, 32)
  mask_vectors.npz       inputs / outputs of the reference's fetchPixelTable,
                         fetchVerticalTable and fetchVerticalTable2
  scene_*.npz            small scenes (all arrays stored, so the fixtures do not
                         depend on any host's math library) with the
                         reference's per-curve entry counts and intersection
                         entries (k_make_intersection_0/1) for the transformed
                         vertices the oracle computes
"""
from __future__ import annotations

import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT / "gpu-scanline-path-rendering_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

import build_oracle  # noqa: E402
import oracle  # noqa: E402
import spr  # noqa: E402


def handmade_scene() -> spr.Scene:
    """Edge cases: grid-aligned lines, degenerate and out-of-view curves, a
    path inside one cell, vertical tangents, a cusp, rational weights."""
    paths = []  # (rule, rgba, [(type, [(x, y), ...], w)])
    L, Q, C, R = spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_CUBIC, spr.CURVE_RATIONAL

    def poly(pts, t=L):
        return [(t, [pts[i], pts[(i + 1) % len(pts)]], 1.0) for i in range(len(pts))]

    paths.append((0, 0xFF2040C0, poly([(8, 8), (40, 8), (40, 24), (8, 24)])))           # on the grid
    paths.append((1, 0xC0208040, poly([(20.5, 4.25), (60.75, 30.5), (10.25, 50.5)])))
    paths.append((0, 0xFF000000, [(L, [(30, 30), (30, 30)], 1.0), (L, [(30, 30), (30, 30)], 1.0)]))  # degenerate
    paths.append((0, 0x80FF0000, poly([(-50, -50), (-10, -50), (-30, -10)])))           # outside
    paths.append((1, 0xA000FF00, poly([(90, 20), (200, 40), (95, 70)])))                # crosses the right edge
    paths.append((0, 0xFFFF00FF, poly([(50.2, 50.2), (51.3, 50.4), (50.6, 51.1)])))     # inside one cell
    paths.append((0, 0xE0FFFF00, [(Q, [(60, 60), (90, 90), (60, 120)], 1.0),          # vertical tangent
                                  (L, [(60, 120), (60, 60)], 1.0)]))
    paths.append((1, 0xD00080FF, [(C, [(10, 70), (60, 120), (0, 120), (50, 70)], 1.0),  # self-crossing cubic
                                  (L, [(50, 70), (10, 70)], 1.0)]))
    paths.append((0, 0xF0800080, [(R, [(70, 10), (100, 10), (100, 40)], 0.7071067811865476),
                                  (R, [(100, 40), (100, 70), (70, 70)], 2.0),
                                  (L, [(70, 70), (70, 10)], 1.0)]))
    paths.append((1, 0xFF40FF40, [(C, [(20, 100), (20, 100), (40, 100), (40, 100)], 1.0),  # cusp-like cubic
                                  (Q, [(40, 100), (30, 127.5), (20, 100)], 1.0)]))
    vert, vpid, cvp, ctype, cpid, cw, rule, rgba = [], [], [], [], [], [], [], []
    for pid, (r, c, curves) in enumerate(paths):
        rule.append(r)
        rgba.append(c)
        for t, pts, w in curves:
            cvp.append(len(vert))
            ctype.append(t)
            cpid.append(pid)
            cw.append(w if t == R else -1.0)
            for p in pts:
                vert.append(p)
                vpid.append(pid)
    return spr.Scene(np.array(vert, np.float32), vpid, cvp, ctype, cpid, cw, rule, rgba)


def scene_cases():
    rot = np.array([[0.9, -0.35, 0.0, 12.0], [0.35, 0.9, 0.0, -7.5], [0.0, 0.0, 1.0, 0.0],
                    [0.0004, 0.0002, 0.0, 1.0]], np.float32)  # rotation, scale, perspective
    return [
        ("random", spr.Scene.generate(spr.SCENE_RANDOM, seed=101, width=128, height=128, n_paths=10,
                                      seg_min=4, seg_max=12, with_rational=True), 128, 128, None),
        ("cubics", spr.Scene.generate(spr.SCENE_CUBICS, seed=102, width=192, height=192, n_paths=8,
                                      seg_min=8, seg_max=16), 192, 192, None),
        ("mixed", spr.Scene.generate(spr.SCENE_MIXED, seed=103, width=256, height=256, n_paths=60,
                                     n_large=6, with_affine=True), 256, 256, None),
        ("oddsize", spr.Scene.generate(spr.SCENE_RANDOM, seed=104, width=129, height=97, n_paths=8,
                                       seg_min=4, seg_max=10, with_rational=True), 129, 97, rot),
        ("handmade", handmade_scene(), 128, 128, None),
    ]


def save_scene(name, scene, W, H, transform):
    r = oracle.run(scene, W, H, samples=8, transform=transform, stop_after=spr.STAGE["INTERSECTION"])
    tv = r["TVERTEX"].reshape(-1, 2)
    vis = r["PATH_VISIBLE"]
    counts, entries = oracle.ref_intersections(scene, tv, vis, W, H)
    arrays = {f: getattr(scene, f) for f in spr.Scene.FIELDS if getattr(scene, f) is not None}
    np.savez_compressed(HERE / f"scene_{name}.npz", width=W, height=H,
                        transform=np.eye(4, dtype=np.float32) if transform is None else transform,
                        has_transform=transform is not None, ref_counts=counts, ref_entries=entries,
                        **arrays)
    print(f"scene_{name}: {scene.n_curves} curves, {len(entries)} entries")


def main():
    if build_oracle.build_ref() is None:
        sys.exit("the reference tree is not mounted; fixtures cannot be regenerated here")
    build_oracle.build_oracle()
    sp = {str(s): [int(v) for v in oracle.ref_sample_positions(s).view(np.uint32).reshape(-1)] for s in (8, 32)}
    (HERE / "sample_positions.json").write_text(json.dumps(sp, indent=1))
    t8, t32 = oracle.ref_mask_table(oracle.sample_positions(8), oracle.sample_positions(32))
    digests = {"8": hashlib.sha256(t8.tobytes()).hexdigest(), "32": hashlib.sha256(t32.tobytes()).hexdigest()}
    (HERE / "mask_tables.json").write_text(json.dumps(digests, indent=1))
    rng = np.random.default_rng(2024)
    vec = {}
    for S, tab in ((8, t8.reshape(-1, 1)), (32, t32)):
        p = rng.uniform(-0.1, 1.1, (3000, 4)).astype(np.float32)
        vec[f"fetch{S}_in"] = p
        vec[f"fetch{S}_out"] = np.array([oracle.ref_fetch_pixel_table(S, tab, q[:2], q[2:]) for q in p])
        ys = rng.uniform(0.0, 1.0, (3000, 2)).astype(np.float32)
        # the reference's host build shifts by the full width where y rounds to
        # zero rows (undefined in C); those inputs are left out of the vectors
        lim = 16 if S == 8 else 64
        keep = [(int(round(float(a) * lim)) > 0 and int(float(a * np.float32(lim)) + 0.5) > 0
                 and int(float(b * np.float32(lim)) + 0.5) > 0) for a, b in ys]
        ys = ys[np.array(keep)]
        vec[f"vert{S}_in"] = ys
        vec[f"vert{S}_out"] = np.array([oracle.ref_vertical_mask(S, a) for a, _ in ys])
        vec[f"vert2_{S}_out"] = np.array([oracle.ref_vertical_mask2(S, a, b) for a, b in ys])
    np.savez_compressed(HERE / "mask_vectors.npz", **vec)
    for name, scene, W, H, tf in scene_cases():
        save_scene(name, scene, W, H, tf)


if __name__ == "__main__":
    main()
