"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Integer and bit-pattern stages must match exactly: intersection counts and
entries, cell keys, path ids with winding changes, scanline winding numbers,
boundary sample masks, the sort permutation, scanned winding numbers, merged
sample masks and the draw list.  The RGBA8 image is allowed +-1 per channel
(the resolve arithmetic is identical on both sides, so in practice it is
exact and the tests report the maximum difference).
"""
import pathlib
import struct
import zlib

import numpy as np
import pytest

import oracle
import spr

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
EXACT = ["TVERTEX", "PATH_VISIBLE", "CURVE_COUNT", "INTERSECTION", "FRAG_KEY", "FRAG_PID", "FRAG_WN",
         "FRAG_MASK", "SORT_PERM", "SORT_KEY", "WN_SCAN", "MERGED_MASK", "DRAW_LIST"]
IMAGE_TOL = 1  # RGBA8 per-channel tolerance


def render(scene, W, H, samples=8, ms=True, srgb=True, transform=None):
    r = spr.VGRasterizer(W, H, samples=samples, ms_output=ms, srgb=srgb)
    if transform is not None:
        r.set_input_transform(transform)
    r.add_vg(scene)
    r.rasterize()
    return r


def check_parity(scene, W, H, samples=8, ms=True, srgb=True, transform=None):
    ref = oracle.run(scene, W, H, samples=samples, ms_output=ms, srgb=srgb, transform=transform)
    with render(scene, W, H, samples, ms, srgb, transform) as r:
        assert r.element_number() == ref.counts
        for st in EXACT:
            got, exp = r.dump(st), ref[st]
            assert got.shape == exp.shape, st
            assert np.array_equal(got.view(np.uint8), exp.view(np.uint8)), st
        img = r.read_image()
        diff = np.abs(img.astype(np.int16) - ref["IMAGE"].reshape(H, W, 4).astype(np.int16)).max()
        assert diff <= IMAGE_TOL
        return ref.counts, int(diff)


def load_golden(name):
    d = np.load(GOLDEN / f"scene_{name}.npz")
    fields = {f: d[f] for f in spr.Scene.FIELDS if f in d.files}
    tf = d["transform"] if bool(d["has_transform"]) else None
    return spr.Scene(**fields), int(d["width"]), int(d["height"]), tf, d["ref_counts"], d["ref_entries"]


@pytest.mark.parametrize("name", ["random", "cubics", "mixed", "oddsize", "handmade"])
@pytest.mark.parametrize("samples", [8, 16, 32])
def test_golden_scenes(name, samples):
    scene, W, H, tf, counts, entries = load_golden(name)
    check_parity(scene, W, H, samples=samples, transform=tf)
    with render(scene, W, H, samples, transform=tf) as r:  # against the reference's own kernels
        assert np.array_equal(r.dump("CURVE_COUNT"), counts)
        assert np.array_equal(r.dump("INTERSECTION").reshape(-1, 2), entries)


@pytest.mark.parametrize("samples", [8, 16, 32])
@pytest.mark.parametrize("ms", [True, False])
@pytest.mark.parametrize("srgb", [True, False])
def test_mode_matrix(samples, ms, srgb):
    scene = spr.Scene.generate(spr.SCENE_RANDOM, seed=21, width=256, height=192, n_paths=24, seg_min=6,
                               seg_max=20, with_rational=True)
    check_parity(scene, 256, 192, samples, ms, srgb)


@pytest.mark.parametrize("kind,size,n,nl", [(spr.SCENE_RANDOM, 512, 64, 0), (spr.SCENE_MIXED, 768, 900, 60),
                                            (spr.SCENE_CUBICS, 640, 48, 0)])
@pytest.mark.parametrize("samples", [16, 32])
def test_scene_families(kind, size, n, nl, samples):
    scene = spr.Scene.generate(kind, seed=31, width=size, height=size, n_paths=n, n_large=nl,
                               seg_min=8 if kind != spr.SCENE_CUBICS else 16,
                               seg_max=32 if kind != spr.SCENE_CUBICS else 64, with_rational=True,
                               with_affine=kind == spr.SCENE_MIXED)
    check_parity(scene, size, size, samples=samples)


def test_transforms():
    scene = spr.Scene.generate(spr.SCENE_MIXED, seed=41, width=400, height=300, n_paths=200, n_large=10,
                               with_affine=True)
    a = np.float32(0.4)
    rot = np.array([[np.cos(a) * 1.3, -np.sin(a), 0, 40], [np.sin(a), np.cos(a) * 0.8, 0, -30], [0, 0, 1, 0],
                    [0.0003, -0.0002, 0, 1]], np.float32)
    check_parity(scene, 400, 300, samples=8, transform=rot)
    zoom = np.diag([3.0, 3.0, 1.0, 1.0]).astype(np.float32)
    zoom[0, 3], zoom[1, 3] = -300, -250
    check_parity(scene, 400, 300, samples=32, transform=zoom)


@pytest.mark.parametrize("W,H", [(1, 1), (3, 5), (4096, 8), (8, 4096), (257, 129)])
def test_sizes(W, H):
    scene = spr.Scene.generate(spr.SCENE_RANDOM, seed=51, width=W, height=H, n_paths=6, seg_min=3, seg_max=8)
    check_parity(scene, W, H, samples=8)


def test_empty_and_invisible_scenes():
    empty = spr.Scene(np.zeros((0, 2), np.float32), [], [], [], [], [], [], [])
    with render(empty, 64, 48) as r:
        assert r.element_number()["curve_fragment"] == 0
        assert np.all(r.read_image() == 255)
    far = spr.Scene.generate(spr.SCENE_RANDOM, seed=52, width=100, height=100, n_paths=5, seg_min=3, seg_max=6)
    far.vertex[:, 0] += 5000.0
    counts, _ = check_parity(far, 100, 100, samples=8)
    assert counts["curve_fragment"] == 0


def test_huge_coordinates_and_degenerate_curves():
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=53, width=200, height=200, n_paths=10, seg_min=4, seg_max=10)
    s.vertex[s.vertex_path_id == 1] *= 1.0e4
    s.vertex[s.vertex_path_id == 2] = s.vertex[s.vertex_path_id == 2][0]  # every point equal
    s.vertex[s.vertex_path_id == 3] = np.round(s.vertex[s.vertex_path_id == 3])  # on the pixel grid
    check_parity(s, 200, 200, samples=32)


def test_errors_leave_the_handle_usable():
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=54, width=64, height=64, n_paths=4, seg_min=3, seg_max=5)
    with spr.VGRasterizer(64, 64, samples=8) as r:
        with pytest.raises(spr.SprError) as e:
            r.rasterize()
        assert e.value.status == spr.ERR_NO_SCENE
        with pytest.raises(spr.SprError) as e:
            r.dump("IMAGE")
        assert e.value.status == spr.ERR_NO_SCENE
        bad = s.copy()
        bad.curve_type[0] = 9
        with pytest.raises(spr.SprError) as e:
            r.add_vg(bad)
        assert e.value.status == spr.ERR_INVALID_SCENE
        with pytest.raises(spr.SprError):
            r.resize_output_buffer(0, 10)
        r.add_vg(s)
        r.rasterize()
        assert r.element_number()["curve_fragment"] > 0


def test_determinism_resize_and_samples():
    s = spr.Scene.generate(spr.SCENE_MIXED, seed=55, width=300, height=300, n_paths=150, n_large=8,
                           with_affine=True)
    with render(s, 300, 300, samples=32) as r:
        a = r.read_image().copy()
        r.rasterize()
        assert np.array_equal(a, r.read_image())
        r.set_samples(8)
        r.rasterize()
        ref8 = oracle.run(s, 300, 300, samples=8)
        assert np.array_equal(r.read_image().reshape(-1), ref8["IMAGE"])
        r.resize_output_buffer(160, 120)
        r.rasterize()
        ref = oracle.run(s, 160, 120, samples=8)
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        assert np.array_equal(r.dump("MERGED_MASK"), ref["MERGED_MASK"])


def _read_png(path):
    data = pathlib.Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (4 * w + 1) + 1:(y + 1) * (4 * w + 1)] for y in range(h)]
    return np.frombuffer(b"".join(rows), np.uint8).reshape(h, w, 4)


def test_save_png_flips_and_forces_alpha(tmp_path):
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=56, width=90, height=70, n_paths=8, seg_min=3, seg_max=9)
    with render(s, 90, 70) as r:
        img = r.read_image()
        r.save_output_to_file(tmp_path / "out.png")
    png = _read_png(tmp_path / "out.png")
    exp = img[::-1].copy()
    exp[..., 3] = 255
    assert np.array_equal(png, exp)


def test_step_timing_and_stats():
    s = spr.Scene.generate(spr.SCENE_RANDOM, seed=57, width=256, height=256, n_paths=20, seg_min=5, seg_max=12)
    with spr.VGRasterizer(256, 256, samples=8) as r:
        r.add_vg(s)
        r.enable_step_timing(True)
        r.rasterize()
        t = r.step_timing()
        assert set(t) >= {"transform", "sort", "resolve"} and all(v >= 0 for v in t.values())
        st = r.frame_stats()
        assert st["kernel_launches"] > 10 and st["host_syncs"] == 2 and st["device_bytes"] > 0  # sized
        r.rasterize()
        assert r.frame_stats()["host_syncs"] == 0  # later frames read nothing back


def test_small_scene_as_specified():
    """The small plain-path workload exactly as specified: 512x512 RGBA8,
    8 samples per pixel, 64 closed paths of 8-32 segments (40% line, 30%
    quadratic, 30% cubic, control points uniform in the viewport), identity
    transform, solid fills (RGB U[0,1], alpha U[0.5,1]), nonzero / even-odd
    50/50, one seed: every stage and the image exact against the oracle."""
    scene = spr.Scene.generate(spr.SCENE_RANDOM, seed=20261203, width=512, height=512, n_paths=64, seg_min=8,
                               seg_max=32)
    types = scene.curve_type
    assert np.all(np.isin(types, [spr.CURVE_LINEAR, spr.CURVE_QUADRATIC, spr.CURVE_CUBIC]))
    for ms in (True, False):
        counts, diff = check_parity(scene, 512, 512, samples=8, ms=ms)
        assert counts["path"] == 64 and counts["curve_fragment"] > 100_000 and diff == 0


def test_benchmark_scene_full_frame():
    """The whole 2048x2048, 32-spp benchmark frame (15,000 glyph-like and
    5,000 large paths): every stage and the image exact against the oracle."""
    import bench

    scene = bench.make_scene()
    counts, diff = check_parity(scene, 2048, 2048, samples=32)
    assert counts["curve_fragment"] > 10_000_000 and diff == 0


def test_memory_limit_refuses_then_recovers():
    """A cap on the handle's device memory (the reference's fixed arena that
    throws when exhausted): a frame that needs more fails with
    ERR_OUT_OF_MEMORY, the handle keeps its scene, and the next frame under a
    larger cap or none renders exactly."""
    s = spr.Scene.generate(spr.SCENE_MIXED, seed=58, width=320, height=240, n_paths=300, n_large=12)
    ref = oracle.run(s, 320, 240, samples=32)
    with spr.VGRasterizer(320, 240, samples=32) as r:
        r.add_vg(s)
        held = r.frame_stats()["device_bytes"]
        r.set_memory_limit(held + 4096)
        with pytest.raises(spr.SprError) as e:
            r.rasterize()
        assert e.value.status == spr.ERR_OUT_OF_MEMORY
        assert r.frame_stats()["device_bytes"] <= held + 4096
        with pytest.raises(spr.SprError):
            r.read_image()  # no valid frame
        r.set_memory_limit(0)
        r.rasterize()
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        need = r.frame_stats()["device_bytes"]
        r.set_memory_limit(need)  # enough for this frame: renders under the cap
        r.rasterize()
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        assert r.frame_stats()["device_bytes"] <= need
        with pytest.raises(spr.SprError):
            r.set_memory_limit(-1)


def test_benchmark_scene_band():
    """A 2048x256 band (rows 896-1151) of the benchmark scene, rendered as the
    CPU arm renders its steps (all 20,000 paths moved by the band's
    transform), exact."""
    import bench

    scene = bench.make_scene()
    y0, bh = 896, bench.BAND_ROWS
    counts, diff = check_parity(scene, 2048, bh, samples=32, transform=bench.band_transform(y0))
    assert counts["curve_fragment"] > 100000 and diff == 0


def test_benchmark_scene_full_frame_invariants():
    """The full 2048x2048 benchmark frame: sort order, permutation, draw list."""
    import bench

    scene = bench.make_scene()
    with spr.VGRasterizer(2048, 2048, samples=32) as r:
        r.add_vg(scene)
        r.rasterize()
        n = r.element_number()
        perm = r.dump("SORT_PERM")
        assert np.array_equal(np.sort(perm), np.arange(n["curve_fragment"], dtype=np.int32))
        keys = r.dump("SORT_KEY")
        pid = r.dump("FRAG_PID") & 0x3FFFFFFF
        assert np.all(np.diff(pid.astype(np.int64)) >= 0)
        same = pid[1:] == pid[:-1]
        assert np.all(keys[1:][same] >= keys[:-1][same])  # signed order within a path
        assert len(r.dump("DRAW_LIST")) == 4 * (n["merged_fragment"] + n["span"])
        a = r.read_image().copy()
        r.rasterize()
        assert np.array_equal(a, r.read_image())


def test_shared_vertex_ranges():
    """Curves that share vertices (curve i uses vertices i and i + 1): the
    reference orients curves in place, in curve order, so a reversed curve
    moves its neighbour's end point too; such scenes take the host upload
    path and must match the oracle bit for bit, as must the same polygons
    written with a vertex range per curve (the device upload path)."""
    rng = np.random.default_rng(57)
    polys = []
    for p in range(12):
        n = int(rng.integers(3, 9))
        c = rng.uniform(20, 180, 2)
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        r = rng.uniform(5, 40, n)
        pts = np.c_[c[0] + r * np.cos(ang), c[1] + r * np.sin(ang)].astype(np.float32)
        polys.append(np.vstack([pts, pts[:1]]))
    vert, vpid, cvp, cpid = [], [], [], []
    vert2, vpid2, cvp2, cpid2 = [], [], [], []
    for p, pts in enumerate(polys):
        base = sum(len(x) for x in vert)
        vert.append(pts)
        vpid += [p] * len(pts)
        for i in range(len(pts) - 1):
            cvp.append(base + i)  # shared end points
            cpid.append(p)
            cvp2.append(sum(len(x) for x in vert2))
            vert2.append(pts[i:i + 2])
            vpid2 += [p, p]
            cpid2.append(p)
    rule = rng.integers(0, 2, 12).astype(np.uint8)
    fill = (rng.integers(0, 2**24, 12) | (rng.integers(128, 256, 12) << 24)).astype(np.uint32)
    types = np.full(len(cvp), spr.CURVE_LINEAR, np.uint8)
    w = np.zeros(len(cvp), np.float32)
    shared = spr.Scene(np.vstack(vert), np.array(vpid, np.uint32), np.array(cvp, np.uint32), types,
                       np.array(cpid, np.uint32), w, rule, fill)
    disjoint = spr.Scene(np.vstack(vert2), np.array(vpid2, np.uint32), np.array(cvp2, np.uint32), types,
                         np.array(cpid2, np.uint32), w, rule, fill)
    check_parity(shared, 200, 200, samples=32)
    check_parity(disjoint, 200, 200, samples=32)


@pytest.mark.parametrize("name", ["random", "cubics", "mixed", "oddsize", "handmade"])
def test_256_samples(name):
    """256 samples per pixel, rendered as 8 passes of 32 (each with its own
    samples and geometry shift): the last pass's stages and the image (the
    exact mean over all 256 samples) match the oracle's passes."""
    scene, W, H, tf, _, _ = load_golden(name)
    check_parity(scene, W, H, samples=256, transform=tf)


@pytest.mark.parametrize("srgb", [True, False])
def test_256_samples_modes_and_limits(srgb):
    scene = spr.Scene.generate(spr.SCENE_MIXED, seed=23, width=160, height=120, n_paths=30, n_large=3,
                               with_rational=True)
    check_parity(scene, 160, 120, 256, True, srgb)
    with render(scene, 160, 120, 256, True, srgb) as r:
        st = r.frame_stats()
        assert st["host_syncs"] == 8 * 2  # two size reads per pass
        r.set_samples(32)  # and back: the tables follow the sample count
        r.rasterize()
        assert np.array_equal(r.read_image().reshape(-1),
                              oracle.run(scene, 160, 120, samples=32, srgb=srgb)["IMAGE"])
        r.set_multisample_output(False)
        with pytest.raises(spr.SprError):
            r.set_samples(256)
    with pytest.raises(spr.SprError):
        spr.VGRasterizer(64, 64, samples=256, ms_output=False)
    with spr.VGRasterizer(64, 64, samples=256) as r:
        with pytest.raises(spr.SprError):
            r.set_multisample_output(False)
    with spr.Batch(ms_output=False) as b:
        with pytest.raises(spr.SprError):
            b.set_scenes([(scene, 64, 64, 256)])


def concat(a, b):
    """Scene a's paths followed by scene b's."""
    P, V = a.n_paths, a.n_vertices
    return spr.Scene(np.concatenate([a.vertex, b.vertex]), np.concatenate([a.vertex_path_id, b.vertex_path_id + P]),
                     np.concatenate([a.curve_vertex_pos, b.curve_vertex_pos + V]),
                     np.concatenate([a.curve_type, b.curve_type]),
                     np.concatenate([a.curve_path_id, b.curve_path_id + P]),
                     np.concatenate([a.curve_arc_w, b.curve_arc_w]),
                     np.concatenate([a.path_fill_rule, b.path_fill_rule]),
                     np.concatenate([a.path_fill_rgba, b.path_fill_rgba]))


def test_long_path_segments():
    """The fragment sort on long paths, against the oracle's stable sort with
    every stage exact: a frame of a few paths of 145k-338k entries each (the
    device-wide radix sort), and 1,100 short paths with three of 29k-36k
    entries (one block per path; the long ones chunked through global
    memory)."""
    for W in (1024, 2048):
        sc = spr.Scene.generate(spr.SCENE_RANDOM, seed=77, width=W, height=W, n_paths=4, seg_min=300, seg_max=400)
        counts, _ = check_parity(sc, W, W, samples=8)
        assert counts["curve_fragment"] > 500_000
    many = spr.Scene.generate(spr.SCENE_MIXED, seed=91, width=1024, height=1024, n_paths=1100, n_large=12)
    longp = spr.Scene.generate(spr.SCENE_RANDOM, seed=5, width=1024, height=1024, n_paths=3, seg_min=60, seg_max=90)
    sc = concat(many, longp)
    counts, _ = check_parity(sc, 1024, 1024, samples=8)
    assert counts["path"] > 1024 and counts["curve_fragment"] > 550_000


def test_tuning_changes_speed_not_results():
    """Every launch choice (fragment sort, emission order, resolve blocks per
    SM) gives the same image and stages; spr_autotune keeps one no slower
    than the built-in rules."""
    W = H = 384
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=17, width=W, height=H, n_paths=1500, n_large=6,
                            with_rational=True)
    with render(sc, W, H, 32) as r:
        ref = r.read_image().copy()
        perm = r.dump("SORT_PERM").copy()
        for sort in (0, 1):
            for emit in (0, 1):
                for bps in (1, 3):
                    r.set_tuning(sort, emit, bps)
                    r.rasterize()
                    assert np.array_equal(r.read_image(), ref), (sort, emit, bps)
                    assert np.array_equal(r.dump("SORT_PERM"), perm)
        for bw in (64, 32, 8, 16):
            r.set_tuning(bin_width=bw)
            r.rasterize()
            assert np.array_equal(r.read_image(), ref), bw
        t = r.autotune(frames=2)
        assert t["sort"] in (-1, 0, 1) and t["emit_order"] in (-1, 0, 1) and t["resolve_bps"] in (0, 2, 3)
        assert t["bin_width"] in (0, 64, 32, 16, 8)
        assert 0 < t["frame_ms"] <= t["default_ms"]
        r.rasterize()
        assert np.array_equal(r.read_image(), ref)
        with pytest.raises(spr.SprError):
            r.set_tuning(2, 0, 0)
        with pytest.raises(spr.SprError):
            r.set_tuning(bin_width=48)


@pytest.mark.parametrize("bin_width", [64, 32, 16, 8])
@pytest.mark.parametrize("samples,ms,srgb", [(8, True, True), (32, True, False), (16, False, True), (256, True, True)])
def test_resolve_tiles(bin_width, samples, ms, srgb):
    """Resolve tiles of 64 x 1, 32 x 2, 16 x 4 and 8 x 8 cells
    (tile width x band height): the image exact against the oracle on an
    odd-sized viewport (partial tiles and bands at the right and bottom
    edges)."""
    W, H = 173, 131
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=23, width=W, height=H, n_paths=80, n_large=5, with_affine=True)
    ref = oracle.run(sc, W, H, samples=samples, ms_output=ms, srgb=srgb)
    r = spr.VGRasterizer(W, H, samples=samples, ms_output=ms, srgb=srgb)
    with r:
        r.set_tuning(bin_width=bin_width)
        r.add_vg(sc)
        r.rasterize()
        diff = np.abs(r.read_image().astype(np.int16) - ref["IMAGE"].reshape(H, W, 4).astype(np.int16)).max()
        assert diff <= IMAGE_TOL


def test_random_configurations():
    """Seeded sweep: scene kind, size, path count, sample count (8/16/32/256),
    output modes, rational segments, per-path affines and a random affine or
    projective input transform, every stage and the image exact."""
    rng = np.random.default_rng(2026)
    kinds = [spr.SCENE_RANDOM, spr.SCENE_MIXED, spr.SCENE_CUBICS, spr.SCENE_LOCAL]
    for case in range(24):
        W, H = int(rng.integers(16, 300)), int(rng.integers(16, 300))
        kind = kinds[case % 4]
        samples = [8, 16, 32, 256][int(rng.integers(0, 4))]
        ms = bool(rng.integers(0, 2)) or samples == 256
        srgb = bool(rng.integers(0, 2))
        sc = spr.Scene.generate(kind, seed=int(rng.integers(1, 1 << 30)), width=W, height=H,
                                n_paths=int(rng.integers(1, 80)), n_large=int(rng.integers(0, 3)),
                                seg_min=3, seg_max=int(rng.integers(4, 24)), with_rational=bool(rng.integers(0, 2)),
                                with_affine=bool(rng.integers(0, 2)))
        tf = None
        if rng.integers(0, 2):
            tf = np.eye(4, dtype=np.float32)
            tf[0, :2] = rng.uniform(-1.3, 1.3, 2)
            tf[1, :2] = rng.uniform(-1.3, 1.3, 2)
            tf[0, 3], tf[1, 3] = rng.uniform(-20, 60, 2)
            if rng.integers(0, 3) == 0:
                tf[3, :2] = rng.uniform(-4e-4, 4e-4, 2)
        check_parity(sc, W, H, samples, ms, srgb, tf)


def drop_curves(sc, keep):
    """The scene with only the curves in `keep` (their vertices stay, so some
    vertices belong to no curve and some contours are left open)."""
    keep = np.asarray(keep, bool)
    out = sc.copy()
    for f in ("curve_vertex_pos", "curve_type", "curve_path_id", "curve_arc_w"):
        setattr(out, f, np.ascontiguousarray(getattr(sc, f)[keep]))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_open_contours_and_alpha_zero_fills(seed):
    """Open contours (winding sums left nonzero on their rows, carried into
    later paths as the reference's scan does), orphaned vertices and fill
    values of alpha 0 that are not 0: every stage bit-exact against the
    oracle, and batched renders equal to the single renders."""
    rng = np.random.default_rng(seed)
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=40 + seed, width=200, height=150, n_paths=30,
                            with_rational=True, with_affine=seed == 2)
    sc = drop_curves(sc, rng.random(sc.n_curves) > 0.08)
    sc.path_fill_rgba = np.where(rng.random(sc.n_paths) < 0.2, rng.integers(1, 0x01000000, sc.n_paths),
                                 sc.path_fill_rgba).astype(np.uint32)
    plain = spr.Scene.generate(spr.SCENE_MIXED, seed=50 + seed, width=120, height=90, n_paths=15)
    for smp, ms in ((8, True), (32, True), (32, False)):
        check_parity(sc, 200, 150, samples=smp, ms=ms)
    items = [(sc, 200, 150, 32), (plain, 120, 90, 32), (sc, 200, 150, 8), (plain, 120, 90, 8)]
    with spr.Batch() as b:
        b.set_scenes(items)
        b.render()
        for i, (s, W, H, smp) in enumerate(items):
            with render(s, W, H, smp) as r:
                assert np.array_equal(b.read_image(i), r.read_image()), i


@pytest.mark.parametrize("samples,ms,srgb", [(8, True, True), (16, True, False), (32, True, True), (32, False, True),
                                             (8, False, False)])
def test_opaque_fills(samples, ms, srgb):
    """Opaque fills (alpha 255) mixed with translucent ones, over deep
    overlap: every stage and the image exact against the oracle."""
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=91, width=160, height=120, n_paths=60, n_large=6)
    rng = np.random.default_rng(4)
    opaque = rng.random(sc.n_paths) < 0.7
    sc.path_fill_rgba = np.where(opaque, sc.path_fill_rgba | 0xFF000000, sc.path_fill_rgba).astype(np.uint32)
    check_parity(sc, 160, 120, samples=samples, ms=ms, srgb=srgb)


def stacked_contours(copies, reverse_every=0):
    """One path per fill rule, each of `copies` slightly shifted copies of
    the same 9-gon (every `reverse_every`-th copy reversed when set): the
    boundary cells hold groups of up to `copies` fragments and the windings
    reach +-copies."""
    vert, vpid, cvp, ctype, cpid, cw = [], [], [], [], [], []
    ang = np.linspace(0, 2 * np.pi, 9, endpoint=False)
    for pid in range(2):
        cx, cy = 40.0 + 70.0 * pid, 40.0
        for k in range(copies):
            pts = [(cx + 27.3 * np.cos(a) + 0.013 * k, cy + 25.1 * np.sin(a) - 0.007 * k) for a in ang]
            if reverse_every and k % reverse_every == 0:
                pts = pts[::-1]
            for i in range(len(pts)):
                cvp.append(len(vert))
                ctype.append(spr.CURVE_LINEAR)
                cpid.append(pid)
                cw.append(-1.0)
                for p in (pts[i], pts[(i + 1) % len(pts)]):
                    vert.append(p)
                    vpid.append(pid)
    return spr.Scene(np.array(vert, np.float32), vpid, cvp, ctype, cpid, cw, [0, 1],
                     [0xC04080F0, 0xB0F08040])


@pytest.mark.parametrize("copies,reverse_every", [(100, 0), (127, 0), (128, 0), (200, 0), (300, 7)])
@pytest.mark.parametrize("samples", [8, 32])
def test_high_winding_numbers(copies, reverse_every, samples):
    """Merged masks where the windings leave the int8 range (groups of up to
    300 fragments in one cell): the bit-sliced counters and the packed 8-bit
    counters they fall back to, exact against the oracle."""
    check_parity(stacked_contours(copies, reverse_every), 150, 80, samples=samples)


def test_built_in_tile_follows_span_lengths():
    """The built-in resolve tile: 16 x 4 cells for scenes of short spans
    (glyph-like paths), 64 x 1 for long spans (large paths), chosen by the
    sized first frame (which bins again if its tile was the other one):
    later frames read nothing back, and the images stay exact."""
    small = spr.Scene.generate(spr.SCENE_MIXED, seed=29, width=256, height=256, n_paths=400)
    large = spr.Scene.generate(spr.SCENE_CUBICS, seed=30, width=256, height=256, n_paths=12, seg_min=16, seg_max=32)
    for sc in (small, large):
        ref = oracle.run(sc, 256, 256, samples=8)
        with render(sc, 256, 256, 8) as r:
            for _ in range(3):
                r.rasterize()
                assert r.frame_stats()["host_syncs"] == 0  # (the first frame chose the tile)
                assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
