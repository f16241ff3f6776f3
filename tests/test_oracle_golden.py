"""The CPU oracle against the reference's own code.

Fixtures in tests/golden/ were produced by tests/golden/make_goldens.py from
the reference's intersection kernels (ras_cut.h k_make_intersection_0/1), its
mask helpers (ras_qm_mask.h makeTable, fetchPixelTable, fetchVerticalTable,
fetchVerticalTable2) and its sample pattern (ras_qm_mask.cu
vg_sample_position), all compiled from the reference sources.  Where the
reference tree is mounted, the same code is also run live on fresh scenes.
"""
import hashlib
import json
import pathlib

import numpy as np
import pytest

import oracle
import spr

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def load_scene(path):
    d = np.load(path)
    fields = {f: d[f] for f in spr.Scene.FIELDS if f in d.files}
    scene = spr.Scene(**fields)
    tf = d["transform"] if bool(d["has_transform"]) else None
    return scene, int(d["width"]), int(d["height"]), tf, d["ref_counts"], d["ref_entries"]


@pytest.mark.parametrize("samples", [8, 32])
def test_sample_positions_match_reference(samples):
    ref = json.loads((GOLDEN / "sample_positions.json").read_text())[str(samples)]
    cell = oracle.sample_positions(samples)
    pixel0 = (cell[:samples] * 2).astype(np.float32)  # cell coords of pixel 0 -> pixel coords
    assert pixel0.view(np.uint32).reshape(-1).tolist() == ref


@pytest.mark.parametrize("samples", [8, 32])
def test_mask_table_matches_reference(samples):
    digest = json.loads((GOLDEN / "mask_tables.json").read_text())[str(samples)]
    t = oracle.mask_table(samples)
    assert hashlib.sha256(t.reshape(-1).tobytes() if samples == 32 else t[:, 0].tobytes()).hexdigest() == digest


@pytest.mark.parametrize("samples", [8, 32])
def test_mask_helpers_match_reference(samples):
    v = np.load(GOLDEN / "mask_vectors.npz")
    w = samples // 8
    for p, exp in zip(v[f"fetch{samples}_in"], v[f"fetch{samples}_out"]):
        assert np.array_equal(oracle.fetch_pixel_table(samples, p[:2], p[2:]), exp[:w])
    for (y0, y1), e1, e2 in zip(v[f"vert{samples}_in"], v[f"vert{samples}_out"], v[f"vert2_{samples}_out"]):
        assert np.array_equal(oracle.vertical_mask(samples, y0), e1[:w])
        assert np.array_equal(oracle.vertical_mask2(samples, y0, y1), e2[:w])


def test_sixteen_sample_pattern():
    """16 samples per pixel (an extension; the reference builds 8 and 32):
    the 8-sample construction on 16 rows, row i at (2i+1)/32 and column =
    bit-reversed i (own bit length) scaled to 16 columns, so every row and
    every column holds exactly one sample."""
    def column(i, n):
        b = f"{i:b}" if i else ""
        return int(int(b[::-1], 2) / (1 << len(b)) * n) if i else 0

    cell = oracle.sample_positions(16)
    p = (cell[:16] * 2).astype(np.float64)
    assert np.allclose(p[:, 1], (2 * np.arange(16) + 1) / 32)
    cols = np.round(p[:, 0] * 16 - 0.5).astype(int)
    assert cols.tolist() == [column(i, 16) for i in range(16)]
    assert sorted(cols) == list(range(16))
    p8 = (oracle.sample_positions(8)[:8] * 2).astype(np.float64)  # same rule, pinned against the reference
    assert np.round(p8[:, 0] * 8 - 0.5).astype(int).tolist() == [column(i, 8) for i in range(8)]
    for k in range(4):  # pixel k of the cell is offset by (k >> 1, k & 1) and halved
        q = cell[16 * k:16 * (k + 1)] * 2 - np.array([k >> 1, k & 1], np.float32)
        assert np.allclose(q, p, atol=1e-6)


def test_sixteen_sample_masks():
    """Vertical masks stack the 32 sample rows of a cell column in one word
    (both columns equal); table fetches give two words."""
    assert oracle.vertical_mask(16, 0.0).tolist() == [0, 0]
    assert oracle.vertical_mask(16, 1.0).tolist() == [0xFFFFFFFF] * 2
    assert oracle.vertical_mask(16, 0.5).tolist() == [0xFFFF] * 2
    assert oracle.vertical_mask2(16, 0.25, 0.75).tolist() == [0x00FFFF00] * 2
    assert oracle.mask_table(16).size == 65536 * 2


@pytest.mark.parametrize("samples", [8, 16, 32])
def test_table_lattice_quality(samples):
    """The reference's (disabled) testFetchTable check: table fetch against the
    exact half-plane test for every lattice segment; it reports segments with
    4 or more wrong bits.  The shared table keeps those rare."""
    h = oracle.fetch_table_selftest(samples, 33)
    assert h.sum() == 33 ** 4 - 33 ** 3  # every pair with y0 != y1
    assert h[5 if samples != 16 else 6:].sum() == 0  # 16 spp: 32 rows share one 256x256 table
    assert h[4:].sum() / h.sum() < 0.005


@pytest.mark.parametrize("name", ["random", "cubics", "mixed", "oddsize", "handmade"])
def test_intersections_match_reference(name):
    scene, W, H, tf, counts, entries = load_scene(GOLDEN / f"scene_{name}.npz")
    r = oracle.run(scene, W, H, samples=8, transform=tf, stop_after=spr.STAGE["INTERSECTION"])
    assert np.array_equal(r["CURVE_COUNT"], counts)
    assert np.array_equal(r["INTERSECTION"].reshape(-1, 2), entries)


def test_srgb_tables_consistent():
    dec, th, bins = oracle.srgb_tables()
    assert np.all(np.diff(dec) > 0) and np.all(np.diff(th) > 0)
    assert dec[0] == 0.0 and dec[255] == 1.0
    # every 8-bit code decodes to a value between its two thresholds
    assert np.all(dec[1:] >= th) and np.all(dec[:-1] < th)


@pytest.mark.skipif(not oracle.have_ref(), reason="reference tree not mounted here")
@pytest.mark.parametrize("kind,size,seed", [(spr.SCENE_RANDOM, 311, 1), (spr.SCENE_MIXED, 512, 2),
                                            (spr.SCENE_CUBICS, 400, 3), (spr.SCENE_RANDOM, 64, 4)])
def test_intersections_live_reference(kind, size, seed):
    scene = spr.Scene.generate(kind, seed=seed, width=size, height=size,
                               n_paths={0: 20, 1: 150, 2: 12}[kind], n_large=8,
                               seg_min=8 if kind != spr.SCENE_CUBICS else 16,
                               seg_max=24 if kind != spr.SCENE_CUBICS else 40,
                               with_rational=True, with_affine=kind == spr.SCENE_MIXED)
    r = oracle.run(scene, size, size, samples=32, stop_after=spr.STAGE["INTERSECTION"])
    counts, entries = oracle.ref_intersections(scene, r["TVERTEX"].reshape(-1, 2), r["PATH_VISIBLE"], size, size)
    assert np.array_equal(r["CURVE_COUNT"], counts)
    assert np.array_equal(r["INTERSECTION"].reshape(-1, 2), entries)


def test_256_sample_pattern_and_passes():
    """256 samples per pixel (an extension): the 8-sample construction on 256
    rows, row i at (2i+1)/512 and column = bit-reversed i on 8 bits.  It is
    rendered as 8 passes of 32 samples: pass g holds rows 8j + g on the
    32-sample rows (2j+1)/64, and moving those rows down by (2g-7)/512 (the
    pass moves the geometry up by as much) gives back exactly the pattern's
    rows; the union of the passes is the whole pattern."""
    cell = oracle.sample_positions(256)
    p = (cell[:256] * 2).astype(np.float64)
    assert np.allclose(p[:, 1], (2 * np.arange(256) + 1) / 512)
    cols = np.round(p[:, 0] * 256 - 0.5).astype(int)
    rev8 = [int(f"{i:08b}"[::-1], 2) for i in range(256)]
    assert cols.tolist() == rev8 and sorted(cols) == list(range(256))
    union = []
    for g in range(8):
        q = oracle.pass_samples_256(g).astype(np.float64)
        assert np.allclose(q[:, 1], (2 * np.arange(32) + 1) / 64)
        assert np.array_equal(q[:, 0], p[8 * np.arange(32) + g, 0])
        union.append(np.c_[q[:, 0], q[:, 1] + (2 * g - 7) / 512])
    union = np.concatenate(union)
    union = union[np.lexsort((union[:, 0], union[:, 1]))]
    assert np.allclose(union, p, atol=1e-9)


def test_256_pass_tables_and_frame():
    """Each pass has its own half-plane table (the 32-sample construction over
    that pass's samples).  A 256-sample frame averages all 256 samples: a
    black square with edges inside pixels, on white without sRGB, gives edge
    pixels whose red channel is the share of the 256 pattern's samples
    outside the square."""
    t = [oracle.pass_mask_table_256(g) for g in range(8)]
    assert all(x.shape == (65536, 4) for x in t)
    assert not np.array_equal(t[0], t[1])
    W = H = 24
    lo, hi = 4.3, 19.7
    pts = [(lo, lo), (hi, lo), (hi, hi), (lo, hi)]
    vert = np.array([p for i in range(4) for p in (pts[i], pts[(i + 1) % 4])], np.float32)
    sc = spr.Scene(vert, [0] * 8, [0, 2, 4, 6], [spr.CURVE_LINEAR] * 4, [0] * 4, [-1.0] * 4, [0],
                   [0xFF000000])
    img = oracle.run(sc, W, H, samples=256, srgb=False)["IMAGE"].reshape(H, W, 4)
    p = (oracle.sample_positions(256)[:256] * 2).astype(np.float64)
    fx, fy = np.float32(lo) - 4, np.float32(hi) - 19
    inside_l = p[:, 0] > fx          # pixel column 4: right of the left edge
    inside_r = p[:, 0] < fy          # pixel column 19: left of the right edge
    inside_t = p[:, 1] > fx          # pixel row 4: below the top edge

    def red(cover):
        return int((256 - int(cover.sum())) / 256 * 255 + 0.5)

    # within two samples (the half-plane table classifies samples within
    # about 1/256 pixel of an edge approximately); 32 samples land elsewhere
    img32 = oracle.run(sc, W, H, samples=32, srgb=False)["IMAGE"].reshape(H, W, 4)
    for (y, x), cover in (((10, 4), inside_l), ((10, 19), inside_r), ((4, 10), inside_t),
                          ((4, 4), inside_l & inside_t)):
        assert abs(int(img[y, x, 0]) - red(cover)) <= 2, (y, x)
        assert img32[y, x, 0] != img[y, x, 0]
    assert img[10, 10, 0] == 0 and img[1, 1, 0] == 255 and img[10, 10, 3] == 255
    with pytest.raises(spr.SprError):
        oracle.run(sc, W, H, samples=256, ms_output=False)
