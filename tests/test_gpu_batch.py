"""Batched rendering (spr_batch_*): every scene of a batch must come out
byte-identical to the same scene rendered alone by a single-scene handle
(which the parity suite checks against the oracle), whatever the mix of
sizes, sample counts, transforms and empty scenes in the batch."""
import numpy as np
import pytest

import oracle
import spr

pytestmark = pytest.mark.gpu


def single(scene, W, H, samples, tf=None, ms=True, srgb=True):
    with spr.VGRasterizer(W, H, samples=samples, ms_output=ms, srgb=srgb) as r:
        if tf is not None:
            r.set_input_transform(tf)
        r.add_vg(scene)
        r.rasterize()
        return r.read_image().copy(), r.element_number()


def uneven_items(seed, n, sizes=((64, 64), (97, 33), (256, 256), (300, 130), (512, 512), (1, 1))):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n):
        W, H = sizes[i % len(sizes)]
        samples = (8, 16, 32)[i % 3]
        kind = (spr.SCENE_LOCAL, spr.SCENE_RANDOM, spr.SCENE_MIXED)[i % 3]
        n_paths = int(np.exp(rng.uniform(np.log(3), np.log(120))))
        sc = spr.Scene.generate(kind, seed=1000 + i, width=W, height=H, n_paths=n_paths, n_large=2,
                                seg_min=8, seg_max=32, with_rational=True, with_affine=(i % 4 == 1))
        tf = None
        if i % 5 == 2:
            tf = np.eye(4, dtype=np.float32)
            tf[0, 0], tf[1, 1], tf[0, 3], tf[1, 3] = 0.7, 1.2, 5.0, -3.0
        items.append((sc, W, H, samples, tf))
    return items


@pytest.mark.parametrize("ms,srgb", [(True, True), (False, False)])
def test_batch_matches_single_scene_renders(ms, srgb):
    items = uneven_items(7, 14)
    items.append((spr.Scene(np.zeros((0, 2), np.float32), [], [], [], [], [], [], []), 40, 30, 8, None))
    with spr.Batch(ms_output=ms, srgb=srgb) as b:
        b.set_scenes(items)
        b.render()
        total = {k: 0 for k in ("path", "curve", "vertex", "curve_fragment", "merged_fragment", "span")}
        for i, (sc, W, H, smp, tf) in enumerate(items):
            exp, counts = single(sc, W, H, smp, tf, ms, srgb)
            got = b.read_image(i)
            assert got.shape == (H, W, 4)
            assert np.array_equal(got, exp), f"scene {i} ({W}x{H}, {smp} spp)"
            for k in total:
                total[k] += counts[k]
        assert b.element_number() == total
        st = b.frame_stats()
        assert st["host_syncs"] == 6 and st["kernel_launches"] > 0  # 2 per sample-count group (first frame)


def test_batch_against_oracle_and_rerender():
    items = uneven_items(11, 6, sizes=((128, 96), (200, 200), (64, 160)))
    with spr.Batch() as b:
        b.set_scenes(items)
        b.render()
        first = [b.read_image(i).copy() for i in range(len(items))]
        b.render()
        for i, (sc, W, H, smp, tf) in enumerate(items):
            assert np.array_equal(b.read_image(i), first[i])
            ref = oracle.run(sc, W, H, samples=smp, transform=tf)
            assert np.array_equal(first[i].reshape(-1), ref["IMAGE"]), f"scene {i}"
        # a new set replaces the old one
        b.set_scenes(items[:2])
        b.render()
        assert np.array_equal(b.read_image(1), first[1])
        with pytest.raises(spr.SprError):
            b.read_image(2)


def test_batch_rejects_bad_input():
    sc = spr.Scene.generate(spr.SCENE_RANDOM, seed=3, width=64, height=64, n_paths=4, seg_min=3, seg_max=5)
    with spr.Batch() as b:
        with pytest.raises(spr.SprError) as e:
            b.render()
        assert e.value.status == spr.ERR_NO_SCENE
        for bad in [(sc, 0, 64, 8), (sc, 64, 5000, 8), (sc, 64, 64, 12)]:
            with pytest.raises(spr.SprError) as e:
                b.set_scenes([bad])
            assert e.value.status == spr.ERR_INVALID_ARG
        broken = sc.copy()
        broken.curve_type[0] = 9
        with pytest.raises(spr.SprError) as e:
            b.set_scenes([(sc, 64, 64, 8), (broken, 64, 64, 8)])
        assert e.value.status == spr.ERR_INVALID_SCENE
        b.set_scenes([(sc, 64, 64, 8)])
        b.render()
        assert np.array_equal(b.read_image(0), single(sc, 64, 64, 8)[0])


def test_batch_with_256_samples():
    """256-sample scenes in a batch (their own group, 8 passes of 32) next to
    8- and 32-sample ones: each scene byte-identical to its single render."""
    items = []
    for i, (W, H, smp) in enumerate([(96, 80, 256), (128, 64, 32), (50, 70, 256), (64, 64, 8)]):
        sc = spr.Scene.generate(spr.SCENE_MIXED, seed=300 + i, width=W, height=H, n_paths=12, n_large=2,
                                with_rational=True)
        items.append((sc, W, H, smp))
    with spr.Batch() as b:
        b.set_scenes(items)
        b.render()
        for i, (sc, W, H, smp) in enumerate(items):
            exp, _ = single(sc, W, H, smp)
            assert np.array_equal(b.read_image(i), exp), f"scene {i} ({smp} spp)"


@pytest.mark.parametrize("srgb", [True, False])
def test_batch_with_gradient_paints(srgb):
    """Loaded documents with gradient paints (an RVG and an SVG document, the
    SVG one twice with different sizes) batched with plain scenes, one with
    alpha-0 fill values that must not pick up another scene's gradient
    entries: every image byte-identical to its single-scene render."""
    from test_rvg import DOC as RVG
    from test_svg import DOC as SVG
    rvg, ri = spr.Scene.parse_rvg(RVG, srgb_ramps=srgb)
    svg, si = spr.Scene.parse_svg(SVG, srgb_ramps=srgb)
    plain = spr.Scene.generate(spr.SCENE_MIXED, seed=4, width=128, height=96, n_paths=20)
    junk = plain.copy()
    junk.path_fill_rgba = np.where(np.arange(junk.n_paths) % 2 == 0, np.arange(junk.n_paths) % 5 + 1,
                                   junk.path_fill_rgba).astype(np.uint32)
    items = [(rvg, ri["width"], ri["height"], 32, None), (plain, 128, 96, 8, None),
             (svg, si["width"], si["height"], 8, None), (junk, 128, 96, 32, None),
             (svg, si["width"], si["height"], 32, None)]
    with spr.Batch(srgb=srgb) as b:
        b.set_scenes(items)
        b.render()
        for i, (sc, W, H, smp, tf) in enumerate(items):
            exp, _ = single(sc, W, H, smp, tf, True, srgb)
            assert np.array_equal(b.read_image(i), exp), i


def test_open_contour_does_not_reach_later_scenes():
    """A contour left open (Z adds no segment in RVG documents) leaves a
    winding sum on its rows that the single-scene scan carries into later
    paths of its scene; in a batch it must not reach the next scenes."""
    L = spr.CURVE_LINEAR
    opened = spr.Scene(np.array([[5, 5], [40, 5], [40, 5], [40, 40]], np.float32), [0] * 4, [0, 2], [L, L],
                       [0, 0], [-1, -1], [0], [0xFF0000FF])
    plain = spr.Scene.generate(spr.SCENE_MIXED, seed=9, width=96, height=64, n_paths=12)
    items = [(opened, 64, 48, 32, None), (plain, 96, 64, 32, None), (opened, 64, 48, 8, None),
             (plain, 96, 64, 8, None)]
    with spr.Batch() as b:
        b.set_scenes(items)
        b.render()
        for i, (sc, W, H, smp, tf) in enumerate(items):
            exp, _ = single(sc, W, H, smp, tf)
            assert np.array_equal(b.read_image(i), exp), i


@pytest.mark.parametrize("ms,srgb", [(True, True), (False, False)])
def test_loaded_documents_across_modes(ms, srgb):
    """Gradient-painted documents at every sample count of the mode (256 with
    multisample output only), alone against the oracle and batched against
    their single renders; and a graph-replayed single frame equal to the
    eager one."""
    from test_rvg import DOC as RVG
    from test_svg import DOC as SVG
    rvg, ri = spr.Scene.parse_rvg(RVG, srgb_ramps=srgb)
    svg, si = spr.Scene.parse_svg(SVG, srgb_ramps=srgb, stroke_to_fill=True)
    counts = (8, 16, 32, 256) if ms else (8, 16, 32)
    items = []
    for smp in counts:
        for sc, info in ((rvg, ri), (svg, si)):
            W, H = info["width"], info["height"]
            exp, _ = single(sc, W, H, smp, None, ms, srgb)
            ref = oracle.run(sc, W, H, samples=smp, ms_output=ms, srgb=srgb)["IMAGE"]
            assert np.array_equal(exp.reshape(-1), ref), (smp, W)
            items.append((sc, W, H, smp, None, exp))
    with spr.Batch(ms_output=ms, srgb=srgb) as b:
        b.set_scenes([it[:5] for it in items])
        b.render()
        for i, it in enumerate(items):
            assert np.array_equal(b.read_image(i), it[5]), i
    W, H = ri["width"], ri["height"]
    with spr.VGRasterizer(W, H, samples=32, ms_output=ms, srgb=srgb) as r:
        r.add_vg(rvg)
        r.set_graph_replay(True)
        for _ in range(3):
            r.rasterize()
        assert r.graph_replays() >= 1
        assert np.array_equal(r.read_image(), items[2 * counts.index(32)][5])
