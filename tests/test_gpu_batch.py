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
        assert st["host_syncs"] == 9 and st["kernel_launches"] > 0  # 3 per sample-count group


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
