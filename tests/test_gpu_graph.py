"""Graph replay of unchanged frames (spr_set_graph_replay): the captured
launch sequence must give the bytes of a normal render, read nothing back,
and be dropped by every change to the handle."""
import numpy as np
import pytest

import spr

pytestmark = pytest.mark.gpu


def plain(scene, W, H, samples, tf=None):
    with spr.VGRasterizer(W, H, samples=samples) as r:
        if tf is not None:
            r.set_input_transform(tf)
        r.add_vg(scene)
        r.rasterize()
        return r.read_image().copy(), r.dump("DRAW_LIST").copy()


def test_replay_matches_and_skips_host_reads():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=81, width=512, height=384, n_paths=400, n_large=30,
                            with_affine=True)
    ref, ref_draw = plain(sc, 512, 384, 32)
    with spr.VGRasterizer(512, 384, samples=32) as r:
        r.set_graph_replay(True)
        r.add_vg(sc)
        r.rasterize()  # renders normally, then captures
        assert r.graph_replays() == 0 and r.frame_stats()["host_syncs"] == 2  # the sized first frame
        assert np.array_equal(r.read_image(), ref)
        for k in range(3):
            r.rasterize()
            assert r.graph_replays() == k + 1 and r.frame_stats()["host_syncs"] == 0
            assert np.array_equal(r.read_image(), ref)
        assert np.array_equal(r.dump("DRAW_LIST"), ref_draw)


def test_changes_drop_the_graph():
    a = spr.Scene.generate(spr.SCENE_RANDOM, seed=82, width=256, height=256, n_paths=40, seg_min=6, seg_max=20)
    b = spr.Scene.generate(spr.SCENE_CUBICS, seed=83, width=256, height=256, n_paths=60, seg_min=8, seg_max=24)
    tf = np.eye(4, dtype=np.float32)
    tf[0, 0], tf[0, 3] = 0.8, 12.0
    with spr.VGRasterizer(256, 256, samples=8) as r:
        r.set_graph_replay(True)
        r.add_vg(a)
        r.rasterize()
        r.rasterize()
        assert np.array_equal(r.read_image(), plain(a, 256, 256, 8)[0])
        r.set_input_transform(tf)
        r.rasterize()
        r.rasterize()
        assert np.array_equal(r.read_image(), plain(a, 256, 256, 8, tf)[0])
        r.add_vg(b)
        r.rasterize()
        r.rasterize()
        assert np.array_equal(r.read_image(), plain(b, 256, 256, 8, tf)[0])
        r.set_samples(32)
        r.rasterize()
        r.rasterize()
        assert np.array_equal(r.read_image(), plain(b, 256, 256, 32, tf)[0])
        r.resize_output_buffer(200, 160)
        r.rasterize()
        r.rasterize()
        assert np.array_equal(r.read_image(), plain(b, 200, 160, 32, tf)[0])
        n = r.graph_replays()
        assert n >= 4
        r.set_graph_replay(False)
        r.rasterize()
        assert r.graph_replays() == n and r.frame_stats()["host_syncs"] == 0  # sized already


def test_batch_replay():
    items = []
    for i, (W, H, smp) in enumerate([(128, 96, 8), (300, 200, 32), (64, 64, 16), (257, 129, 32)]):
        sc = spr.Scene.generate(spr.SCENE_LOCAL, seed=90 + i, width=W, height=H, n_paths=50 + 40 * i, seg_min=8,
                                seg_max=24)
        items.append((sc, W, H, smp))
    with spr.Batch() as b:
        b.set_graph_replay(True)
        b.set_scenes(items)
        for _ in range(4):
            b.render()
        for i, (sc, W, H, smp) in enumerate(items):
            assert np.array_equal(b.read_image(i), plain(sc, W, H, smp)[0])
        assert b.frame_stats()["host_syncs"] == 0
