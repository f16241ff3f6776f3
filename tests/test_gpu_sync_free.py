"""Frames without host reads: after the first (sized) frame of a scene every
kernel takes its sizes from device memory, so a frame whose geometry changes
needs no read-back; one that outgrows its buffers is rendered again before
its results are read.  Captured frames replay across moved vertices.  The
single-pass scans' waits are bounded: a tile that never publishes makes the
frame fail with ERR_TIMEOUT, and the handle stays usable."""
import numpy as np
import pytest

import oracle
import spr

pytestmark = pytest.mark.gpu


def zoom(s, cx, cy):
    m = np.eye(4, dtype=np.float32)
    m[0, 0] = m[1, 1] = s
    m[0, 3], m[1, 3] = cx, cy
    return m


def far():
    """A transform that leaves the scene outside the viewport (almost no
    entries: the first, sized frame sets small buffers)."""
    m = np.eye(4, dtype=np.float32)
    m[0, 3] = 5000.0
    return m


def test_changing_sizes_without_reads():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=61, width=384, height=320, n_paths=500, n_large=20)
    with spr.VGRasterizer(384, 320, samples=32) as r:
        r.set_input_transform(far())
        r.add_vg(sc)
        r.rasterize()
        assert r.frame_stats()["host_syncs"] == 2 and r.element_number()["curve_fragment"] == 0
        # the scene in view: far more entries than the buffers hold, so the
        # frame is rendered again (sized) when its image is read
        r.set_input_transform(np.eye(4, dtype=np.float32))
        r.rasterize()
        ref = oracle.run(sc, 384, 320, samples=32)
        assert r.frame_stats()["host_syncs"] == 2  # (reading the stats settles the frame: rendered again, sized)
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        assert r.element_number() == ref.counts
        assert np.array_equal(r.dump("DRAW_LIST"), ref["DRAW_LIST"])
        # a small change: fits the grown buffers, no read-back
        tf = zoom(1.02, -3.0, 2.0)
        r.set_input_transform(tf)
        r.rasterize()
        assert r.frame_stats()["host_syncs"] == 0
        ref = oracle.run(sc, 384, 320, samples=32, transform=tf)
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        assert r.element_number() == ref.counts


def test_overflowed_frame_with_changed_inputs_is_an_error():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=62, width=256, height=256, n_paths=300, n_large=10)
    with spr.VGRasterizer(256, 256, samples=8) as r:
        r.set_input_transform(far())
        r.add_vg(sc)
        r.rasterize()
        r.set_input_transform(np.eye(4, dtype=np.float32))
        r.rasterize()  # outgrows the buffers
        r.set_input_transform(far())  # its inputs are gone before it is read
        with pytest.raises(spr.SprError) as e:
            r.read_image()
        assert e.value.status == spr.ERR_CAPACITY_EXCEEDED
        r.set_input_transform(np.eye(4, dtype=np.float32))
        r.rasterize()
        assert np.array_equal(r.read_image().reshape(-1), oracle.run(sc, 256, 256, samples=8)["IMAGE"])


def test_graph_replay_across_moved_vertices():
    """A captured frame replayed after the vertices move on the device (the
    sizes change from frame to frame), against fresh renders."""
    import torch

    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=63, width=320, height=256, n_paths=80, seg_min=8, seg_max=24)
    rng = np.random.default_rng(63)
    with spr.VGRasterizer(320, 256, samples=16) as r:
        r.set_graph_replay(True)
        r.add_vg(sc)
        r.rasterize()
        r.rasterize()
        n0 = r.graph_replays()
        assert n0 >= 1
        sizes = set()
        for k in range(4):
            moved = sc.copy()
            moved.vertex = (sc.vertex + rng.normal(0, 1.5, sc.vertex.shape)).astype(np.float32)
            v = torch.tensor(moved.vertex, device="cuda")
            r.update_vertices(v.data_ptr())
            r.rasterize()
            torch.cuda.synchronize()
            ref = oracle.run(moved, 320, 256, samples=16)
            assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"]), k
            sizes.add(ref.counts["curve_fragment"])
        assert r.graph_replays() == n0 + 4
        assert len(sizes) > 1  # the sizes did change


def test_lookback_wait_gives_up():
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=64, width=512, height=512, n_paths=2000, n_large=10)
    assert sc.n_curves > 3 * 2048  # several tiles in the entry-offset scan
    ref = oracle.run(sc, 512, 512, samples=8)
    with spr.VGRasterizer(512, 512, samples=8) as r:
        r.add_vg(sc)
        r.debug_set_lookback(spin_cap=2000, hold_tile=0)  # tile 0 never publishes: a flag nothing sets
        with pytest.raises(spr.SprError) as e:
            r.rasterize()
            r.read_image()
        assert e.value.status == spr.ERR_TIMEOUT
        r.debug_set_lookback()  # the defaults: the handle renders normally again
        r.rasterize()
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        r.rasterize()  # and without host reads
        assert r.frame_stats()["host_syncs"] == 0
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])


def test_same_structure_scene_keeps_capacities():
    """A new scene with the same element counts (the same scene set again, or
    moved geometry) renders without host reads; one that outgrows the kept
    buffers is rendered again, sized, when read, and stays exact."""
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=63, width=320, height=256, n_paths=200, n_large=8)
    with spr.VGRasterizer(320, 256, samples=32) as r:
        r.add_vg(sc)
        r.rasterize()
        assert r.frame_stats()["host_syncs"] == 2  # the sized first frame
        r.add_vg(sc)
        r.rasterize()
        assert r.frame_stats()["host_syncs"] == 0
        ref = oracle.run(sc, 320, 256, samples=32)
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        # the same structure, every path scaled up 3x about the centre: far
        # more entries than the kept buffers hold
        big = sc.copy()
        big.vertex = ((big.vertex - [160.0, 128.0]) * 3.0 + [160.0, 128.0]).astype(np.float32)
        r.add_vg(big)
        r.rasterize()
        ref = oracle.run(big, 320, 256, samples=32)
        assert np.array_equal(r.read_image().reshape(-1), ref["IMAGE"])
        assert r.element_number() == ref.counts
