"""The output transform (setOutputTransform / enableOutputTransform and
drawOutputResize's nearest-texel view, ras_base.cpp:586-593, 760-803):
spr_read_output against the oracle's restatement, oracle.output_view."""
import numpy as np
import pytest

import oracle
import spr


def zoom(s, cx, cy):
    """Scale by s about (cx, cy), row-major 4x4."""
    return np.array([[s, 0, 0, cx - s * cx], [0, s, 0, cy - s * cy], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)


def test_oracle_view():
    img = np.arange(6 * 5 * 4, dtype=np.uint32).astype(np.uint8).reshape(6, 5, 4)
    assert np.array_equal(oracle.output_view(img, np.eye(4)), img)
    # zoom 2 about the origin: pixel (x, y) shows texel (floor((x + .5) / 2), ...)
    v = oracle.output_view(img, zoom(2, 0, 0))
    assert np.array_equal(v[3, 4], img[1, 2]) and np.array_equal(v[5, 0], img[2, 0])
    # a translation past the edge clamps
    t = np.eye(4, dtype=np.float32)
    t[0, 3] = 100
    assert np.array_equal(oracle.output_view(img, t), np.repeat(img[:, :1], 5, axis=1))
    m = np.random.default_rng(1).normal(size=(4, 4))
    inv = np.linalg.inv(m)[np.ix_([0, 1, 3], [0, 1, 3])]
    assert np.allclose(oracle.output_inverse(m.reshape(16)), inv, rtol=1e-5, atol=1e-6)
    with pytest.raises(ValueError):
        oracle.output_inverse(np.zeros(16))


@pytest.mark.gpu
def test_gpu_output_view():
    W, H = 256, 200
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=13, width=W, height=H, n_paths=60)
    rng = np.random.default_rng(3)
    rot = np.array([[0, -1, 0, W / 2 + H / 2], [1, 0, 0, H / 2 - W / 2], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)
    aff = np.eye(4, dtype=np.float32)
    aff[:2, :2] = rng.normal(1, 0.3, (2, 2))
    aff[:2, 3] = rng.normal(0, 20, 2)
    proj = np.eye(4, dtype=np.float32)
    proj[3, 0], proj[3, 1] = 1e-3, -5e-4
    with spr.VGRasterizer(W, H, samples=32) as r:
        r.add_vg(sc)
        r.rasterize()
        img = r.read_image()
        assert np.array_equal(r.read_output(), img)  # off: the image itself
        r.enable_output_transform(True)
        for m in (np.eye(4, dtype=np.float32), zoom(2, 64, 50), zoom(0.5, 0, 0), rot, aff, proj):
            r.set_output_transform(m)
            assert np.array_equal(r.read_output(), oracle.output_view(img, m))
        assert np.array_equal(r.read_image(), img)  # the image stays unzoomed
        with pytest.raises(spr.SprError) as e:
            r.set_output_transform(np.zeros((4, 4), np.float32))
        assert e.value.status == spr.ERR_INVALID_ARG
