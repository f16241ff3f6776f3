"""Differentiable rendering (spr_diff_render / spr_diff_backward) on the GPU.

* the float composite against the oracle's restatement;
* gradients against the oracle's reference gradient (same estimator, double
  accumulation): relative error <= 1e-3 per gradient group;
* vertex gradients against central differences of the rendered loss,
  averaged over sub-pixel jitters of the scene (a 16-spp render under 64
  jitters samples every pixel 1024 times);
* a thin torch.autograd.Function over the C ABI, used by these tests only.
"""
import numpy as np
import pytest

import oracle
import spr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


class DiffRender(torch.autograd.Function):
    """image = render(fill, vertex[, affine]) through the C ABI."""

    @staticmethod
    def forward(ctx, fill, vertex, affine, r, scene, W, H):
        sc = scene.copy()
        sc.vertex = vertex.detach().cpu().numpy().astype(np.float32)
        if affine is not None:
            sc.path_affine = affine.detach().cpu().numpy().astype(np.float32)
        r.add_vg(sc)
        fill = fill.detach().contiguous()
        img = torch.empty((H, W, 4), device="cuda", dtype=torch.float32)
        r.diff_render(fill.data_ptr(), img.data_ptr(), torch.cuda.current_stream().cuda_stream)
        ctx.r, ctx.n_v, ctx.has_affine = r, sc.n_vertices, affine is not None
        ctx.save_for_backward(fill)
        return img

    @staticmethod
    def backward(ctx, grad_img):
        (fill,) = ctx.saved_tensors
        gi = grad_img.contiguous().float()
        gf = torch.empty_like(fill)
        gv = torch.empty((ctx.n_v, 2), device="cuda", dtype=torch.float32)
        ga = torch.empty((fill.shape[0], 6), device="cuda", dtype=torch.float32) if ctx.has_affine else None
        ctx.r.diff_backward(fill.data_ptr(), gi.data_ptr(), gf.data_ptr(), gv.data_ptr(),
                            None if ga is None else ga.data_ptr(), torch.cuda.current_stream().cuda_stream)
        return gf, gv, ga, None, None, None, None


def fills(P, seed):
    rng = np.random.default_rng(seed)
    return np.c_[rng.uniform(0, 1, (P, 3)), rng.uniform(0.5, 1.0, (P, 1))].astype(np.float32)


def gpu_diff(scene, W, H, fill, G, samples=16, transform=None):
    with spr.VGRasterizer(W, H, samples=samples) as r:
        if transform is not None:
            r.set_input_transform(transform)
        r.add_vg(scene)
        f = torch.tensor(fill, device="cuda")
        img = torch.empty((H, W, 4), device="cuda")
        r.diff_render(f.data_ptr(), img.data_ptr())
        gi = torch.tensor(G, device="cuda")
        gf = torch.empty_like(f)
        gv = torch.empty((scene.n_vertices, 2), device="cuda")
        ga = torch.empty((scene.n_paths, 6), device="cuda") if scene.path_affine is not None else None
        r.diff_backward(f.data_ptr(), gi.data_ptr(), gf.data_ptr(), gv.data_ptr(), None if ga is None else ga.data_ptr())
        torch.cuda.synchronize()
        return (img.cpu().numpy(), gf.cpu().numpy(), gv.cpu().numpy(), None if ga is None else ga.cpu().numpy())


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def smooth_weights(W, H):
    yy, xx = np.mgrid[0:H, 0:W] / max(W, H)
    return np.stack([np.sin(3 * xx + 1), np.cos(2 * yy), np.sin(2 * xx + 3 * yy), 0.5 * np.cos(xx - yy)],
                    -1).astype(np.float32)


@pytest.mark.parametrize("samples", [8, 16, 32])
@pytest.mark.parametrize("kind", [spr.SCENE_CUBICS, spr.SCENE_RANDOM, spr.SCENE_MIXED])
def test_against_reference_gradient(samples, kind):
    W, H = 160, 128
    sc = spr.Scene.generate(kind, seed=61 + kind, width=W, height=H, n_paths=24, n_large=3, seg_min=6,
                            seg_max=16, with_rational=True, with_affine=kind == spr.SCENE_MIXED)
    fill = fills(sc.n_paths, 7)
    G = np.random.default_rng(8).normal(size=(H, W, 4)).astype(np.float32)
    img, gf, gv, ga = gpu_diff(sc, W, H, fill, G, samples)
    ref_img, ref = oracle.diff(sc, W, H, fill, grad_image=G, samples=samples)
    assert np.abs(img - ref_img).max() < 1e-5
    assert rel(gf, ref["fill"]) < REL_TOL
    assert rel(gv, ref["vertex"]) < REL_TOL
    if ga is not None:
        assert rel(ga, ref["affine"]) < REL_TOL


def test_transform_and_deep_overlap():
    """A projective input transform, and 300 overlapping viewport-sized paths
    (samples under hundreds of layers: the tape grows past its first size)."""
    W, H = 96, 80
    sc = spr.Scene.generate(spr.SCENE_RANDOM, seed=71, width=W, height=H, n_paths=300, seg_min=4, seg_max=8)
    fill = fills(sc.n_paths, 9)
    tf = np.array([[1.1, 0.1, 0, 2], [-0.05, 0.9, 0, 3], [0, 0, 1, 0], [0.0005, 0.0002, 0, 1]], np.float32)
    G = smooth_weights(W, H)
    img, gf, gv, _ = gpu_diff(sc, W, H, fill, G, 16, tf)
    ref_img, ref = oracle.diff(sc, W, H, fill, grad_image=G, samples=16, transform=tf)
    assert np.abs(img - ref_img).max() < 1e-5
    assert rel(gf, ref["fill"]) < REL_TOL and rel(gv, ref["vertex"]) < REL_TOL


def test_many_paths():
    """More paths than the block-wide fill-gradient accumulators hold (4096):
    the backward pass accumulates in per-warp path caches instead, whose
    evictions (paths equal modulo the cache size) go to the global gradient."""
    W, H = 128, 128
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=81, width=W, height=H, n_paths=4200, n_large=60, seg_min=3,
                            seg_max=6)
    assert sc.n_paths > 4096
    fill = fills(sc.n_paths, 3)
    G = np.random.default_rng(8).normal(size=(H, W, 4)).astype(np.float32)
    img, gf, gv, _ = gpu_diff(sc, W, H, fill, G, 8)
    ref_img, ref = oracle.diff(sc, W, H, fill, grad_image=G, samples=8)
    assert np.abs(img - ref_img).max() < 1e-5
    assert rel(gf, ref["fill"]) < REL_TOL and rel(gv, ref["vertex"]) < REL_TOL


def test_256_samples_against_reference_gradient():
    """256 samples per pixel (8 passes of 32, each weighted 1/8): image and
    gradients against the oracle's passes."""
    W, H = 96, 80
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=67, width=W, height=H, n_paths=12, n_large=2, seg_min=4,
                            seg_max=10, with_rational=True, with_affine=True)
    fill = fills(sc.n_paths, 17)
    G = np.random.default_rng(18).normal(size=(H, W, 4)).astype(np.float32)
    img, gf, gv, ga = gpu_diff(sc, W, H, fill, G, 256)
    ref_img, ref = oracle.diff(sc, W, H, fill, grad_image=G, samples=256)
    assert np.abs(img - ref_img).max() < 1e-5
    assert rel(gf, ref["fill"]) < REL_TOL and rel(gv, ref["vertex"]) < REL_TOL
    assert rel(ga, ref["affine"]) < REL_TOL


def test_empty_scene_and_errors():
    empty = spr.Scene(np.zeros((0, 2), np.float32), [], [], [], [], [], [], [])
    with spr.VGRasterizer(48, 40, samples=16) as r:
        r.add_vg(empty)
        f = torch.zeros((1, 4), device="cuda")
        img = torch.zeros((40, 48, 4), device="cuda")
        r.diff_render(f.data_ptr(), img.data_ptr())
        g = torch.ones((40, 48, 4), device="cuda")
        gf = torch.ones((1, 4), device="cuda")
        gv = torch.ones((1, 2), device="cuda")
        r.diff_backward(f.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr())
        torch.cuda.synchronize()
        assert torch.all(img == 1.0)
        with pytest.raises(spr.SprError) as e:
            r.diff_render(0, img.data_ptr())
        assert e.value.status == spr.ERR_INVALID_ARG
        with pytest.raises(spr.SprError) as e:  # no per-path affine in this scene
            r.diff_backward(f.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr(), gf.data_ptr())
        assert e.value.status == spr.ERR_INVALID_ARG


@pytest.mark.parametrize("samples,n_jit,h", [(16, 64, 0.1), (256, 4, 0.1), (256, 16, 0.01)])
def test_finite_differences_on_jittered_renders(samples, n_jit, h):
    """dL/d(vertex) against central differences (step h px: 0.1, or 0.01 on
    256-sample renders) of the rendered loss, both averaged over sub-pixel
    translations (16 spp x 64 translations, 256 spp x 4 or 256 spp x 16);
    coincident endpoint copies of a contour move together (one contour
    point)."""
    W = H = 96
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=5, width=W, height=H, n_paths=6, seg_min=4, seg_max=6)
    fill = fills(sc.n_paths, 1)
    G = smooth_weights(W, H)
    rng = np.random.default_rng(2)
    jit = [np.eye(4, dtype=np.float32) for _ in range(n_jit)]
    for t in jit:
        t[0, 3], t[1, 3] = rng.uniform(0, 1), rng.uniform(0, 1)
    Gt = torch.tensor(G, device="cuda")
    with spr.VGRasterizer(W, H, samples=samples) as r:
        f = torch.tensor(fill, device="cuda")
        img = torch.empty((H, W, 4), device="cuda")

        def loss(scene, t):
            r.set_input_transform(t)
            r.add_vg(scene)
            r.diff_render(f.data_ptr(), img.data_ptr())
            return float((img * Gt).sum())

        gv = np.zeros((sc.n_vertices, 2))
        gfv = torch.empty_like(f)
        g2 = torch.empty((sc.n_vertices, 2), device="cuda")
        for t in jit:
            r.set_input_transform(t)
            r.add_vg(sc)
            r.diff_backward(f.data_ptr(), Gt.data_ptr(), gfv.data_ptr(), g2.data_ptr())
            gv += g2.cpu().numpy()
        gv /= len(jit)
        an, fd = [], []
        for vi in [3, 10, 17, 25, 40, 41, 55, 70, 88, 101]:
            grp = np.nonzero((sc.vertex_path_id == sc.vertex_path_id[vi]) & np.all(sc.vertex == sc.vertex[vi], 1))[0]
            for c in range(2):
                acc = 0.0
                for t in jit:
                    sp, sm = sc.copy(), sc.copy()
                    sp.vertex[grp, c] += h
                    sm.vertex[grp, c] -= h
                    acc += (loss(sp, t) - loss(sm, t)) / (2 * h)
                an.append(gv[grp, c].sum())
                fd.append(acc / len(jit))
    an, fd = np.array(an), np.array(fd)
    cos = float(an @ fd / (np.linalg.norm(an) * np.linalg.norm(fd)))
    assert cos > 0.97, (cos, an, fd)
    assert rel(an, fd) < 0.2


def test_autograd_fit_step():
    """The autograd wrapper: one gradient step on fills and vertices lowers an
    L2 loss against a target rendered from perturbed parameters."""
    W = H = 128
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=9, width=W, height=H, n_paths=12, seg_min=4, seg_max=8)
    rng = np.random.default_rng(3)
    fill0 = fills(sc.n_paths, 4)
    with spr.VGRasterizer(W, H, samples=16) as r:
        tgt_scene = sc.copy()
        tgt_scene.vertex = tgt_scene.vertex + rng.normal(0, 2.0, tgt_scene.vertex.shape).astype(np.float32)
        tgt_fill = np.clip(fill0 + rng.normal(0, 0.05, fill0.shape), 0, 1).astype(np.float32)
        target = DiffRender.apply(torch.tensor(tgt_fill, device="cuda"),
                                  torch.tensor(tgt_scene.vertex, device="cuda"), None, r, sc, W, H).detach()
        # contour points: the coincident end point copies of consecutive curves are one parameter
        keys = np.c_[sc.vertex_path_id[:, None].astype(np.float64), sc.vertex.astype(np.float64)]
        uniq, inv = np.unique(keys, axis=0, return_inverse=True)
        idx = torch.tensor(inv.reshape(-1), device="cuda")
        fill = torch.tensor(fill0, device="cuda", requires_grad=True)
        pts = torch.tensor(uniq[:, 1:].astype(np.float32), device="cuda", requires_grad=True)
        img = DiffRender.apply(fill, pts[idx], None, r, sc, W, H)
        loss = ((img - target) ** 2).sum()
        loss.backward()
        assert fill.grad is not None and pts.grad is not None
        assert torch.isfinite(fill.grad).all() and torch.isfinite(pts.grad).all()
        with torch.no_grad():
            f2 = fill - 1e-3 * fill.grad / fill.grad.abs().max()
            p2 = pts - 0.1 * pts.grad / pts.grad.abs().max()
            loss2 = ((DiffRender.apply(f2, p2[idx], None, r, sc, W, H) - target) ** 2).sum()
        assert float(loss2) < float(loss.detach())


def test_batch_matches_single_scene_diff():
    """Batched forward and backward (one sample count): every scene's image
    and gradients equal those of its own handle (summation order aside)."""
    sizes = [(160, 128), (96, 200), (64, 64), (257, 129)]
    items, scenes = [], []
    for i, (W, H) in enumerate(sizes):
        sc = spr.Scene.generate(spr.SCENE_CUBICS if i % 2 else spr.SCENE_MIXED, seed=300 + i, width=W, height=H,
                                n_paths=10 + 5 * i, n_large=2, seg_min=4, seg_max=10, with_affine=True)
        tf = None
        if i == 1:
            tf = np.eye(4, dtype=np.float32)
            tf[0, 0], tf[1, 3] = 0.9, 4.0
        items.append((sc, W, H, 16) + ((tf,) if tf is not None else ()))
        scenes.append((sc, W, H, tf))
    fills_all = [fills(sc.n_paths, 20 + i) for i, (sc, _, _, _) in enumerate(scenes)]
    rng = np.random.default_rng(21)
    Gs = [rng.normal(size=(H, W, 4)).astype(np.float32) for (_, W, H, _) in scenes]
    with spr.Batch() as b:
        b.set_scenes(items)
        off = b.image_offsets()
        f = torch.tensor(np.concatenate(fills_all), device="cuda")
        img = torch.empty((int(off[-1]), 4), device="cuda")
        b.diff_render(f.data_ptr(), img.data_ptr())
        G = torch.tensor(np.concatenate([g.reshape(-1, 4) for g in Gs]), device="cuda")
        P = f.shape[0]
        V = sum(sc.n_vertices for sc, _, _, _ in scenes)
        gf = torch.empty((P, 4), device="cuda")
        gv = torch.empty((V, 2), device="cuda")
        ga = torch.empty((P, 6), device="cuda")
        b.diff_backward(f.data_ptr(), G.data_ptr(), gf.data_ptr(), gv.data_ptr(), ga.data_ptr())
        torch.cuda.synchronize()
        img, gf, gv, ga = img.cpu().numpy(), gf.cpu().numpy(), gv.cpu().numpy(), ga.cpu().numpy()
    p0 = v0 = 0
    for i, (sc, W, H, tf) in enumerate(scenes):
        si, sgf, sgv, sga = gpu_diff(sc, W, H, fills_all[i], Gs[i], 16, tf)
        assert np.abs(img[off[i]:off[i + 1]].reshape(H, W, 4) - si).max() < 1e-6
        P_i, V_i = sc.n_paths, sc.n_vertices
        assert rel(gf[p0:p0 + P_i], sgf) < 1e-4
        assert rel(gv[v0:v0 + V_i], sgv) < 1e-4
        assert rel(ga[p0:p0 + P_i], sga) < 1e-4
        p0 += P_i
        v0 += V_i


def test_update_vertices_equals_a_new_upload():
    """spr_update_vertices (device vertices) renders exactly what a new
    spr_set_scene with the moved vertices renders, plain and differentiable."""
    W = H = 192
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=33, width=W, height=H, n_paths=20, seg_min=6, seg_max=16)
    moved = sc.copy()
    moved.vertex = (sc.vertex + np.random.default_rng(4).normal(0, 3.0, sc.vertex.shape)).astype(np.float32)
    fill = torch.tensor(fills(sc.n_paths, 5), device="cuda")
    with spr.VGRasterizer(W, H, samples=16) as a, spr.VGRasterizer(W, H, samples=16) as b:
        a.add_vg(sc)
        a.rasterize()
        vdev = torch.tensor(moved.vertex, device="cuda")
        a.update_vertices(vdev.data_ptr())
        a.rasterize()
        b.add_vg(moved)
        b.rasterize()
        assert np.array_equal(a.read_image(), b.read_image())
        ia = torch.empty((H, W, 4), device="cuda")
        ib = torch.empty((H, W, 4), device="cuda")
        a.diff_render(fill.data_ptr(), ia.data_ptr())
        b.diff_render(fill.data_ptr(), ib.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(ia, ib)


def test_backward_reuses_the_held_forward_frame():
    """A backward right after a differentiable forward of the same inputs runs
    the adjoint kernels only (one host read: the tape-depth check); any
    change in between (a plain frame, moved vertices) makes it recompute
    every stage.  Gradients agree either way."""
    W, H = 160, 112
    sc = spr.Scene.generate(spr.SCENE_CUBICS, seed=41, width=W, height=H, n_paths=30, seg_min=6, seg_max=16)
    moved = sc.copy()
    moved.vertex = (sc.vertex + np.random.default_rng(6).normal(0, 2.0, sc.vertex.shape)).astype(np.float32)
    f = torch.tensor(fills(sc.n_paths, 12), device="cuda")
    g = torch.tensor(smooth_weights(W, H), device="cuda")
    img = torch.empty((H, W, 4), device="cuda")

    def backward(r):
        gf = torch.empty_like(f)
        gv = torch.empty((sc.n_vertices, 2), device="cuda")
        r.diff_backward(f.data_ptr(), g.data_ptr(), gf.data_ptr(), gv.data_ptr())
        torch.cuda.synchronize()
        return gf.cpu().numpy(), gv.cpu().numpy(), r.frame_stats()

    with spr.VGRasterizer(W, H, samples=16) as r:
        r.add_vg(sc)
        r.diff_render(f.data_ptr(), img.data_ptr())
        gf1, gv1, st1 = backward(r)
        gf2, gv2, st2 = backward(r)  # still held
        r.rasterize()
        gf3, gv3, st3 = backward(r)  # recomputed
        assert st1["host_syncs"] == 1 and st2["host_syncs"] == 1 and st3["host_syncs"] == 3
        assert st1["kernel_launches"] < st3["kernel_launches"]
        for a, b in ((gf1, gf2), (gf1, gf3), (gv1, gv2), (gv1, gv3)):
            assert rel(a, b) < 1e-5
        # moved vertices between the forward and the backward
        r.diff_render(f.data_ptr(), img.data_ptr())
        vdev = torch.tensor(moved.vertex, device="cuda")
        r.update_vertices(vdev.data_ptr())
        gf4, gv4, st4 = backward(r)
        assert st4["host_syncs"] == 3
    with spr.VGRasterizer(W, H, samples=16) as r:
        r.add_vg(moved)
        r.diff_render(f.data_ptr(), img.data_ptr())
        gf5, gv5, _ = backward(r)
    assert rel(gf4, gf5) < 1e-5 and rel(gv4, gv5) < 1e-5


def test_open_contours_against_reference_gradient():
    """Open contours (winding sums carried past their rows, as in the plain
    frame) and orphaned vertices: image and gradients against the CPU
    reference gradient."""
    from test_gpu_parity import drop_curves
    W, H = 160, 128
    sc = spr.Scene.generate(spr.SCENE_MIXED, seed=77, width=W, height=H, n_paths=24, n_large=3, seg_min=6,
                            seg_max=16, with_rational=True)
    sc = drop_curves(sc, np.random.default_rng(5).random(sc.n_curves) > 0.1)
    fill = fills(sc.n_paths, 11)
    G = np.random.default_rng(12).normal(size=(H, W, 4)).astype(np.float32)
    img, gf, gv, _ = gpu_diff(sc, W, H, fill, G, 16)
    ref_img, ref = oracle.diff(sc, W, H, fill, grad_image=G, samples=16)
    assert np.abs(img - ref_img).max() < 1e-5
    assert rel(gf, ref["fill"]) < REL_TOL and rel(gv, ref["vertex"]) < REL_TOL


def test_batch_plain_and_differentiable_frames_alternate():
    """A batch of glyph-like scenes rendered plain (the built-in resolve tile
    of short spans), then differentiable (64 x 1 tiles), then plain again:
    the scene table follows each frame's tile, the plain images equal the
    single-scene renders both times and the differentiable image equals the
    single-scene one."""
    sizes = [(256, 256), (192, 160)]
    scenes = [spr.Scene.generate(spr.SCENE_MIXED, seed=400 + i, width=W, height=H, n_paths=300)
              for i, (W, H) in enumerate(sizes)]
    items = [(sc, W, H, 16) for sc, (W, H) in zip(scenes, sizes)]
    fills_all = [fills(sc.n_paths, 40 + i) for i, sc in enumerate(scenes)]
    with spr.Batch() as b:
        b.set_scenes(items)
        b.render()
        first = [b.read_image(i).copy() for i in range(len(items))]
        off = b.image_offsets()
        f = torch.tensor(np.concatenate(fills_all), device="cuda")
        img = torch.empty((int(off[-1]), 4), device="cuda")
        b.diff_render(f.data_ptr(), img.data_ptr())
        torch.cuda.synchronize()
        dimg = img.cpu().numpy()
        b.render()
        again = [b.read_image(i).copy() for i in range(len(items))]
    for i, (sc, (W, H)) in enumerate(zip(scenes, sizes)):
        with spr.VGRasterizer(W, H, samples=16) as r:
            r.add_vg(sc)
            r.rasterize()
            single = r.read_image()
        assert np.array_equal(first[i], single), i
        assert np.array_equal(again[i], single), i
        si = gpu_diff(sc, W, H, fills_all[i], np.zeros((H, W, 4), np.float32), 16)[0]
        assert np.abs(dimg[off[i]:off[i + 1]].reshape(H, W, 4) - si).max() < 1e-6
