"""ctypes wrapper of the CPU oracle (liboracle.so) and of the reference's own
intersection / mask code compiled in place (oracle/_ref/libref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, always as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import sys

import numpy as np

ORACLE_DIR = pathlib.Path(__file__).resolve().parent
ROOT = ORACLE_DIR.parent
sys.path.insert(0, str(ROOT / "gpu-scanline-path-rendering_gb300"))
import spr  # noqa: E402  (ctypes struct layouts of include/spr.h)

LIB_PATH = ORACLE_DIR / "liboracle.so"
REF_PATH = ORACLE_DIR / "_ref" / "libref.so"


class OrcConfig(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("samples", C.c_int32),
                ("ms_output", C.c_int32), ("srgb", C.c_int32), ("threads", C.c_int32),
                ("has_transform", C.c_int32), ("transform", C.c_float * 16),
                ("stop_after", C.c_int32), ("grad_table", C.c_void_p), ("n_grad", C.c_uint32),
                ("grad_ramp", C.c_void_p), ("n_ramp", C.c_uint32), ("has_rev", C.c_int32),
                ("rev", C.c_float * 13)]


def _paints(cfg, scene, rev):
    """Points cfg at the scene's gradient table and ramp (kept alive by the
    returned tuple) and at the reverse transform."""
    keep = ()
    g = getattr(scene, "gradients", None)
    if g is not None:
        table, ramp = (np.ascontiguousarray(x, dtype=np.uint32) for x in g)
        cfg.grad_table, cfg.n_grad = table.ctypes.data, len(table) // 12
        cfg.grad_ramp, cfg.n_ramp = ramp.ctypes.data, len(ramp)
        keep = (table, ramp)
    if rev is not None:
        cfg.has_rev = 1
        for i, v in enumerate(np.asarray(rev, dtype=np.float32).reshape(13)):
            cfg.rev[i] = float(v)
    return keep


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing: run oracle/build_oracle.py")
        L = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        L.orc_run.argtypes = [C.POINTER(spr.SceneView), C.POINTER(OrcConfig), C.POINTER(vp)]
        L.orc_get.argtypes = [vp, C.c_int32, C.POINTER(vp), C.POINTER(C.c_size_t)]
        L.orc_counts.argtypes = [vp, C.POINTER(spr.ElementNumber)]
        L.orc_stage_ms.argtypes = [vp, C.POINTER(C.c_double), C.c_int32]
        L.orc_free.argtypes = [vp]
        L.orc_free.restype = None
        L.orc_sample_positions.argtypes = [C.c_int32, vp]
        L.orc_mask_table.argtypes = [C.c_int32, vp]
        L.orc_pass_samples_256.argtypes = [C.c_int32, vp]
        L.orc_pass_mask_table_256.argtypes = [C.c_int32, vp]
        L.orc_srgb_tables.argtypes = [vp, vp, vp]
        f = C.c_float
        L.orc_fetch_pixel_table.argtypes = [C.c_int32, f, f, f, f, vp]
        L.orc_vertical_mask.argtypes = [C.c_int32, f, vp]
        L.orc_vertical_mask2.argtypes = [C.c_int32, f, f, vp]
        L.orc_fetch_table_selftest.argtypes = [C.c_int32, C.c_int32, vp]
        L.orc_diff.argtypes = [C.POINTER(spr.SceneView), C.POINTER(OrcConfig), vp, vp, vp, vp, vp, vp]
        L.orc_intersection_error.argtypes = [C.POINTER(spr.SceneView), vp, vp, C.c_int64, C.c_int32, C.c_int32,
                                             C.c_int32, C.POINTER(XErr)]
        _lib = L
    return _lib


class XErr(C.Structure):
    _fields_ = [("max_err_px", C.c_double), ("mean_err_px", C.c_double), ("max_resid_px", C.c_double),
                ("n_crossings", C.c_int64), ("n_over_1px", C.c_int64), ("n_unbracketed", C.c_int64),
                ("n_mismatched", C.c_int64), ("worst_entry", C.c_int64)]


def intersection_error(scene: "spr.Scene", tvertex: np.ndarray, entries: np.ndarray, width, height,
                       threads=0) -> dict:
    """FP32 crossing points (the entries' t on the FP32 transformed curves)
    against the exact FP64 crossings with the same cut lines: the error along
    the cut line in pixels (max, mean), with counts."""
    tv = np.ascontiguousarray(tvertex, dtype=np.float32).reshape(-1)
    en = np.ascontiguousarray(entries, dtype=np.int32).reshape(-1)
    out = XErr()
    v = scene.view()
    st = lib().orc_intersection_error(C.byref(v), tv.ctypes.data, en.ctypes.data, len(en) // 2, width, height,
                                      threads, C.byref(out))
    if st != 0:
        raise spr.SprError(st, "orc_intersection_error")
    return {n: (float(getattr(out, n)) if t is C.c_double else int(getattr(out, n))) for n, t in XErr._fields_}


def have_ref() -> bool:
    return REF_PATH.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        L = C.CDLL(str(REF_PATH))
        vp, i32, f = C.c_void_p, C.c_int32, C.c_float
        L.ref_count.argtypes = [i32, vp, vp, vp, vp, vp, i32, vp, i32, i32, vp, vp, vp]
        L.ref_emit.argtypes = [i32, vp, vp, vp, vp, vp, i32, vp, i32, i32, vp, vp, vp, C.c_int64, vp]
        L.ref_mask_table.argtypes = [vp, vp, vp]
        L.ref_fetch_pixel_table.argtypes = [i32, vp, f, f, f, f, vp]
        L.ref_vertical_mask.argtypes = [i32, f, vp]
        L.ref_vertical_mask2.argtypes = [i32, f, f, vp]
        L.ref_sample_positions.argtypes = [i32, vp]
        _ref = L
    return _ref


class Result:
    """Stage outputs of one oracle run (numpy arrays, copied out)."""

    def __init__(self, handle, samples):
        self.samples = samples
        L = lib()
        self.stages = {}
        for name in spr.STAGES:
            p, n = C.c_void_p(), C.c_size_t()
            L.orc_get(handle, spr.STAGE[name], C.byref(p), C.byref(n))
            dt = np.dtype(spr.STAGE_DTYPE[name])
            if n.value and p.value:
                a = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), (n.value,))
                self.stages[name] = a.view(dt).copy()
            else:
                self.stages[name] = np.zeros(0, dtype=dt)
        e = spr.ElementNumber()
        L.orc_counts(handle, C.byref(e))
        self.counts = e.as_dict()
        ms = (C.c_double * len(spr.STAGES))()
        L.orc_stage_ms(handle, ms, len(spr.STAGES))
        self.stage_ms = {spr.STAGES[i]: ms[i] for i in range(len(spr.STAGES))}

    def __getitem__(self, k):
        return self.stages[k]


def run(scene: "spr.Scene", width, height, samples=8, ms_output=True, srgb=True, threads=0,
        transform=None, stop_after=-1, rev=None) -> Result:
    cfg = OrcConfig(width, height, samples, int(ms_output), int(srgb), threads,
                    0 if transform is None else 1, (C.c_float * 16)(), stop_after)
    keep = _paints(cfg, scene, rev)  # noqa: F841 (alive through the call)
    if transform is not None:
        t = np.asarray(transform, dtype=np.float32).reshape(16)
        for i in range(16):
            cfg.transform[i] = float(t[i])
    v = scene.view()
    h = C.c_void_p()
    st = lib().orc_run(C.byref(v), C.byref(cfg), C.byref(h))
    try:
        if st != 0:
            raise spr.SprError(st, "orc_run")
        return Result(h, samples)
    finally:
        if h.value:
            lib().orc_free(h)


def diff(scene: "spr.Scene", width, height, fill, grad_image=None, samples=16, transform=None, threads=0):
    """Reference differentiable render: returns (image (H, W, 4) float64, and
    when grad_image is given grads {fill (P, 4), vertex (V, 2), affine (P, 6)
    or None})."""
    cfg = OrcConfig(width, height, samples, 1, 0, threads, 0 if transform is None else 1, (C.c_float * 16)(), -1)
    if transform is not None:
        t = np.asarray(transform, dtype=np.float32).reshape(16)
        for i in range(16):
            cfg.transform[i] = float(t[i])
    fill = np.ascontiguousarray(fill, dtype=np.float32).reshape(-1, 4)
    img = np.zeros((height, width, 4), np.float64)
    gi = None if grad_image is None else np.ascontiguousarray(grad_image, dtype=np.float32).reshape(height, width, 4)
    gf = np.zeros((scene.n_paths, 4), np.float64)
    gv = np.zeros((scene.n_vertices, 2), np.float64)
    ga = np.zeros((scene.n_paths, 6), np.float64) if scene.path_affine is not None else None
    v = scene.view()
    st = lib().orc_diff(C.byref(v), C.byref(cfg), fill.ctypes.data, None if gi is None else gi.ctypes.data,
                        img.ctypes.data, gf.ctypes.data if gi is not None else None,
                        gv.ctypes.data if gi is not None else None,
                        ga.ctypes.data if (gi is not None and ga is not None) else None)
    if st != 0:
        raise spr.SprError(st, "orc_diff")
    if gi is None:
        return img, None
    return img, {"fill": gf, "vertex": gv, "affine": ga}


def time_run(scene: "spr.Scene", width, height, samples=8, ms_output=True, srgb=True, threads=0,
             transform=None):
    """Runs the whole pipeline and returns (milliseconds summed over the stages,
    element counts) without copying any stage output."""
    cfg = OrcConfig(width, height, samples, int(ms_output), int(srgb), threads,
                    0 if transform is None else 1, (C.c_float * 16)(), -1)
    if transform is not None:
        t = np.asarray(transform, dtype=np.float32).reshape(16)
        for i in range(16):
            cfg.transform[i] = float(t[i])
    v = scene.view()
    h = C.c_void_p()
    st = lib().orc_run(C.byref(v), C.byref(cfg), C.byref(h))
    try:
        if st != 0:
            raise spr.SprError(st, "orc_run")
        ms = (C.c_double * len(spr.STAGES))()
        lib().orc_stage_ms(h, ms, len(spr.STAGES))
        e = spr.ElementNumber()
        lib().orc_counts(h, C.byref(e))
        return float(sum(ms)), e.as_dict()
    finally:
        if h.value:
            lib().orc_free(h)


def sample_positions(samples) -> np.ndarray:
    out = np.zeros((4 * samples, 2), dtype=np.float32)
    lib().orc_sample_positions(samples, out.ctypes.data)
    return out


def pass_samples_256(g) -> np.ndarray:
    out = np.zeros((32, 2), dtype=np.float32)
    st = lib().orc_pass_samples_256(g, out.ctypes.data)
    if st != 0:
        raise spr.SprError(st, "orc_pass_samples_256")
    return out


def pass_mask_table_256(g) -> np.ndarray:
    out = np.zeros((65536, 4), dtype=np.uint32)
    st = lib().orc_pass_mask_table_256(g, out.ctypes.data)
    if st != 0:
        raise spr.SprError(st, "orc_pass_mask_table_256")
    return out


def mask_table(samples) -> np.ndarray:
    out = np.zeros((65536, samples // 8), dtype=np.uint32)
    lib().orc_mask_table(samples, out.ctypes.data)
    return out


def srgb_tables():
    dec = np.zeros(256, np.float32)
    th = np.zeros(255, np.float32)
    bins = np.zeros(4096, np.uint8)
    lib().orc_srgb_tables(dec.ctypes.data, th.ctypes.data, bins.ctypes.data)
    return dec, th, bins


def fetch_pixel_table(samples, p0, p1) -> np.ndarray:
    out = np.zeros(samples // 8, np.uint32)
    lib().orc_fetch_pixel_table(samples, p0[0], p0[1], p1[0], p1[1], out.ctypes.data)
    return out


def fetch_table_selftest(samples, res=33) -> np.ndarray:
    hist = np.zeros(33, np.int64)
    lib().orc_fetch_table_selftest(samples, res, hist.ctypes.data)
    return hist


def vertical_mask(samples, y) -> np.ndarray:
    out = np.zeros(samples // 8, np.uint32)
    lib().orc_vertical_mask(samples, y, out.ctypes.data)
    return out


def vertical_mask2(samples, y0, y1) -> np.ndarray:
    out = np.zeros(samples // 8, np.uint32)
    lib().orc_vertical_mask2(samples, y0, y1, out.ctypes.data)
    return out


# ---- the reference's own code, compiled in place --------------------------
def ref_intersections(scene: "spr.Scene", tvertex: np.ndarray, visible: np.ndarray, width, height):
    """Counts and entries from the reference's k_make_intersection_0/1."""
    L = ref()
    nc = scene.n_curves
    tv = np.ascontiguousarray(tvertex, dtype=np.float32)
    vis = np.ascontiguousarray(visible, dtype=np.uint8)
    counts = np.zeros(nc, np.int32)
    tcut = np.zeros((nc, 4), np.float32)
    ncut = np.zeros(nc, np.int8)
    args = (nc, tv.ctypes.data, scene.curve_vertex_pos.ctypes.data, scene.curve_type.ctypes.data,
            scene.curve_path_id.ctypes.data, scene.curve_arc_w.ctypes.data, scene.n_paths,
            vis.ctypes.data, width, height)
    L.ref_count(*args, counts.ctypes.data, tcut.ctypes.data, ncut.ctypes.data)
    offs = np.zeros(nc, np.int32)
    if nc:
        offs[1:] = np.cumsum(counts[:-1], dtype=np.int64).astype(np.int32)
    nf = int(counts.sum(dtype=np.int64))
    entries = np.zeros((max(nf, 1), 2), np.int32)
    L.ref_emit(*args, offs.ctypes.data, tcut.ctypes.data, ncut.ctypes.data, nf, entries.ctypes.data)
    return counts, entries[:nf]


def ref_sample_positions(samples) -> np.ndarray:
    """Pixel sample pattern from the reference's vg_sample_position."""
    out = np.zeros((samples, 2), np.float32)
    ref().ref_sample_positions(samples, out.ctypes.data)
    return out


def ref_mask_table(samples8_cell: np.ndarray, samples32_cell: np.ndarray):
    s = np.concatenate([samples8_cell.reshape(-1, 2), samples32_cell.reshape(-1, 2)]).astype(np.float32)
    assert s.shape == (160, 2)
    s = np.ascontiguousarray(s)
    t8 = np.zeros(65536, np.int32)
    t32 = np.zeros((65536, 4), np.int32)
    ref().ref_mask_table(s.ctypes.data, t8.ctypes.data, t32.ctypes.data)
    return t8.view(np.uint32), t32.view(np.uint32)


def ref_fetch_pixel_table(samples, table: np.ndarray, p0, p1) -> np.ndarray:
    t = np.ascontiguousarray(table).view(np.int32)
    out = np.zeros(4, np.int32)
    ref().ref_fetch_pixel_table(samples, t.ctypes.data, p0[0], p0[1], p1[0], p1[1], out.ctypes.data)
    return out.view(np.uint32)[: samples // 8]


def ref_vertical_mask(samples, y) -> np.ndarray:
    out = np.zeros(4, np.int32)
    ref().ref_vertical_mask(samples, y, out.ctypes.data)
    return out.view(np.uint32)[: samples // 8]


def ref_vertical_mask2(samples, y0, y1) -> np.ndarray:
    out = np.zeros(4, np.int32)
    ref().ref_vertical_mask2(samples, y0, y1, out.ctypes.data)
    return out.view(np.uint32)[: samples // 8]


def output_inverse(m):
    """Rows 0, 1, 3 / columns 0, 1, 3 of the inverse of the row-major 4x4 m,
    by Gauss-Jordan elimination with partial pivoting in double precision,
    then rounded to float32 (spr_set_output_transform's arithmetic)."""
    a = [[float(m[4 * r + c]) for c in range(4)] + [1.0 if k == r else 0.0 for k in range(4)] for r in range(4)]
    for c in range(4):
        piv = c
        for r in range(c + 1, 4):
            if abs(a[r][c]) > abs(a[piv][c]):
                piv = r
        if not abs(a[piv][c]) > 0.0:
            raise ValueError("singular output transform")
        a[c], a[piv] = a[piv], a[c]
        d = a[c][c]
        a[c] = [v / d for v in a[c]]
        for r in range(4):
            if r != c:
                f = a[r][c]
                a[r] = [a[r][k] - f * a[c][k] for k in range(8)]
    return np.array([[a[r][4 + c] for c in (0, 1, 3)] for r in (0, 1, 3)], np.float32)


def output_view(image, m):
    """The output view (drawOutputResize, ras_base.cpp:760-803, with
    output_scale.vert.glsl / .frag.glsl): pixel (x, y) takes the texel
    nearest to inverse(m) * (x + 0.5, y + 0.5, 0, 1) / w, clamped to the edge
    (GL_NEAREST, GL_CLAMP_TO_EDGE).  image: (H, W, 4) uint8."""
    H, W = image.shape[:2]
    inv = output_inverse(np.asarray(m, np.float32).reshape(16))
    py, px = np.meshgrid(np.arange(H, dtype=np.float32) + np.float32(0.5),
                         np.arange(W, dtype=np.float32) + np.float32(0.5), indexing="ij")
    q = [(inv[r, 0] * px + inv[r, 1] * py) + inv[r, 2] for r in range(3)]
    with np.errstate(divide="ignore", invalid="ignore"):
        u, v = q[0] / q[2], q[1] / q[2]
    u = np.clip(np.nan_to_num(np.floor(u), nan=0.0), 0, W - 1).astype(np.int64)
    v = np.clip(np.nan_to_num(np.floor(v), nan=0.0), 0, H - 1).astype(np.int64)
    return image[v, u]
