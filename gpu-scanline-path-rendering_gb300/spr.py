"""Python mirror of the renderer's C ABI (include/spr.h).

The class :class:`VGRasterizer` mirrors the reference plugin interface
``RasterizerBase::VGRasterizer`` (gpu-scanline/src/rasterizer/shared/
ras_base.h:133-378): ``addVg`` -> :meth:`VGRasterizer.add_vg`,
``setInputTransform`` -> :meth:`set_input_transform`, ``rasterize`` ->
:meth:`rasterize`, ``elementNumber`` -> :meth:`element_number`,
``saveOutputToFile`` -> :meth:`save_output_to_file`, ``setSamples`` /
``setMultisampleOutput`` / ``enableSRGBCorrection`` and step timing.  Errors
come back from the library as status codes and are raised here as
:class:`SprError`.

The binding loads the in-tree ``libspr.so`` built by ``build.py``; it never
falls back to another implementation.  Host-only entry points (the scene
generator, validation) work without a GPU; everything that renders needs one.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

import numpy as np

PKG_DIR = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libspr.so"

# ---- status codes (enum spr_status) ---------------------------------------
OK = 0
ERR_INVALID_ARG = 1
ERR_INVALID_SCENE = 2
ERR_OUT_OF_MEMORY = 3
ERR_CAPACITY_EXCEEDED = 4
ERR_TIMEOUT = 5
ERR_CUDA = 6
ERR_NO_SCENE = 7
ERR_UNSUPPORTED = 8

# ---- curve types / fill rules / stages / scene kinds -----------------------
CURVE_LINEAR, CURVE_QUADRATIC, CURVE_CUBIC, CURVE_RATIONAL = 0x02, 0x03, 0x04, 0x13
RVG_A128, RVG_SRGB_RAMPS = 1, 2
FILL_NONZERO, FILL_EVEN_ODD = 0, 1
SCENE_RANDOM, SCENE_MIXED, SCENE_CUBICS, SCENE_LOCAL = 0, 1, 2, 3

STAGES = [
    "TVERTEX", "PATH_VISIBLE", "CURVE_COUNT", "INTERSECTION", "FRAG_KEY", "FRAG_PID", "FRAG_WN",
    "FRAG_MASK", "SORT_PERM", "SORT_KEY", "WN_SCAN", "MERGED_MASK", "DRAW_LIST", "IMAGE",
]
STAGE = {n: i for i, n in enumerate(STAGES)}
STAGE_DTYPE = {
    "TVERTEX": np.float32, "PATH_VISIBLE": np.uint8, "CURVE_COUNT": np.int32,
    "INTERSECTION": np.int32, "FRAG_KEY": np.int32, "FRAG_PID": np.uint32, "FRAG_WN": np.int8,
    "FRAG_MASK": np.uint32, "SORT_PERM": np.int32, "SORT_KEY": np.int32, "WN_SCAN": np.int8,
    "MERGED_MASK": np.uint32, "DRAW_LIST": np.int32, "IMAGE": np.uint8,
}


class SprError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: status {status}" if what else f"status {status}")


class SceneView(C.Structure):
    _fields_ = [
        ("n_paths", C.c_uint32), ("n_curves", C.c_uint32), ("n_vertices", C.c_uint32),
        ("vertex", C.c_void_p), ("vertex_path_id", C.c_void_p), ("curve_vertex_pos", C.c_void_p),
        ("curve_type", C.c_void_p), ("curve_path_id", C.c_void_p), ("curve_arc_w", C.c_void_p),
        ("path_fill_rule", C.c_void_p), ("path_fill_rgba", C.c_void_p), ("path_affine", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("samples", C.c_int32),
                ("ms_output", C.c_int32), ("srgb", C.c_int32), ("device", C.c_int32)]


class ElementNumber(C.Structure):
    _fields_ = [(n, C.c_int32) for n in
                ("path", "curve", "vertex", "curve_fragment", "merged_fragment", "span")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class FrameStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_int32), ("host_syncs", C.c_int32),
                ("resolve_pairs", C.c_int64), ("device_bytes", C.c_int64)]


class RvgInfo(C.Structure):
    _fields_ = [("viewport", C.c_float * 4), ("window", C.c_float * 4), ("width", C.c_int32),
                ("height", C.c_int32), ("n_elements", C.c_int32), ("n_gradient_paths", C.c_int32)]

    def as_dict(self):
        return {"viewport": list(self.viewport), "window": list(self.window), "width": self.width,
                "height": self.height, "n_elements": self.n_elements, "n_gradient_paths": self.n_gradient_paths}


class Tune(C.Structure):
    _fields_ = [("sort", C.c_int32), ("emit_order", C.c_int32), ("resolve_bps", C.c_int32),
                ("bin_width", C.c_int32), ("frame_ms", C.c_float), ("default_ms", C.c_float)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class VgInfo(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("n_contours", C.c_int32)]


class SvgInfo(C.Structure):
    _fields_ = [("view_box", C.c_float * 4), ("width", C.c_int32), ("height", C.c_int32),
                ("n_paths", C.c_int32), ("n_gradient_paths", C.c_int32), ("n_stroked_paths", C.c_int32)]

    def as_dict(self):
        return {"view_box": list(self.view_box), "width": self.width, "height": self.height,
                "n_paths": self.n_paths, "n_gradient_paths": self.n_gradient_paths,
                "n_stroked_paths": self.n_stroked_paths}


SVG_A128, SVG_SRGB_RAMPS, SVG_STROKE_TO_FILL = 1, 2, 4


class StrokeInfo(C.Structure):
    _fields_ = [("n_fill_paths", C.c_uint32), ("n_stroke_paths", C.c_uint32), ("n_offset_pieces", C.c_uint32),
                ("max_depth", C.c_int32)]


# spr_stroke_style: one per path
STROKE_STYLE = np.dtype([("rgba", "<u4"), ("width", "<f4")])


class SceneSpec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("seed", C.c_uint64), ("width", C.c_int32),
                ("height", C.c_int32), ("n_paths", C.c_int32), ("n_large", C.c_int32),
                ("seg_min", C.c_int32), ("seg_max", C.c_int32), ("with_rational", C.c_int32),
                ("with_affine", C.c_int32)]


class BatchScene(C.Structure):
    _fields_ = [("scene", SceneView), ("width", C.c_int32), ("height", C.c_int32), ("samples", C.c_int32),
                ("has_transform", C.c_int32), ("transform", C.c_float * 16), ("grad_table", C.c_void_p),
                ("n_grad", C.c_uint32), ("grad_ramp", C.c_void_p), ("n_ramp", C.c_uint32)]


_lib = None


def lib() -> C.CDLL:
    """Loads libspr.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with build.py "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(str(LIB_PATH))
        vp, i32, sz = C.c_void_p, C.c_int32, C.c_size_t
        L.spr_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
        L.spr_destroy.argtypes = [vp]
        L.spr_resize.argtypes = [vp, i32, i32]
        L.spr_set_samples.argtypes = [vp, i32]
        L.spr_set_multisample_output.argtypes = [vp, i32]
        L.spr_enable_srgb_correction.argtypes = [vp, i32]
        L.spr_set_scene.argtypes = [vp, C.POINTER(SceneView)]
        L.spr_set_transform.argtypes = [vp, C.POINTER(C.c_float)]
        L.spr_validate_scene.argtypes = [C.POINTER(SceneView)]
        L.spr_render.argtypes = [vp, vp]
        L.spr_image_device_ptr.argtypes = [vp, C.POINTER(vp)]
        L.spr_read_image.argtypes = [vp, vp, vp]
        L.spr_save_png.argtypes = [vp, C.c_char_p]
        L.spr_get_counts.argtypes = [vp, C.POINTER(ElementNumber)]
        L.spr_enable_step_timing.argtypes = [vp, i32]
        L.spr_step_timing.argtypes = [vp, C.POINTER(C.c_double), i32, C.POINTER(i32)]
        L.spr_get_frame_stats.argtypes = [vp, C.POINTER(FrameStats)]
        L.spr_set_memory_limit.argtypes = [vp, C.c_int64]
        L.spr_debug_set_lookback.argtypes = [vp, C.c_uint32, C.c_int64]
        L.spr_step_name.argtypes = [i32]
        L.spr_step_name.restype = C.c_char_p
        L.spr_debug_dump.argtypes = [vp, i32, vp, sz, C.POINTER(sz)]
        L.spr_selftest.argtypes = [vp, C.POINTER(C.c_int64)]
        L.spr_status_string.argtypes = [i32]
        L.spr_status_string.restype = C.c_char_p
        L.spr_scene_generate.argtypes = [C.POINTER(SceneSpec), C.POINTER(vp)]
        L.spr_scene_view_of.argtypes = [vp, C.POINTER(SceneView)]
        L.spr_scene_free.argtypes = [vp]
        L.spr_scene_free.restype = None
        L.spr_rvg_load.argtypes = [C.c_char_p, i32, C.POINTER(vp), C.POINTER(RvgInfo)]
        L.spr_rvg_parse.argtypes = [C.c_char_p, sz, i32, C.POINTER(vp), C.POINTER(RvgInfo)]
        u32p = C.POINTER(C.c_uint32)
        L.spr_scene_gradients.argtypes = [vp, C.POINTER(vp), u32p, C.POINTER(vp), u32p]
        L.spr_set_gradients.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32]
        L.spr_set_rev_transform.argtypes = [vp, C.POINTER(C.c_float)]
        L.spr_autotune.argtypes = [vp, i32, vp, C.POINTER(Tune)]
        L.spr_set_tuning.argtypes = [vp, C.POINTER(Tune)]
        L.spr_vg_load.argtypes = [C.c_char_p, C.POINTER(vp), C.POINTER(VgInfo)]
        L.spr_vg_save.argtypes = [vp, i32, i32, C.c_char_p]
        L.spr_scene_from_view.argtypes = [C.POINTER(SceneView), C.POINTER(vp)]
        L.spr_scene_set_gradients.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32]
        L.spr_set_output_transform.argtypes = [vp, C.POINTER(C.c_float)]
        L.spr_enable_output_transform.argtypes = [vp, i32]
        L.spr_output_device_ptr.argtypes = [vp, C.POINTER(vp), vp]
        L.spr_read_output.argtypes = [vp, vp, vp]
        L.spr_svg_load.argtypes = [C.c_char_p, i32, C.POINTER(vp), C.POINTER(SvgInfo)]
        L.spr_svg_parse.argtypes = [C.c_char_p, sz, i32, C.POINTER(vp), C.POINTER(SvgInfo)]
        L.spr_stroke_to_fill.argtypes = [C.POINTER(SceneView), vp, C.POINTER(vp), C.POINTER(StrokeInfo)]
        L.spr_set_graph_replay.argtypes = [vp, i32]
        L.spr_graph_replays.argtypes = [vp, C.POINTER(i32)]
        L.spr_batch_set_graph_replay.argtypes = [vp, i32]
        L.spr_update_vertices.argtypes = [vp, vp, vp]
        L.spr_batch_diff_render.argtypes = [vp, vp, vp, vp]
        L.spr_batch_diff_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.spr_batch_update_vertices.argtypes = [vp, vp, vp]
        L.spr_diff_render.argtypes = [vp, vp, vp, vp]
        L.spr_diff_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.spr_batch_create.argtypes = [i32, i32, i32, C.POINTER(vp)]
        L.spr_batch_destroy.argtypes = [vp]
        L.spr_batch_set_scenes.argtypes = [vp, C.POINTER(BatchScene), i32]
        L.spr_batch_render.argtypes = [vp, vp]
        L.spr_batch_image_device_ptr.argtypes = [vp, i32, C.POINTER(vp)]
        L.spr_batch_read_image.argtypes = [vp, i32, vp, vp]
        L.spr_batch_get_counts.argtypes = [vp, C.POINTER(ElementNumber)]
        L.spr_batch_get_frame_stats.argtypes = [vp, C.POINTER(FrameStats)]
        L.spr_batch_enable_step_timing.argtypes = [vp, i32]
        L.spr_batch_step_timing.argtypes = [vp, C.POINTER(C.c_double), i32, C.POINTER(i32)]
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != OK:
        msg = lib().spr_status_string(status).decode()
        raise SprError(status, f"{what} ({msg})" if what else msg)


def _ptr(a):
    return None if a is None else a.ctypes.data


class Scene:
    """A host scene in the reference's SoA layout (numpy arrays).

    Construct from arrays, or with :meth:`generate` from a seeded synthetic
    spec.  :meth:`view` returns the C view (the arrays stay owned here).
    """

    FIELDS = ("vertex", "vertex_path_id", "curve_vertex_pos", "curve_type", "curve_path_id",
              "curve_arc_w", "path_fill_rule", "path_fill_rgba", "path_affine")

    def __init__(self, vertex, vertex_path_id, curve_vertex_pos, curve_type, curve_path_id,
                 curve_arc_w, path_fill_rule, path_fill_rgba, path_affine=None):
        self.vertex = np.ascontiguousarray(vertex, dtype=np.float32).reshape(-1, 2)
        self.vertex_path_id = np.ascontiguousarray(vertex_path_id, dtype=np.uint32)
        self.curve_vertex_pos = np.ascontiguousarray(curve_vertex_pos, dtype=np.uint32)
        self.curve_type = np.ascontiguousarray(curve_type, dtype=np.uint8)
        self.curve_path_id = np.ascontiguousarray(curve_path_id, dtype=np.uint32)
        self.curve_arc_w = np.ascontiguousarray(curve_arc_w, dtype=np.float32)
        self.path_fill_rule = np.ascontiguousarray(path_fill_rule, dtype=np.uint8)
        self.path_fill_rgba = np.ascontiguousarray(path_fill_rgba, dtype=np.uint32)
        self.path_affine = (None if path_affine is None else
                            np.ascontiguousarray(path_affine, dtype=np.float32).reshape(-1, 6))
        # gradient paints: (table uint32[12 * entries], ramp uint32[texels]) or None
        self.gradients = None

    @property
    def n_paths(self):
        return len(self.path_fill_rule)

    @property
    def n_curves(self):
        return len(self.curve_type)

    @property
    def n_vertices(self):
        return len(self.vertex)

    def view(self) -> SceneView:
        return SceneView(self.n_paths, self.n_curves, self.n_vertices, _ptr(self.vertex),
                         _ptr(self.vertex_path_id), _ptr(self.curve_vertex_pos),
                         _ptr(self.curve_type), _ptr(self.curve_path_id), _ptr(self.curve_arc_w),
                         _ptr(self.path_fill_rule), _ptr(self.path_fill_rgba),
                         _ptr(self.path_affine))

    def validate(self) -> int:
        """Host-side scene checks of spr_set_scene; returns the status code."""
        v = self.view()
        return lib().spr_validate_scene(C.byref(v))

    def copy(self) -> "Scene":
        s = Scene(*[None if getattr(self, f) is None else getattr(self, f).copy() for f in self.FIELDS])
        if self.gradients is not None:
            s.gradients = tuple(x.copy() for x in self.gradients)
        return s

    @classmethod
    def generate(cls, kind=SCENE_RANDOM, seed=1, width=512, height=512, n_paths=64, n_large=0,
                 seg_min=8, seg_max=32, with_rational=False, with_affine=False) -> "Scene":
        spec = SceneSpec(kind, seed, width, height, n_paths, n_large, seg_min, seg_max,
                         int(with_rational), int(with_affine))
        h = C.c_void_p()
        check(lib().spr_scene_generate(C.byref(spec), C.byref(h)), "spr_scene_generate")
        return cls._take(h)

    @classmethod
    def load_rvg(cls, path, a128=False, srgb_ramps=True):
        """An RVG document (RVG::load): returns (scene, info dict); gradient
        paints in ``scene.gradients``."""
        h, info = C.c_void_p(), RvgInfo()
        flags = (RVG_A128 if a128 else 0) | (RVG_SRGB_RAMPS if srgb_ramps else 0)
        check(lib().spr_rvg_load(str(path).encode(), flags, C.byref(h), C.byref(info)), "spr_rvg_load")
        return cls._take(h), info.as_dict()

    @classmethod
    def parse_rvg(cls, text, a128=False, srgb_ramps=True):
        """An RVG document from a string: returns (scene, info dict)."""
        b = text.encode() if isinstance(text, str) else bytes(text)
        h, info = C.c_void_p(), RvgInfo()
        flags = (RVG_A128 if a128 else 0) | (RVG_SRGB_RAMPS if srgb_ramps else 0)
        check(lib().spr_rvg_parse(b, len(b), flags, C.byref(h), C.byref(info)), "spr_rvg_parse")
        return cls._take(h), info.as_dict()

    @classmethod
    def load_vg(cls, path):
        """A .vgb / .vgt scene file (VGContainer::load): returns (scene, info dict)."""
        h, info = C.c_void_p(), VgInfo()
        check(lib().spr_vg_load(str(path).encode(), C.byref(h), C.byref(info)), "spr_vg_load")
        return cls._take(h), {n: int(getattr(info, n)) for n, _ in VgInfo._fields_}

    def save_vg(self, path, width, height):
        """Writes the scene as a .vgb / .vgt file (by the suffix)."""
        h = C.c_void_p()
        check(lib().spr_scene_from_view(C.byref(self.view()), C.byref(h)), "spr_scene_from_view")
        try:
            if self.gradients is not None:
                t, r = (np.ascontiguousarray(x, dtype=np.uint32) for x in self.gradients)
                check(lib().spr_scene_set_gradients(h, t.ctypes.data, len(t) // 12, r.ctypes.data, len(r)),
                      "spr_scene_set_gradients")
            check(lib().spr_vg_save(h, int(width), int(height), str(path).encode()), "spr_vg_save")
        finally:
            lib().spr_scene_free(h)

    @staticmethod
    def _svg_flags(a128, srgb_ramps, stroke_to_fill):
        return ((SVG_A128 if a128 else 0) | (SVG_SRGB_RAMPS if srgb_ramps else 0) |
                (SVG_STROKE_TO_FILL if stroke_to_fill else 0))

    @classmethod
    def load_svg(cls, path, a128=False, srgb_ramps=True, stroke_to_fill=False):
        """An SVG document (SVG::load + addVg): returns (scene, info dict)."""
        h, info = C.c_void_p(), SvgInfo()
        check(lib().spr_svg_load(str(path).encode(), cls._svg_flags(a128, srgb_ramps, stroke_to_fill),
                                 C.byref(h), C.byref(info)), "spr_svg_load")
        return cls._take(h), info.as_dict()

    @classmethod
    def parse_svg(cls, text, a128=False, srgb_ramps=True, stroke_to_fill=False):
        """An SVG document from a string: returns (scene, info dict)."""
        b = text.encode() if isinstance(text, str) else bytes(text)
        h, info = C.c_void_p(), SvgInfo()
        check(lib().spr_svg_parse(b, len(b), cls._svg_flags(a128, srgb_ramps, stroke_to_fill), C.byref(h),
                                  C.byref(info)), "spr_svg_parse")
        return cls._take(h), info.as_dict()

    def stroke_to_fill(self, rgba, width):
        """Stroke-to-fill (spr_stroke_to_fill): rgba and width per path (or
        one value for all).  Returns (scene, info dict); the gradient paints
        carry over."""
        n = self.n_paths
        st = np.zeros(n, dtype=STROKE_STYLE)
        st["rgba"] = np.broadcast_to(np.asarray(rgba, dtype=np.uint32), (n,))
        st["width"] = np.broadcast_to(np.asarray(width, dtype=np.float32), (n,))
        h, info = C.c_void_p(), StrokeInfo()
        check(lib().spr_stroke_to_fill(C.byref(self.view()), st.ctypes.data, C.byref(h), C.byref(info)),
              "spr_stroke_to_fill")
        out = Scene._take(h)
        out.gradients = self.gradients
        return out, {k: int(getattr(info, k)) for k, _ in StrokeInfo._fields_}

    @classmethod
    def _take(cls, h) -> "Scene":
        """Copies a library-owned scene into numpy arrays and frees it."""
        try:
            v = SceneView()
            check(lib().spr_scene_view_of(h, C.byref(v)), "spr_scene_view_of")

            def arr(p, n, dt):
                if not p or n == 0:
                    return np.zeros(n, dtype=dt)
                return np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                             (n,)).copy()
            s = cls(arr(v.vertex, 2 * v.n_vertices, np.float32),
                    arr(v.vertex_path_id, v.n_vertices, np.uint32),
                    arr(v.curve_vertex_pos, v.n_curves, np.uint32),
                    arr(v.curve_type, v.n_curves, np.uint8),
                    arr(v.curve_path_id, v.n_curves, np.uint32),
                    arr(v.curve_arc_w, v.n_curves, np.float32),
                    arr(v.path_fill_rule, v.n_paths, np.uint8),
                    arr(v.path_fill_rgba, v.n_paths, np.uint32),
                    None if not v.path_affine else arr(v.path_affine, 6 * v.n_paths, np.float32))
            tp, rp, nt, nr = C.c_void_p(), C.c_void_p(), C.c_uint32(), C.c_uint32()
            check(lib().spr_scene_gradients(h, C.byref(tp), C.byref(nt), C.byref(rp), C.byref(nr)),
                  "spr_scene_gradients")
            if nt.value and s.path_fill_rgba.size and np.any(s.path_fill_rgba - 1 < 0x01000000):
                s.gradients = (arr(tp.value, 12 * nt.value, np.uint32), arr(rp.value, nr.value, np.uint32))
        finally:
            lib().spr_scene_free(h)
        return s


class VGRasterizer:
    """Mirror of RasterizerBase::VGRasterizer over the C ABI."""

    def __init__(self, width=512, height=512, samples=8, ms_output=True, srgb=True, device=0):
        cfg = Config(width, height, samples, int(ms_output), int(srgb), device)
        h = C.c_void_p()
        check(lib().spr_create(C.byref(cfg), C.byref(h)), "spr_create")
        self._h = h
        self.width, self.height, self.samples = width, height, samples
        self._scene = None

    def close(self):
        if self._h:
            lib().spr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration -------------------------------------------------------
    def resize_output_buffer(self, width, height):
        check(lib().spr_resize(self._h, width, height), "spr_resize")
        self.width, self.height = width, height

    def set_samples(self, s):
        check(lib().spr_set_samples(self._h, s), "spr_set_samples")
        self.samples = s

    def set_multisample_output(self, f):
        check(lib().spr_set_multisample_output(self._h, int(f)), "spr_set_multisample_output")

    def enable_srgb_correction(self, f=True):
        check(lib().spr_enable_srgb_correction(self._h, int(f)), "spr_enable_srgb_correction")

    # -- scene and frame -----------------------------------------------------
    def add_vg(self, scene: Scene):
        """The scene, and its gradient paints when it has them."""
        v = scene.view()
        check(lib().spr_set_scene(self._h, C.byref(v)), "spr_set_scene")
        self._scene = scene
        self.set_gradients(scene.gradients)

    def set_gradients(self, gradients):
        """(table uint32[12 * entries], ramp uint32[texels]) or None."""
        if gradients is None:
            check(lib().spr_set_gradients(self._h, None, 0, None, 0), "spr_set_gradients")
            self._grad = None
            return
        table, ramp = (np.ascontiguousarray(x, dtype=np.uint32) for x in gradients)
        check(lib().spr_set_gradients(self._h, table.ctypes.data, len(table) // 12, ramp.ctypes.data, len(ramp)),
              "spr_set_gradients")
        self._grad = (table, ramp)

    def autotune(self, frames=3, stream=None) -> dict:
        """Times the launch choices on the current scene and keeps the fastest."""
        t = Tune()
        check(lib().spr_autotune(self._h, int(frames), stream, C.byref(t)), "spr_autotune")
        return t.as_dict()

    def set_tuning(self, sort=-1, emit_order=-1, resolve_bps=0, bin_width=0):
        t = Tune(sort, emit_order, resolve_bps, bin_width, 0.0, 0.0)
        check(lib().spr_set_tuning(self._h, C.byref(t)), "spr_set_tuning")

    def set_rev_transform(self, ctx):
        c = np.ascontiguousarray(ctx, dtype=np.float32).reshape(13)
        check(lib().spr_set_rev_transform(self._h, c.ctypes.data_as(C.POINTER(C.c_float))), "spr_set_rev_transform")

    def set_input_transform(self, m):
        m = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
        check(lib().spr_set_transform(self._h, m.ctypes.data_as(C.POINTER(C.c_float))),
              "spr_set_transform")

    def rasterize(self, stream=None):
        check(lib().spr_render(self._h, stream), "spr_render")

    def image_device_ptr(self) -> int:
        p = C.c_void_p()
        check(lib().spr_image_device_ptr(self._h, C.byref(p)), "spr_image_device_ptr")
        return p.value or 0

    def read_image(self, out=None, stream=None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        check(lib().spr_read_image(self._h, out.ctypes.data, stream), "spr_read_image")
        return out

    def save_output_to_file(self, path):
        check(lib().spr_save_png(self._h, os.fsencode(str(path))), "spr_save_png")

    def set_output_transform(self, m):
        """setOutputTransform: row-major 4x4 (the zoomed view, read_output)."""
        a = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
        check(lib().spr_set_output_transform(self._h, a.ctypes.data_as(C.POINTER(C.c_float))),
              "spr_set_output_transform")

    def enable_output_transform(self, f=True):
        check(lib().spr_enable_output_transform(self._h, int(bool(f))), "spr_enable_output_transform")

    def read_output(self, out=None, stream=None) -> np.ndarray:
        """The output view of the last image (the image itself when the
        output transform is off)."""
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        check(lib().spr_read_output(self._h, out.ctypes.data, stream), "spr_read_output")
        return out

    def element_number(self) -> dict:
        e = ElementNumber()
        check(lib().spr_get_counts(self._h, C.byref(e)), "spr_get_counts")
        return e.as_dict()

    def enable_step_timing(self, f=True):
        check(lib().spr_enable_step_timing(self._h, int(f)), "spr_enable_step_timing")

    def step_timing(self) -> dict:
        buf = (C.c_double * 64)()
        n = C.c_int32()
        check(lib().spr_step_timing(self._h, buf, 64, C.byref(n)), "spr_step_timing")
        return {lib().spr_step_name(i).decode(): buf[i] for i in range(n.value)}

    def debug_set_lookback(self, spin_cap=1 << 24, hold_tile=-1):
        """Test hook of the bounded look-back waits: polls before a wait gives
        up, and a tile of the entry-offset scan that never publishes."""
        check(lib().spr_debug_set_lookback(self._h, int(spin_cap), int(hold_tile)), "spr_debug_set_lookback")

    def set_memory_limit(self, nbytes: int):
        """Cap on the handle's device memory (0 = none); a frame that would
        need more raises SprError(ERR_OUT_OF_MEMORY) and the handle stays
        usable."""
        check(lib().spr_set_memory_limit(self._h, int(nbytes)), "spr_set_memory_limit")

    def frame_stats(self) -> dict:
        st = FrameStats()
        check(lib().spr_get_frame_stats(self._h, C.byref(st)), "spr_get_frame_stats")
        return {n: int(getattr(st, n)) for n, _ in FrameStats._fields_}

    def selftest(self) -> dict:
        n = C.c_int64()
        check(lib().spr_selftest(self._h, C.byref(n)), "spr_selftest")
        return {"srgb_encode_mismatches": int(n.value)}

    def set_graph_replay(self, f=True):
        check(lib().spr_set_graph_replay(self._h, int(f)), "spr_set_graph_replay")

    def graph_replays(self) -> int:
        n = C.c_int32()
        check(lib().spr_graph_replays(self._h, C.byref(n)), "spr_graph_replays")
        return int(n.value)

    def update_vertices(self, vertex_ptr: int, stream=None):
        """New vertex positions (pointer to float32[V, 2], host or device)."""
        check(lib().spr_update_vertices(self._h, vertex_ptr, stream), "spr_update_vertices")

    def diff_render(self, fill_ptr: int, image_ptr: int, stream=None):
        """Float composite with per-path linear RGBA fills (device pointers:
        fill float32[P, 4], image float32[H, W, 4])."""
        check(lib().spr_diff_render(self._h, fill_ptr, image_ptr, stream), "spr_diff_render")

    def diff_backward(self, fill_ptr: int, grad_image_ptr: int, grad_fill_ptr: int, grad_vertex_ptr: int,
                      grad_affine_ptr=None, stream=None):
        """Gradients (device pointers: grad_fill float32[P, 4], grad_vertex
        float32[V, 2], grad_affine float32[P, 6] or None)."""
        check(lib().spr_diff_backward(self._h, fill_ptr, grad_image_ptr, grad_fill_ptr, grad_vertex_ptr,
                                      grad_affine_ptr, stream), "spr_diff_backward")

    def dump(self, stage) -> np.ndarray:
        sid = STAGE[stage] if isinstance(stage, str) else int(stage)
        name = STAGES[sid]
        need = C.c_size_t()
        check(lib().spr_debug_dump(self._h, sid, None, 0, C.byref(need)), f"spr_debug_dump({name})")
        dt = np.dtype(STAGE_DTYPE[name])
        out = np.empty(need.value // dt.itemsize, dtype=dt)
        if need.value:
            check(lib().spr_debug_dump(self._h, sid, out.ctypes.data, need.value, C.byref(need)),
                  f"spr_debug_dump({name})")
        return out


class Batch:
    """Many independent scenes rendered together (spr_batch_*).

    ``set_scenes`` takes a list of ``(scene, width, height, samples)`` or
    ``(scene, width, height, samples, transform)`` tuples; image ``i`` of
    ``read_image(i)`` is the one a :class:`VGRasterizer` with the same
    settings renders for scene ``i``.
    """

    def __init__(self, ms_output=True, srgb=True, device=0):
        self._h = C.c_void_p()
        check(lib().spr_batch_create(device, int(ms_output), int(srgb), C.byref(self._h)), "spr_batch_create")
        self._sizes = []
        self._keep = []

    def close(self):
        if self._h:
            lib().spr_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_scenes(self, items):
        arr = (BatchScene * max(len(items), 1))()
        keep = []
        for i, it in enumerate(items):
            scene, w, h, smp = it[:4]
            tf = it[4] if len(it) > 4 else None
            arr[i].scene = scene.view()
            keep.append(scene)
            if scene.gradients is not None:
                t, r = (np.ascontiguousarray(x, dtype=np.uint32) for x in scene.gradients)
                keep += [t, r]
                arr[i].grad_table, arr[i].n_grad = t.ctypes.data, len(t) // 12
                arr[i].grad_ramp, arr[i].n_ramp = r.ctypes.data, len(r)
            arr[i].width, arr[i].height, arr[i].samples = int(w), int(h), int(smp)
            arr[i].has_transform = 0 if tf is None else 1
            if tf is not None:
                m = np.ascontiguousarray(tf, dtype=np.float32).reshape(16)
                for j in range(16):
                    arr[i].transform[j] = float(m[j])
        check(lib().spr_batch_set_scenes(self._h, arr, len(items)), "spr_batch_set_scenes")
        self._sizes = [(int(it[1]), int(it[2])) for it in items]
        self._keep = keep

    def render(self, stream=None):
        check(lib().spr_batch_render(self._h, stream), "spr_batch_render")

    def image_device_ptr(self, i) -> int:
        p = C.c_void_p()
        check(lib().spr_batch_image_device_ptr(self._h, i, C.byref(p)), "spr_batch_image_device_ptr")
        return p.value or 0

    def read_image(self, i, out=None, stream=None) -> np.ndarray:
        if not 0 <= i < len(self._sizes):
            raise SprError(ERR_INVALID_ARG, f"spr_batch_read_image: no scene {i}")
        w, h = self._sizes[i]
        if out is None:
            out = np.empty((h, w, 4), dtype=np.uint8)
        check(lib().spr_batch_read_image(self._h, i, out.ctypes.data, stream), "spr_batch_read_image")
        return out

    def element_number(self) -> dict:
        e = ElementNumber()
        check(lib().spr_batch_get_counts(self._h, C.byref(e)), "spr_batch_get_counts")
        return e.as_dict()

    def debug_set_lookback(self, spin_cap=1 << 24, hold_tile=-1):
        """Test hook of the bounded look-back waits: polls before a wait gives
        up, and a tile of the entry-offset scan that never publishes."""
        check(lib().spr_debug_set_lookback(self._h, int(spin_cap), int(hold_tile)), "spr_debug_set_lookback")

    def set_memory_limit(self, nbytes: int):
        """Cap on the handle's device memory (0 = none); a frame that would
        need more raises SprError(ERR_OUT_OF_MEMORY) and the handle stays
        usable."""
        check(lib().spr_set_memory_limit(self._h, int(nbytes)), "spr_set_memory_limit")

    def frame_stats(self) -> dict:
        st = FrameStats()
        check(lib().spr_batch_get_frame_stats(self._h, C.byref(st)), "spr_batch_get_frame_stats")
        return {n: int(getattr(st, n)) for n, _ in FrameStats._fields_}

    def set_graph_replay(self, f=True):
        check(lib().spr_batch_set_graph_replay(self._h, int(f)), "spr_batch_set_graph_replay")

    def image_offsets(self):
        """First pixel of every scene's image in the concatenated image of a
        single-sample-count batch (scene order)."""
        import numpy as _np
        return _np.concatenate([[0], _np.cumsum([w * h for w, h in self._sizes])]).astype(_np.int64)

    def diff_render(self, fill_ptr: int, image_ptr: int, stream=None):
        check(lib().spr_batch_diff_render(self._h, fill_ptr, image_ptr, stream), "spr_batch_diff_render")

    def diff_backward(self, fill_ptr: int, grad_image_ptr: int, grad_fill_ptr: int, grad_vertex_ptr: int,
                      grad_affine_ptr=None, stream=None):
        check(lib().spr_batch_diff_backward(self._h, fill_ptr, grad_image_ptr, grad_fill_ptr, grad_vertex_ptr,
                                            grad_affine_ptr, stream), "spr_batch_diff_backward")

    def update_vertices(self, vertex_ptr: int, stream=None):
        check(lib().spr_batch_update_vertices(self._h, vertex_ptr, stream), "spr_batch_update_vertices")

    def enable_step_timing(self, f=True):
        check(lib().spr_batch_enable_step_timing(self._h, int(f)), "spr_batch_enable_step_timing")

    def step_timing(self) -> dict:
        buf = (C.c_double * 64)()
        n = C.c_int32()
        check(lib().spr_batch_step_timing(self._h, buf, 64, C.byref(n)), "spr_batch_step_timing")
        return {lib().spr_step_name(i).decode(): buf[i] for i in range(n.value)}
