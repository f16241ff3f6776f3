"""The allocation-free scan entry point (spr_scan_offsets_noalloc).

Some callers cannot allocate device memory while they work -- plugin hosts
that hand out all device memory from their own pools, and real-time loops
that must not call cudaMalloc / cudaFree -- so the library offers this one
entry point whose scratch is a fixed array compiled into the library.  This
test calls it through the C ABI on caller-owned device buffers and checks its
output against what the regular render entry point produced for the same
curves: the offsets at which spr_render placed each curve's intersection
entries.  It makes two calls in a row on different inputs (the scratch keeps
the previous call's contents) and checks the size limit.

The file name makes pytest collect it after every other test file.
"""
import ctypes as C

import numpy as np
import pytest

import spr

pytestmark = pytest.mark.gpu

MAX_N = 16384 * 2048


def _entry():
    f = spr.lib().spr_scan_offsets_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    f.restype = C.c_int
    return f


def _render_offsets(seed, size):
    """Per-curve counts and entry offsets from the regular render path."""
    scene = spr.Scene.generate(spr.SCENE_RANDOM, seed=seed, width=size, height=size, n_paths=24,
                               seg_min=4, seg_max=16)
    with spr.VGRasterizer(size, size, samples=8) as r:
        r.add_vg(scene)
        r.rasterize()
        counts = r.dump("CURVE_COUNT").view(np.uint32)
        entries = r.dump("INTERSECTION").reshape(-1, 2)
    # entries are laid out curve by curve; curve c starts at its offset
    first = np.searchsorted(entries[:, 0], np.arange(len(counts)), side="left")
    expected = np.append(first, len(entries)).astype(np.uint32)
    return counts, expected


def _noalloc(counts):
    import torch

    d_in = torch.from_numpy(counts.view(np.int32).copy()).cuda()
    d_out = torch.full((len(counts) + 1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = _entry()(d_in.data_ptr(), d_out.data_ptr(), len(counts), stream.cuda_stream)
    assert st == spr.OK, spr.lib().spr_status_string(st)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint32)


def test_noalloc_scan_matches_render_offsets_two_calls():
    """Two calls in a row on the curves of two scenes against the offsets at
    which spr_render placed each curve's intersection entries."""
    for seed, size in ((11, 256), (12, 384)):
        counts, expected = _render_offsets(seed, size)
        got = _noalloc(counts)
        np.testing.assert_array_equal(got, expected)


def _expected(counts):
    return np.concatenate([[0], np.cumsum(counts, dtype=np.uint64)]).astype(np.uint32)


def test_noalloc_scan_synthetic_sizes_in_a_row():
    """Synthetic counts against np.cumsum, one call after another on the
    shared scratch: nothing, one count, more than 1,024 tiles of 2,048 counts
    (the tile-sum scan then carries across its 1,024-tile chunks), a smaller
    multi-tile input right after it (so stale tile sums of the larger call
    lie beyond its end), and exactly the maximum size."""
    rng = np.random.default_rng(5)
    for n in (0, 1, 2048 * 1100 + 7, 3 * 2048 + 5, MAX_N, 2047):
        counts = rng.integers(0, 64, n, dtype=np.uint32)  # totals stay below 2^32
        got = _noalloc(counts)
        np.testing.assert_array_equal(got, _expected(counts), err_msg=f"n = {n}")


def test_noalloc_scan_rejects_oversize():
    st = _entry()(C.c_void_p(8), C.c_void_p(8), MAX_N + 1, None)
    assert st == spr.ERR_CAPACITY_EXCEEDED
