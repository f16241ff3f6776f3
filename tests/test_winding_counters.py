"""The merged-mask pass's two forms of the per-sample winding counters, on
the CPU: the packed 8-bit counters (four per 32-bit word, one word per mask
bit position b of a mask word, as the reference keeps them) and the
bit-sliced 7-bit counters the CUDA pass uses, which must give the same
merged mask bits whenever |w0| + (fragments) <= 127.  Pure host arithmetic
(numpy uint32, wrapping like the device's 32-bit registers)."""
import numpy as np
import pytest


def packed(w0, frags, fill_rule):
    """Merged mask word of one mask word position: frags = [(chg, mask)]."""
    init = (0x01010101 * (w0 & 0xFFFFFFFF)) & 0xFFFFFFFF
    acc = [init] * 8
    for chg, m in frags:
        for b in range(8):
            bits = (m >> b) & 0x01010101
            acc[b] = (acc[b] + bits) & 0xFFFFFFFF if chg > 0 else (acc[b] - bits) & 0xFFFFFFFF
    ret = 0
    for b in range(8):
        wv = ((0x80808080 + acc[b]) & 0xFFFFFFFF) & 0x7F7F7F7F
        if fill_rule == 0:
            wv |= wv >> 4
            wv |= wv >> 2
            wv |= wv >> 1
        ret |= (wv & 0x01010101) << b
    return ret


def bitsliced(w0, frags, fill_rule):
    pl = [0xFFFFFFFF if ((w0 & 0xFFFFFFFF) >> q) & 1 else 0 for q in range(7)]
    for chg, m in frags:
        c = m
        for q in range(7):
            t = (pl[q] & c) if chg > 0 else (~pl[q] & 0xFFFFFFFF & c)
            pl[q] ^= c
            c = t
    if fill_rule == 0:
        r = 0
        for q in range(7):
            r |= pl[q]
        return r
    return pl[0]


@pytest.mark.parametrize("seed", range(4))
def test_bitsliced_counters_equal_packed_in_range(seed):
    rng = np.random.default_rng(seed)
    checked = 0
    for _ in range(3000):
        k = int(rng.integers(1, 24))
        w0 = int(rng.integers(-128, 128))
        if abs(w0) + k > 127:
            continue
        frags = [(int(rng.choice([-1, 1])), int(rng.integers(0, 2**32))) for _ in range(k)]
        for fr in (0, 1):
            assert bitsliced(w0, frags, fr) == packed(w0, frags, fr), (w0, frags, fr)
        checked += 1
    assert checked > 1000


def test_windings_near_the_int8_edge():
    """|w0| + k = 127 exactly, all fragments covering every sample in the
    same direction: both forms agree at the edge of the range."""
    for w0, chg in ((120, 1), (-120, -1), (-127, 0), (127, 0)):
        frags = [(chg, 0xFFFFFFFF)] * (127 - abs(w0)) if chg else []
        for fr in (0, 1):
            assert bitsliced(w0, frags, fr) == packed(w0, frags, fr)
