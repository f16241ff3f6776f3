"""End-to-end parity of the CUDA path against the CPU oracle on small scenes."""
import numpy as np
import pytest

import oracle
import spr

pytestmark = pytest.mark.gpu


def test_smoke():
    import __graft_entry__

    __graft_entry__.smoke()


def test_srgb_encode_selftest():
    with spr.VGRasterizer(64, 64, samples=8) as r:
        assert r.selftest()["srgb_encode_mismatches"] == 0
