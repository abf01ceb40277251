"""Tile sampling as wndchrm does it (remainder dropped, x-major order)."""
import numpy as np

import synth_loader  # noqa: F401
import wndcharm


def test_tiles_layout():
    a = np.arange(11 * 10).reshape(11, 10)  # H = 11, W = 10
    t = wndcharm.tiles(a, 4, 3)  # tw = 2, th = 3
    assert len(t) == 12 and all(x.shape == (3, 2) for x in t)
    # ix outer, iy inner
    np.testing.assert_array_equal(t[0], a[0:3, 0:2])
    np.testing.assert_array_equal(t[1], a[3:6, 0:2])
    np.testing.assert_array_equal(t[3], a[0:3, 2:4])
    np.testing.assert_array_equal(t[11], a[6:9, 6:8])
