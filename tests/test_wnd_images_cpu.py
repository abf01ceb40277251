"""Per-image classification over tiles (TrainingSet::ClassifyImage, WND-5):
the oracle against the reference's own results, bit for bit, with and
without the most-similar-tile rule."""
import ctypes

import numpy as np
import pytest

from conftest import golden, oracle_lib
import synth_loader  # noqa: F401

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)


def oracle_wnd_images(lib, xtr, ytr, xte, C, frac, tiles, max_tile):
    n_img = xte.shape[0] // tiles
    p, pr, nf = np.zeros((n_img, C)), np.zeros(n_img, dtype=np.int32), np.zeros(n_img)
    lib.wco_wnd_images(np.ascontiguousarray(xtr, dtype=np.float64).ctypes.data_as(D), xtr.shape[0], xtr.shape[1],
                       np.ascontiguousarray(ytr, dtype=np.int32).ctypes.data_as(I), C, ctypes.c_double(frac),
                       np.ascontiguousarray(xte, dtype=np.float64).ctypes.data_as(D), n_img, tiles, max_tile,
                       p.ctypes.data_as(D), pr.ctypes.data_as(I), nf.ctypes.data_as(D))
    return p, pr, nf


def inputs():
    from wndcharm import synth
    return synth.feature_vectors(200, 48, 2919, 6, 7)


@pytest.mark.parametrize("max_tile", [0, 1])
def test_oracle_classify_images_matches_reference(max_tile):
    g = golden("reference_wnd_images.npz")
    xtr, ytr, xte, _ = inputs()
    p, pr, nf = oracle_wnd_images(oracle_lib(), xtr, ytr, xte, 6, 0.15, 4, max_tile)
    np.testing.assert_array_equal(pr, g["pred_max_tile%d" % max_tile])
    np.testing.assert_array_equal(p, g["probs_max_tile%d" % max_tile])
    assert (nf > 0).all()


def test_one_tile_per_image_is_plain_classify2():
    """tiles = 1: the per-image results are classify2's own."""
    from conftest import oracle_wnd
    xtr, ytr, xte, _ = inputs()
    lib = oracle_lib()
    p, pr, _ = oracle_wnd_images(lib, xtr, ytr, xte, 6, 0.15, 1, 0)
    _, _, _, p1, pr1 = oracle_wnd(lib, xtr, ytr, xte, 6, 0.15)
    np.testing.assert_array_equal(p, p1)
    np.testing.assert_array_equal(pr, pr1)
