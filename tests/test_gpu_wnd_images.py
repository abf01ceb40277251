"""wc_wnd_classify_images (TrainingSet::ClassifyImage with WND-5) on the GPU:
against the oracle and the reference, both tile rules and both forms, and
against the plain per-row classification averaged on the host."""
import numpy as np
import pytest

from conftest import golden, oracle_lib
import synth_loader  # noqa: F401
from test_wnd_images_cpu import inputs, oracle_wnd_images

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("max_tile", [0, 1])
def test_classify_images(prec, max_tile):
    import wndcharm
    g = golden("reference_wnd_images.npz")
    xtr, ytr, xte, _ = inputs()
    eng = wndcharm.Engine(0, prec)
    w, mn, mx = eng.wnd_fit(xtr, ytr, 6, 0.15)
    p, pr, nf = eng.wnd_classify_images(xtr, ytr, 6, w, mn, mx, xte, 4, max_tile=bool(max_tile))
    op, opr, onf = oracle_wnd_images(oracle_lib(), xtr, ytr, xte, 6, 0.15, 4, max_tile)
    np.testing.assert_array_equal(pr, opr)
    np.testing.assert_array_equal(pr, g["pred_max_tile%d" % max_tile])
    # FP64 form: the reference's arithmetic; mixed form (distances on the tensor
    # cores): the stated WND tolerance, probabilities within 1e-6
    atol, nrtol = (1e-12, 1e-9) if prec == "fp64" else (1e-6, 1e-6)
    np.testing.assert_allclose(p, op, rtol=0, atol=atol)
    np.testing.assert_allclose(p, g["probs_max_tile%d" % max_tile], rtol=0, atol=atol)
    np.testing.assert_allclose(nf, onf, rtol=nrtol)
    if not max_tile:
        pt, prt = eng.wnd_classify(xtr, ytr, 6, w, mn, mx, xte)
        avg = np.zeros((12, 6))
        for k in range(4):  # tile order, each tile's row divided by the tile count
            avg += pt.reshape(12, 4, 6)[:, k, :] / 4.0
        np.testing.assert_array_equal(p, avg)


def test_classify_images_rejects_bad_tiles():
    import wndcharm
    xtr, ytr, xte, _ = inputs()
    eng = wndcharm.Engine(0, "fp64")
    w, mn, mx = eng.wnd_fit(xtr, ytr, 6, 0.15)
    with pytest.raises(wndcharm.WndcharmError):
        eng.wnd_classify_images(xtr, ytr, 6, w, mn, mx, xte[:47], 4)
