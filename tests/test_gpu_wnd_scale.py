"""WND-5 at the full classification scale: 100,000 training vectors x 2919
features, 10 classes, 10,000 test vectors (per-feature N(mu_cf, 1), class means
N(0, 0.5), seed 4).  The GPU fit and classification run on all of it; the
oracle (same algorithm on the CPU) classifies the first 100 test vectors
against the same training set: predicted classes identical, marginal
probabilities within 1e-6."""
import time

import numpy as np
import pytest

from conftest import oracle_lib, oracle_wnd
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


def test_wnd_full_scale():
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, yte = synth.feature_vectors(100000, 10000, 2919, 10, 4)
    eng = wndcharm.Engine(0, "fp64")
    t0 = time.perf_counter()
    w, mn, mx = eng.wnd_fit(xtr, ytr, 10, 0.15)
    t1 = time.perf_counter()
    p, pred = eng.wnd_classify(xtr, ytr, 10, w, mn, mx, xte)
    t2 = time.perf_counter()
    kept = int((w >= np.finfo(np.float64).eps).sum())
    print("fit %.2f s, classify %.2f s (%d x %d x %d selected features)" % (t1 - t0, t2 - t1, 10000, 100000, kept))
    assert p.shape == (10000, 10)
    np.testing.assert_allclose(p.sum(axis=1), 1.0, atol=1e-12)
    assert (pred >= 1).all() and (pred <= 10).all()
    assert (pred == yte).mean() > 0.9  # the synthetic classes are well separated
    lib = oracle_lib()
    ow, omn, omx, op, opred = oracle_wnd(lib, xtr, ytr, xte[:100], 10, 0.15)
    np.testing.assert_allclose(w, ow, rtol=1e-12, atol=0)
    np.testing.assert_array_equal(mn, omn)
    np.testing.assert_array_equal(mx, omx)
    np.testing.assert_array_equal(pred[:100], opred)
    np.testing.assert_allclose(p[:100], op, rtol=0, atol=1e-6)


def test_wnd_full_scale_mixed_matches_fp64():
    """The mixed form (distances on the tensor cores, uncertified rows
    recomputed in FP64) at full scale: predicted classes identical to the FP64
    form, marginal probabilities within 1e-6."""
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, yte = synth.feature_vectors(100000, 10000, 2919, 10, 4)
    e64, emx = wndcharm.Engine(0, "fp64"), wndcharm.Engine(0, "mixed")
    w, mn, mx = e64.wnd_fit(xtr, ytr, 10, 0.15)
    p64, pr64 = e64.wnd_classify(xtr, ytr, 10, w, mn, mx, xte)
    t0 = time.perf_counter()
    pmx, prmx = emx.wnd_classify(xtr, ytr, 10, w, mn, mx, xte)
    st = emx.wnd_last_stats()
    print("mixed classify %.2f s (tensor cores: %d, rows re-checked in FP64: %d, K = %d)"
          % (time.perf_counter() - t0, st[0], st[1], st[2]))
    assert st[0] == 1
    np.testing.assert_array_equal(prmx, pr64)
    np.testing.assert_allclose(pmx, p64, rtol=0, atol=1e-6)
    print("max |p_mixed - p_fp64| = %.3g" % np.abs(pmx - p64).max())
