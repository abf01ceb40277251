"""Failure detection without a GPU fault: every failure is made on the host
(bad sizes, NaN / infinite pixels) or by lowering a
bounded wait's limit through an engine option, and each must come back as a
status (or the reference's defined result), never a fault, with the engine
still usable for the next call."""
import numpy as np
import pytest

from conftest import golden_names, oracle_features, oracle_lib
from gpu_helpers import images
from parity import compare, f14_columns
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu

WC_ERR_ARG, WC_ERR_DEVICE = -1, -5


def _rc_of(fn):
    import wndcharm
    try:
        fn()
    except wndcharm.WndcharmError as e:
        return str(e)
    return None


@pytest.fixture(scope="module")
def long_plan():
    import wndcharm
    return wndcharm.StdFeatureComputationPlans.getFeatureSetLong()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_union_find_cap_reports_device_error_then_recovers(prec, long_plan):
    """The object labelling's union-find links are bounded loops; a cap of one
    iteration makes every multi-pixel object run out.  The batch must report
    WC_ERR_DEVICE (the kernels' error word), and the next batch on the same
    engine, with the cap restored, must be correct."""
    import wndcharm
    eng = wndcharm.Engine(0, prec)
    imgs = images(seed=3, sizes=[(64, 64), (40, 33)])
    good = eng.extract(long_plan, imgs)
    eng.set_option("union_find_cap", 1)
    L = wndcharm.lib()
    out = np.zeros((2, long_plan.n_features))
    descs = (wndcharm._lib.wc_image_desc * 2)()
    keep = [np.ascontiguousarray(a) for a in imgs]
    for i, a in enumerate(keep):
        descs[i] = wndcharm._lib.wc_image_desc(a.ctypes.data, wndcharm._lib.WC_U16, a.shape[1], a.shape[0], 16, 0)
    rc = L.wc_extract_batch(eng._h, long_plan.handle, descs, 2, out.ctypes.data, 0)
    assert rc == WC_ERR_DEVICE, (rc, L.wc_last_error())
    assert b"error code 2" in L.wc_last_error()
    eng.set_option("union_find_cap", 0)
    again = eng.extract(long_plan, imgs)
    np.testing.assert_array_equal(again, good)


def test_qr_iteration_limit_gives_reference_result(long_plan):
    """The real-Schur QR has the reference's iteration limit (40 per tone, as
    Eigen's solver); a matrix that runs out gives that angle's f14 = 0, as the
    oracle does for the reference's unconverged solver.  With one iteration
    per tone most matrices run out: f14 (mean and range over the 4 angles)
    changes, stays finite and in range, nothing else changes, and the default
    limit restores the default result."""
    import wndcharm
    eng = wndcharm.Engine(0, "fp64")
    imgs = images(seed=9, sizes=[(64, 64), (80, 48)])
    good = eng.extract(long_plan, imgs)
    eng.set_option("qr_iter_per_tone", 1)
    capped = eng.extract(long_plan, imgs)
    eng.set_option("qr_iter_per_tone", 40)
    cols = f14_columns(golden_names(1))
    a, b = capped[:, cols], good[:, cols]
    assert np.mean(a != b) > 0.5, np.mean(a != b)
    assert np.all(np.isfinite(a)) and np.all((a >= 0) & (a <= 1.5))
    others = np.setdiff1d(np.arange(long_plan.n_features), cols)
    np.testing.assert_array_equal(capped[:, others], good[:, others])
    np.testing.assert_array_equal(eng.extract(long_plan, imgs), good)


def test_bad_sizes_and_options_are_arguments_errors(long_plan):
    import wndcharm
    eng = wndcharm.Engine(0, "fp64")
    L = wndcharm.lib()
    buf = np.zeros(16, dtype=np.uint16)
    out = np.zeros(long_plan.n_features)
    for (w, h) in [(0, 4), (4, 0), (-3, 5), (40000, 2), (20000, 20000)]:
        d = (wndcharm._lib.wc_image_desc * 1)()
        d[0] = wndcharm._lib.wc_image_desc(buf.ctypes.data, wndcharm._lib.WC_U16, w, h, 16, 0)
        assert L.wc_extract_batch(eng._h, long_plan.handle, d, 1, out.ctypes.data, 0) == WC_ERR_ARG, (w, h)
    assert L.wc_engine_set_option(eng._h, b"no such option", 1) == WC_ERR_ARG
    assert L.wc_engine_set_option(eng._h, b"qr_iter_per_tone", 0) == WC_ERR_ARG
    # and the engine still works
    img = images(seed=1, sizes=[(32, 32)])
    exp = oracle_features(oracle_lib(), img[0])
    assert not compare(eng.extract(long_plan, img)[0], exp, golden_names(1), rtol=1e-7, f14="exact")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_nan_and_inf_pixels_give_a_status_not_a_fault(prec, long_plan):
    """Floating-point images with NaN and infinite pixels (the reference has no
    defined result for them): the call returns a status, and the engine's next
    batch is still bit-identical to a fresh engine's."""
    import wndcharm
    eng = wndcharm.Engine(0, prec)
    rng = np.random.default_rng(5)
    bad = rng.uniform(0, 4095, size=(48, 40))
    bad[3, 4] = np.nan
    bad[10, 11] = np.inf
    bad[20, 2] = -np.inf
    allnan = np.full((24, 24), np.nan)
    for img in (bad, allnan):
        msg = _rc_of(lambda: eng.extract(long_plan, [img]))
        assert msg is None or isinstance(msg, str)
    imgs = images(seed=12, sizes=[(48, 40)])
    fresh = wndcharm.Engine(0, prec).extract(long_plan, imgs)
    np.testing.assert_array_equal(eng.extract(long_plan, imgs), fresh)
