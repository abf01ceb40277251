"""The engine's launch-shape tuner: while it tries its candidates (the
real-Schur work queue with and without 4-warp groups and at two grid sizes,
the Wavelet and Edge block shapes), every batch's features must be the same
bit for bit (a launch shape changes the schedule, never the arithmetic),
and after one batch per candidate every key has chosen one."""
import numpy as np
import pytest

from gpu_helpers import images
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_tuned_shapes_give_identical_features(prec):
    import wndcharm
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    imgs = images(seed=31, sizes=[(96, 80), (64, 64), (130, 70), (48, 99)])
    eng = wndcharm.Engine(0, prec)
    first = eng.extract(plan, imgs)
    for _ in range(4):
        np.testing.assert_array_equal(eng.extract(plan, imgs), first)
    tune = eng.tuning()
    assert any(k.startswith("har_qr/") for k in tune), tune
    assert any(k.startswith("wavelet/") for k in tune) and any(k.startswith("edge/") for k in tune), tune
    for k, (chosen, ms) in tune.items():
        assert chosen >= 0 and min(ms) >= 0, (k, chosen, ms)
    # and with the tuner off: the first candidates, the same features
    off = wndcharm.Engine(0, prec)
    off.set_option("autotune", 0)
    np.testing.assert_array_equal(off.extract(plan, imgs), first)
    assert off.tuning() == {}
