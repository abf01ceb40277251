"""Mixed-precision form against the oracle: every family within its stated
tolerance (FP64 rules for the families that stay FP64, MIXED_RULES for the
FP32 ones), plus per-family error report."""
import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_lib
from gpu_helpers import images
from parity import compare_mixed, family_errors
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import wndcharm
    return wndcharm.Engine(0, "mixed")


@pytest.fixture(scope="module")
def long_plan():
    import wndcharm
    return wndcharm.StdFeatureComputationPlans.getFeatureSetLong()


def test_mixed_synthetic_vs_oracle(eng, long_plan):
    imgs = images(seed=41, sizes=[(128, 128), (96, 80), (200, 150), (33, 47)])
    got = eng.extract(long_plan, imgs)
    names = golden_names(1)
    lib = oracle_lib()
    worst = {}
    for i, img in enumerate(imgs):
        exp = oracle_features(lib, img)
        fails = compare_mixed(got[i], exp, names, f14="exact")
        assert not fails, (img.shape, list(fails.items())[:3])
        for k, v in family_errors(got[i], exp, names).items():
            w = worst.get(k, (0.0, 0.0, ""))
            worst[k] = (max(w[0], v[0]), max(w[1], v[1]), v[2] if v[1] >= w[1] else w[2])
    for k in sorted(worst):
        print("%-40s max rel %.3g  max rel-to-group %.3g  %s" % (k, worst[k][0], worst[k][1], worst[k][2]))


def test_mixed_reference_fixtures(eng, long_plan):
    g = golden("reference_synthetic.npz")
    names = golden_names(1)
    for i in range(6):
        got = eng.extract(long_plan, [g["img_%d" % i]])[0]
        fails = compare_mixed(got, g["long_%d" % i], names)
        assert not fails, (i, list(fails.items())[:3])


def test_mixed_deterministic(eng, long_plan):
    imgs = images(seed=43, sizes=[(64, 64), (40, 52)])
    a = eng.extract(long_plan, imgs)
    b = eng.extract(long_plan, imgs)
    np.testing.assert_array_equal(a, b)


def test_serialised_profile_same_features(eng, long_plan):
    """Engine.profile(serial=True) runs every lane on the engine's stream:
    the same features, and a time for every stage."""
    imgs = images(seed=47, sizes=[(96, 96), (64, 80)])
    a = eng.extract(long_plan, imgs)
    eng.profile(True, serial=True)
    try:
        b = eng.extract(long_plan, imgs)
        rep = {name: ms for name, ms, _ in eng.profile_report()}
    finally:
        eng.profile(False)
    np.testing.assert_array_equal(a, b)
    for stage in ("Chebyshev", "Fourier", "Haralick Textures", "Haralick: real Schur (f14)", "Tamura Textures",
                  "Zernike Coefficients", "PixStats+Gini (sort)"):
        assert rep.get(stage, 0.0) > 0.0, stage
    c = eng.extract(long_plan, imgs)  # and back to the lanes
    np.testing.assert_array_equal(a, c)


def test_512_workload_both_forms(long_plan):
    """Two 512 x 512 images of the benchmark workload through both forms, against
    the oracle (run on two host threads)."""
    import ctypes
    import wndcharm
    from wndcharm import synth
    from conftest import D
    from parity import compare
    imgs, _ = synth.config2(n_per_class=1, size=512, seed=1)
    imgs = imgs[:2]
    lib = oracle_lib()
    pix = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel() for a in imgs])
    offs = np.array([0, imgs[0].size], dtype=np.int64)
    ws = np.array([512, 512], dtype=np.int32)
    exp = np.zeros((2, 2919))
    lib.wco_extract_std_batch(1, pix.ctypes.data_as(D), offs.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                              ws.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                              ws.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 2, 16, exp.ctypes.data_as(D), 2)
    names = golden_names(1)
    for prec, cmp in (("fp64", compare), ("mixed", compare_mixed)):
        got = wndcharm.Engine(0, prec).extract(long_plan, imgs)
        for i in range(2):
            for k, v in sorted(family_errors(got[i], exp[i], names).items()):
                if v[1] > 0:
                    print(prec, i, "%-32s rel %.3g group %.3g %s" % (k, v[0], v[1], v[2]))
        for i in range(2):
            fails = cmp(got[i], exp[i], names, f14="exact")
            assert not fails, (prec, i, list(fails.items())[:4])
