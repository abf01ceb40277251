"""GPU parity on whole plans against the golden fixtures: the reference's own
test images (and their precalculated signatures), seeded synthetic images run
through the unmodified reference build, and the WND-5 fixtures; plus
determinism, batching and edge cases."""
import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_lib, oracle_wnd
from gpu_helpers import images, oracle_group
from parity import F14, compare, group_of, index_of
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import wndcharm
    return wndcharm.Engine(0, "fp64")


@pytest.fixture(scope="module")
def long_plan():
    import wndcharm
    return wndcharm.StdFeatureComputationPlans.getFeatureSetLong()


@pytest.fixture(scope="module")
def short_plan():
    import wndcharm
    return wndcharm.StdFeatureComputationPlans.getFeatureSet()


@pytest.mark.parametrize("key", ["t1_s01_c05_ij", "binuc1", "norm1", "010067_301x300"])
def test_reference_images(eng, long_plan, key):
    g = golden("reference_images.npz")
    names = golden_names(1)
    got = eng.extract(long_plan, [g["img_" + key]], bits=int(g["bits_" + key]))[0]
    fails = compare(got, g["ref_" + key], names, rtol=1e-7, atol=1e-9, count_moves=0)
    assert not fails, fails
    # the reference's precalculated signature (%.8g text, f14 from before its 2017 fix)
    f14 = np.array([group_of(n).startswith("Haralick") and index_of(n) in F14 for n in names])
    sig = g["sig_" + key]
    rel = np.abs(got - sig) / np.maximum(np.abs(sig), 1e-300)
    bad = (rel > 1e-6) & (np.abs(got - sig) > 1e-7) & ~f14
    hist_groups = ("Chebyshev-Fourier", "Chebyshev Coefficients", "Comb", "Radon")
    bad &= ~np.array([group_of(n).startswith(hist_groups) for n in names])
    assert not bad.any(), [(names[i], got[i], sig[i]) for i in np.nonzero(bad)[0][:10]]


@pytest.mark.parametrize("i", range(6))
def test_synthetic_fixtures_both_plans(eng, long_plan, short_plan, i):
    g = golden("reference_synthetic.npz")
    img = g["img_%d" % i]
    for plan, key, kind in ((long_plan, "long_%d" % i, 1), (short_plan, "short_%d" % i, 0)):
        got = eng.extract(plan, [img])[0]
        fails = compare(got, g[key], golden_names(kind), rtol=1e-7, atol=1e-9, count_moves=0)
        assert not fails, (kind, fails)


def test_uint8_fixture(eng, long_plan):
    g = golden("reference_synthetic.npz")
    got = eng.extract(long_plan, [g["img_u8"]], bits=8)[0]
    assert not compare(got, g["long_u8"], golden_names(1), rtol=1e-7, atol=1e-9, count_moves=0)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_f14_bit_exact(prec):
    """Haralick f14 (eigenvalue #2 of Q in real-Schur order) is the same
    algorithm and rounding as the oracle, in both forms (the mixed form's f14
    goes through the FP64 chain by default): every transform plane is
    bit-identical to the oracle's, so f14 must agree exactly on all 12."""
    import wndcharm
    from gpu_helpers import CHAINS as chains
    eng = wndcharm.Engine(0, prec)
    plan = wndcharm.FeatureComputationPlan("f14")
    for c in chains:
        plan.add("Haralick Textures %s" % c)
    imgs = images(seed=5)
    got = eng.extract(plan, imgs)
    for i, img in enumerate(imgs):
        exp = np.concatenate([oracle_group("Haralick Textures %s" % c, img) for c in chains])
        for g in range(len(chains)):
            np.testing.assert_array_equal(got[i][28 * g + 16: 28 * g + 18], exp[28 * g + 16: 28 * g + 18],
                                          err_msg="%s %s" % (chains[g], img.shape))


def test_deterministic_and_batch_invariant(eng, long_plan):
    imgs = images(seed=21, sizes=[(64, 64), (40, 52), (33, 33)])
    a = eng.extract(long_plan, imgs)
    b = eng.extract(long_plan, imgs)
    np.testing.assert_array_equal(a, b)
    for i, img in enumerate(imgs):
        np.testing.assert_array_equal(eng.extract(long_plan, [img])[0], a[i])


def test_edge_cases(eng, long_plan):
    """Small, odd-sized, constant and mostly-zero images: finite where the
    oracle is finite, and matching it."""
    rng = np.random.default_rng(3)
    cases = [rng.integers(0, 4096, size=(16, 16)).astype(np.uint16),
             rng.integers(0, 4096, size=(13, 11)).astype(np.uint16),
             np.zeros((20, 24), dtype=np.uint16) + 7]
    z = np.zeros((32, 32), dtype=np.uint16)
    z[10:14, 5:9] = 1000
    cases.append(z)
    names = golden_names(1)
    lib = oracle_lib()
    for k, img in enumerate(cases):
        got = eng.extract(long_plan, [img])[0]
        exp = oracle_features(lib, img)
        fin = np.isfinite(exp)
        diff = np.nonzero(np.isfinite(got) != fin)[0]
        assert not len(diff), (img.shape, [(names[i], got[i], exp[i]) for i in diff[:8]])
        # The DFT of the constant image is zero off DC and the block image has
        # exact sinc zeros: what an FFT returns there is rounding noise, which the
        # oracle's DFT reproduces bit for bit (same operations), so even the
        # features that test "> 0" (Gini) or bin that noise are compared.
        fails = compare(np.where(fin, got, 0), np.where(fin, exp, 0), names, rtol=1e-7, atol=1e-9, count_moves=0,
                        f14="exact")
        assert not fails, (img.shape, list(fails.items())[:3])


def test_wnd_fixtures(eng):
    g = golden("reference_wnd.npz")
    X, y = g["fit_X"], g["fit_y"]
    w, mn, mx = eng.wnd_fit(X, y, 2, 0.15)
    np.testing.assert_allclose(w, g["ref_w"], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(mn, g["ref_min"])
    np.testing.assert_array_equal(mx, g["ref_max"])
    p, pred = eng.wnd_classify(X, y, 2, w, mn, mx, X)
    np.testing.assert_array_equal(pred, g["classify_pred"])
    np.testing.assert_allclose(p, g["ref_p"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(p, g["classify_table"][:, 1:3], atol=5e-4 + 1e-12)
    w1, _, _ = eng.wnd_fit(X, y, 2, 1.0)
    np.testing.assert_allclose(w1, g["weights_f1"], atol=1e-5)


def test_wnd_synthetic_vs_oracle(eng):
    from wndcharm import synth
    g = golden("reference_wnd.npz")
    xtr, ytr, xte, _ = synth.feature_vectors(300, 40, 2919, 10, 4)
    w, mn, mx = eng.wnd_fit(xtr, ytr, 10, 0.15)
    np.testing.assert_allclose(w, g["syn_w"], rtol=1e-12, atol=0)
    p, pred = eng.wnd_classify(xtr, ytr, 10, w, mn, mx, xte)
    np.testing.assert_array_equal(pred, g["syn_pred"])
    np.testing.assert_allclose(p, g["syn_p"], rtol=0, atol=1e-6)
    lib = oracle_lib()
    ow, omn, omx, op, opred = oracle_wnd(lib, xtr, ytr, xte, 10, 0.15)
    np.testing.assert_array_equal(pred, opred)
