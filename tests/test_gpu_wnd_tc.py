"""WND-5 distances on the tensor cores (the mixed form's wc_wnd_classify*):
against the FP64 form (the reference's order, itself pinned to the oracle
and the reference's fixtures), predicted classes identical and marginal
probabilities within 1e-6, on the synthetic feature vectors of the WND
workload (per-feature N(mu_cf, 1), class means N(0, 0.5)), with duplicated
rows (distance 0: the reference skips them; the tensor-core pass must hand
them to the FP64 re-check), with more weighted features than the digit
sums allow (the pairs-of-floats path), and through the device-pointer entry
point."""
import numpy as np
import pytest

import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


def _fit(e64, xtr, ytr, C, frac):
    return e64.wnd_fit(xtr, ytr, C, frac)


@pytest.mark.parametrize("n_train,n_test,F,C,seed", [(3000, 700, 2919, 10, 4), (1500, 300, 1059, 4, 7),
                                                       (200, 129, 300, 3, 1)])
def test_tensor_core_matches_fp64(n_train, n_test, F, C, seed):
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(n_train, n_test, F, C, seed)
    e64, emx = wndcharm.Engine(0, "fp64"), wndcharm.Engine(0, "mixed")
    w, mn, mx = e64.wnd_fit(xtr, ytr, C, 0.15)
    p64, pr64 = e64.wnd_classify(xtr, ytr, C, w, mn, mx, xte)
    pmx, prmx = emx.wnd_classify(xtr, ytr, C, w, mn, mx, xte)
    stats = emx.wnd_last_stats()
    assert stats[0] == 1, stats  # the tensor-core path ran
    np.testing.assert_array_equal(prmx, pr64)
    np.testing.assert_allclose(pmx, p64, rtol=0, atol=1e-6)
    print("K=%d: max |p_tc - p_fp64| = %.3g, %d of %d rows re-checked in FP64"
          % (stats[2], np.abs(pmx - p64).max(), stats[1], n_test))
    assert stats[1] <= n_test // 20  # the re-check is the exception


def test_duplicates_and_near_duplicates_go_to_the_fp64_recheck():
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(1000, 200, 500, 5, 11)
    xte[:10] = xtr[:10]              # exact duplicates: distance 0 (skipped by the reference)
    xte[10:20] = xtr[20:30] + 1e-9   # near-duplicates
    e64, emx = wndcharm.Engine(0, "fp64"), wndcharm.Engine(0, "mixed")
    w, mn, mx = e64.wnd_fit(xtr, ytr, 5, 0.15)
    p64, pr64 = e64.wnd_classify(xtr, ytr, 5, w, mn, mx, xte)
    pmx, prmx = emx.wnd_classify(xtr, ytr, 5, w, mn, mx, xte)
    stats = emx.wnd_last_stats()
    assert stats[0] == 1 and stats[1] >= 20, stats
    np.testing.assert_array_equal(prmx, pr64)
    np.testing.assert_allclose(pmx, p64, rtol=0, atol=1e-6)
    # recomputed by the FP64 kernel itself (its chunks of training rows are
    # split finer for a few rows: the sums differ from the full pass in the last bits)
    np.testing.assert_allclose(pmx[:20], p64[:20], rtol=0, atol=1e-14)


def test_many_weighted_features_use_pairs_of_floats():
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(800, 100, 1200, 4, 3)
    e64, emx = wndcharm.Engine(0, "fp64"), wndcharm.Engine(0, "mixed")
    w, mn, mx = e64.wnd_fit(xtr, ytr, 4, 1.0)  # every feature weighted
    p64, pr64 = e64.wnd_classify(xtr, ytr, 4, w, mn, mx, xte)
    pmx, prmx = emx.wnd_classify(xtr, ytr, 4, w, mn, mx, xte)
    assert emx.wnd_last_stats()[0] == 0
    np.testing.assert_array_equal(prmx, pr64)
    np.testing.assert_allclose(pmx, p64, rtol=0, atol=1e-6)


def test_device_entry_points_match_host_ones():
    import torch
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(2000, 256, 700, 6, 5)
    emx = wndcharm.Engine(0, "mixed")
    w, mn, mx = emx.wnd_fit(xtr, ytr, 6, 0.15)
    p, pr = emx.wnd_classify(xtr, ytr, 6, w, mn, mx, xte)
    d = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dt, device="cuda")  # noqa
    X, y, T = d(xtr), d(ytr, torch.int32), d(xte)
    dw, dmn, dmx = (torch.empty(700, dtype=torch.float64, device="cuda") for _ in range(3))
    emx.wnd_fit_device(X, y, 6, 0.15, dw, dmn, dmx)
    np.testing.assert_array_equal(dw.cpu().numpy(), w)
    np.testing.assert_array_equal(dmn.cpu().numpy(), mn)
    np.testing.assert_array_equal(dmx.cpu().numpy(), mx)
    dp = torch.empty((256, 6), dtype=torch.float64, device="cuda")
    dpr = torch.empty(256, dtype=torch.int32, device="cuda")
    emx.wnd_classify_device(X, y, 6, dw, dmn, dmx, T, dp, dpr)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dpr.cpu().numpy(), pr)
    np.testing.assert_array_equal(dp.cpu().numpy(), p)


def test_normalisation_matches_the_division():
    """signatures::normalize on the GPU (the values every WND-5 kernel
    compares) takes the quotient by Markstein's method: equal bit for bit to
    numpy's IEEE division on random rows and on the edges (the range's ends,
    NaN, values outside it, a range below DBL_EPSILON, subnormal and huge
    offsets, ranges near 2^900 and 2^-900)."""
    import wndcharm
    rng = np.random.default_rng(11)
    F = 64
    mn = rng.normal(size=F) * 10.0 ** rng.integers(-8, 9, size=F)
    mx = mn + np.abs(rng.normal(size=F)) * 10.0 ** rng.integers(-12, 12, size=F)
    mn[0], mx[0] = 0.0, 2.0 ** 950
    mn[1], mx[1] = 1.0, 1.0 + 2.0 ** -40
    mn[2], mx[2] = 5.0, 5.0 + 1e-17  # range below DBL_EPSILON
    mn[3], mx[3] = -2.0 ** 901, 2.0 ** 901
    mn[4], mx[4] = 0.0, 1e-300
    X = mn + (mx - mn) * rng.uniform(-0.1, 1.1, size=(20000, F))
    X[0] = mn
    X[1] = mx
    X[2] = np.nan
    X[3] = np.nextafter(mn, np.inf)
    X[4, 4] = 5e-324
    X[5, 4] = 2.0 ** -1000
    X[6, 0] = 2.0 ** -901
    out = wndcharm.Engine(0, "fp64").wnd_normalize(X, mn, mx)
    with np.errstate(all="ignore"):
        ref = 100 * ((X - mn) / (mx - mn))
    ref = np.where(X > mx, 100.0, ref)
    ref = np.where(np.isnan(X) | (X < mn) | ((mx - mn) < np.finfo(np.float64).eps), 0.0, ref)
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fit_classify_matches_separate_calls(prec):
    import wndcharm
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(2500, 300, 1059, 5, 9)
    e = wndcharm.Engine(0, prec)
    w, mn, mx = e.wnd_fit(xtr, ytr, 5, 0.15)
    p, pr = e.wnd_classify(xtr, ytr, 5, w, mn, mx, xte)
    p2, pr2, w2, mn2, mx2 = e.wnd_fit_classify(xtr, ytr, 5, xte, 0.15)
    for a, b in ((w2, w), (mn2, mn), (mx2, mx), (pr2, pr), (p2, p)):
        np.testing.assert_array_equal(a, b)


def test_class_sums_over_shards_give_classify2():
    """wc_wnd_class_sums on two halves of the training rows, added (what the
    all-reduce of the sharded path does) and finished: the FP64 form's
    classify2 on the whole set."""
    import wndcharm
    from wndcharm import synth
    from wndcharm.dist import wnd_finish
    xtr, ytr, xte, _ = synth.feature_vectors(3001, 200, 1059, 6, 12)
    e = wndcharm.Engine(0, "fp64")
    w, mn, mx = e.wnd_fit(xtr, ytr, 6, 0.15)
    p, pr = e.wnd_classify(xtr, ytr, 6, w, mn, mx, xte)
    s1, c1 = e.wnd_class_sums(xtr[:1400], ytr[:1400], 6, w, mn, mx, xte)
    s2, c2 = e.wnd_class_sums(xtr[1400:], ytr[1400:], 6, w, mn, mx, xte)
    probs, pred, _ = wnd_finish(s1 + s2, c1 + c2)
    np.testing.assert_array_equal(pred, pr)
    np.testing.assert_allclose(probs, p, rtol=1e-12, atol=1e-15)


def test_fit_stats_over_shards_give_wnd_fit():
    """wc_wnd_fit_stats on three shards of the training rows, combined as the
    sharded fit's all-reduces combine them (min, max, sums), and
    wc_wnd_fisher: wc_wnd_fit's ranges exactly, its weights and selection."""
    import wndcharm
    from wndcharm import synth
    from wndcharm.dist import class_means
    xtr, ytr, _, _ = synth.feature_vectors(5000, 10, 2919, 10, 13)
    xtr[17, 5] = np.nan
    e = wndcharm.Engine(0, "fp64")
    w, mn, mx = e.wnd_fit(xtr, ytr, 10, 0.15)
    parts = [(xtr[a:b], ytr[a:b]) for a, b in ((0, 1700), (1700, 3300), (3300, 5000))]
    st0 = [e.wnd_fit_stats(0, X, y, 10) for X, y in parts]
    gmn = np.min([s[0] for s in st0], axis=0)
    gmx = np.max([s[1] for s in st0], axis=0)
    cnt = np.sum([s[2] for s in st0], axis=0)
    np.testing.assert_array_equal(gmn, mn)
    np.testing.assert_array_equal(gmx, mx)
    sums = np.sum([e.wnd_fit_stats(1, X, y, 10, gmn, gmx) for X, y in parts], axis=0)
    means = class_means(sums, cnt)
    sq = np.sum([e.wnd_fit_stats(2, X, y, 10, gmn, gmx, means) for X, y in parts], axis=0)
    w2 = e.wnd_fisher(10, 0.15, sums, cnt, sq)
    np.testing.assert_array_equal(w2 == 0, w == 0)
    np.testing.assert_allclose(w2, w, rtol=1e-12, atol=0)
