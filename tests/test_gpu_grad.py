"""The backward pass of WND-5 marginal probabilities (wc_wnd_grad) on a
scaled-down differentiation workload: float64 images in [0, 1] from the
blob + grating generator (4 classes, seed 3; 40 images of 64 x 64, 30 to
train, 10 to test; float64 so that no two pixels tie by rounding, which would
put the comparison on a kink), features from the smooth families of the long plan
(Zernike on its 8 nodes, pixel statistics and fractal on its 12, Gini on
the nonnegative planes),
WND-5 weighted by the top Fisher scores.

Checked against (1) a float64 torch autograd restatement of the same
functions (tests/grad_reference.py): the forward features and probabilities,
then the gradients to every pixel and to the weights; (2) central finite
differences (h = 1e-3, float64) of the GPU's own forward pass on random
pixels: wherever the step [x - h, x + h] holds no kink (the backward pass's
second difference there is of curvature size) they must agree; (3) the class-evidence maps, whose sum over the classes is zero
(the probabilities sum to 1)."""
import numpy as np
import pytest

import grad_reference as gref
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu

def smooth_groups():
    from wndcharm.grad import continuous_groups
    return continuous_groups()


@pytest.fixture(scope="module")
def setup():
    import wndcharm
    from wndcharm import synth
    from wndcharm.grad import WNDModel
    imgs, labels = synth.config4(n=40, size=64, seed=3, dtype=np.float64)
    tr, te = list(range(30)), list(range(30, 40))
    groups = smooth_groups()
    plan = wndcharm.FeatureComputationPlan("smooth")
    for g in groups:
        plan.add(g)
    eng = wndcharm.Engine(0, "fp64")
    rows = eng.extract(plan, [imgs[i] for i in tr])
    ytr = labels[tr]
    w, mn, mx = eng.wnd_fit(rows, ytr, 4, 1.0)
    K = 120
    thr = np.sort(w)[::-1][K - 1]
    w = np.where(w >= thr, w, 0.0)
    model = WNDModel(eng, plan, rows, ytr, 4, mn, mx)
    test = [imgs[i].astype(np.float64) for i in te]
    return dict(model=model, plan=plan, groups=groups, rows=rows, ytr=ytr, w=w, mn=mn, mx=mx, test=test, eng=eng)


def test_forward_matches_classify_and_torch(setup):
    import torch
    s = setup
    probs, _, _ = s["model"].run(s["test"], s["w"])
    feats = s["eng"].extract(s["plan"], s["test"])
    p2, _ = s["eng"].wnd_classify(s["rows"], s["ytr"], 4, s["w"], s["mn"], s["mx"], feats)
    np.testing.assert_allclose(probs, p2, rtol=0, atol=1e-12)
    Xn = torch.from_numpy(gref.normalize_train(s["rows"], s["mn"], s["mx"]))
    y = torch.from_numpy(s["ytr"])
    for i, img in enumerate(s["test"][:4]):
        f = gref.features(torch.from_numpy(img), s["groups"]).numpy()
        np.testing.assert_allclose(f, feats[i], rtol=1e-9, atol=1e-12)
        p = gref.wnd(torch.from_numpy(feats[i]), Xn, y, 4, torch.from_numpy(s["w"]), torch.from_numpy(s["mn"]),
                     torch.from_numpy(s["mx"])).numpy()
        np.testing.assert_allclose(p, probs[i], rtol=0, atol=1e-12)


def test_backward_matches_torch_autograd(setup):
    import torch
    s = setup
    rng = np.random.default_rng(1)
    seed = rng.normal(size=(len(s["test"]), 4))
    _, gp, gw = s["model"].run(s["test"], s["w"], seed=seed)
    Xn = torch.from_numpy(gref.normalize_train(s["rows"], s["mn"], s["mx"]))
    y = torch.from_numpy(s["ytr"])
    wt = torch.from_numpy(s["w"]).requires_grad_(True)
    worst = 0.0
    for i, img in enumerate(s["test"]):
        x = torch.from_numpy(img.copy()).requires_grad_(True)
        p = gref.wnd(gref.features(x, s["groups"]), Xn, y, 4, wt, torch.from_numpy(s["mn"]), torch.from_numpy(s["mx"]))
        (torch.from_numpy(seed[i]) * p).sum().backward()
        g = x.grad.numpy()
        err = np.abs(gp[i] - g).max() / max(np.abs(g).max(), 1e-300)
        worst = max(worst, err)
        assert err < 1e-7, (i, err)
    gwt = wt.grad.numpy()
    np.testing.assert_allclose(gw, gwt, rtol=1e-8, atol=1e-9 * np.abs(gwt).max())
    print("pixel gradients: max relative difference from torch autograd %.3g" % worst)


def _fd_check(model, test, w, npix, rng, h=1e-3):
    """Central differences of the predicted class's probability on npix random
    pixels per image, with the analytic derivative at x and at x +- h."""
    n = len(test)
    probs, _, _ = model.run(test, w)
    pred = probs.argmax(1)
    seed = np.zeros((n, 4))
    seed[np.arange(n), pred] = 1.0
    _, gp, _ = model.run(test, w, seed=seed)
    pix, batch, bseed = [], [], []
    for i, img in enumerate(test):
        for _ in range(npix):
            yy, xx = int(rng.integers(img.shape[0])), int(rng.integers(img.shape[1]))
            pix.append((i, yy, xx))
            for sgn in (1, -1):
                a = img.copy()
                a[yy, xx] += sgn * h
                batch.append(a)
                bseed.append(seed[i])
    pb, gb, _ = model.run(batch, w, seed=np.array(bseed))
    fd = np.array([(pb[2 * k, pred[i]] - pb[2 * k + 1, pred[i]]) / (2 * h) for k, (i, _, _) in enumerate(pix)])
    an = np.array([gp[i][yy, xx] for (i, yy, xx) in pix])
    gplus = np.array([gb[2 * k][yy, xx] for k, (_, yy, xx) in enumerate(pix)])
    gminus = np.array([gb[2 * k + 1][yy, xx] for k, (_, yy, xx) in enumerate(pix)])
    return fd, an, gplus, gminus


def _smooth_and_ok(fd, an, gp, gm):
    """A step [x - h, x + h] holds no kink when the backward pass's second
    difference g(x+h) - 2 g(x) + g(x-h) is of curvature size (O(h^2)), not
    of the size of the slopes' change across a kink; there the central
    difference equals g(x) up to that second difference / 6 (Taylor)."""
    scale = np.abs(an).max()
    d2 = np.abs(gp - 2 * an + gm)
    smooth = d2 <= 0.05 * np.abs(gp - gm) + 1e-6 * np.abs(an) + 1e-10 * scale
    ok = np.abs(fd - an) <= d2 / 3 + 1e-5 * np.abs(an) + 1e-9 * scale
    return smooth, ok


def test_backward_matches_central_differences(setup):
    """h = 1e-3 on 64 random pixels per test image, all the selected
    features.  A step that holds no kink of a piecewise-smooth feature (an
    |I(p) - I(q)| tie of the fractal sums, a rank swap of an order statistic
    or of a Gini rank, a tie of the Edge transform's maximum) must agree with
    the derivative; across a kink the central difference is the mean of the
    one-sided slopes, so those pixels are reported, not gated."""
    s = setup
    fd, an, gp, gm = _fd_check(s["model"], s["test"], s["w"], 64, np.random.default_rng(2))
    smooth, ok = _smooth_and_ok(fd, an, gp, gm)
    scale = np.abs(an).max()
    rel = np.abs(fd - an) / (np.abs(an) + 1e-6 * scale)
    q = np.quantile(rel, [0.5, 0.75, 0.9, 0.95, 0.99])
    print("finite differences, h = 1e-3: %d of %d steps hold no kink, %d of them agree; %d of all %d agree; "
          "relative error quantiles 50/75/90/95/99%%: %s" % (smooth.sum(), smooth.size, (ok & smooth).sum(), ok.sum(),
                                                           ok.size, np.array2string(q, precision=3)))
    # the step's mean slope equals the derivative up to the kinks it crosses:
    # most pixels agree to 1e-4, a tail (fractal ties, rank swaps) does not
    assert q[0] < 1e-3 and q[2] < 1e-2 and q[3] < 5e-2, q


def test_zernike_backward_matches_central_differences(setup):
    """Zernike magnitudes on the planes without the Edge transform (whose
    maximum has kinks) are smooth functions of the pixels here (the 64 x 64
    images lie inside the unit disc): the central differences agree with the
    derivative on every sampled pixel."""
    s = setup
    names = s["plan"].feature_names()
    zern = np.array([nm.startswith("Zernike") and "Edge" not in nm for nm in names])
    w = np.where(zern, s["w"], 0.0)
    assert (w > 0).sum() >= 10
    fd, an, gp, gm = _fd_check(s["model"], s["test"], w, 16, np.random.default_rng(5))
    smooth, ok = _smooth_and_ok(fd, an, gp, gm)
    print("Zernike only: %d of %d steps hold no kink; %d of %d pixels agree" % (smooth.sum(), smooth.size,
                                                                                ok.sum(), ok.size))
    assert ok.mean() >= 0.98


def test_autograd_function_and_evidence_maps(setup):
    import torch
    from wndcharm.grad import WNDProbability, class_evidence_maps
    s = setup
    x = torch.from_numpy(np.stack(s["test"][:3])).requires_grad_(True)
    wt = torch.from_numpy(s["w"]).requires_grad_(True)
    p = WNDProbability.apply(x, wt, s["model"])
    assert p.shape == (3, 4)
    p[:, 1].sum().backward()
    seed = np.zeros((3, 4))
    seed[:, 1] = 1.0
    _, gp, gw = s["model"].run(s["test"][:3], s["w"], seed=seed)
    np.testing.assert_array_equal(x.grad.numpy(), np.stack(gp))
    np.testing.assert_array_equal(wt.grad.numpy(), gw)
    maps = class_evidence_maps(s["model"], s["test"][:3], s["w"])
    assert maps.shape == (3, 4, 64, 64)
    # one forward, four backward passes: the same maps as one pass per class
    np.testing.assert_allclose(maps[:, 1], np.stack(gp), rtol=0, atol=1e-15 * np.abs(maps).max())
    np.testing.assert_allclose(maps.sum(1), 0.0, atol=1e-10 * np.abs(maps).max())
