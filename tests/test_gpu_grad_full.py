"""The backward pass of WND-5 marginal probabilities at the full
differentiation workload: 256 images of 256 x 256 in [0, 1] (blob + grating,
4 classes, seed 3, float64 so that no two pixels tie by rounding), WND-5
trained on 192 of them over the 400 features of the continuous families
with the top Fisher scores; the 64 others are the test images.

Checked (1) against a float64 torch autograd restatement of the same
functions on 4 test images (every pixel's gradient and the weights'), and
(2) against central differences (h = 1e-3) of the GPU's own forward pass on
64 random pixels of each of 8 test images, with the kink criterion of the
scaled-down test: where the step [x - h, x + h] holds no kink they agree."""
import numpy as np
import pytest

import grad_reference as gref
import synth_loader  # noqa: F401
from test_gpu_grad import _fd_check, _smooth_and_ok

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full():
    import wndcharm
    from wndcharm import synth
    from wndcharm.grad import WNDModel, continuous_groups
    imgs, labels = synth.config4(n=256, size=256, seed=3, dtype=np.float64)
    tr, te = list(range(192)), list(range(192, 256))
    groups = continuous_groups()
    plan = wndcharm.FeatureComputationPlan("continuous")
    for g in groups:
        plan.add(g)
    eng = wndcharm.Engine(0, "fp64")
    rows = eng.extract(plan, [imgs[i] for i in tr])
    ytr = labels[tr]
    w, mn, mx = eng.wnd_fit(rows, ytr, 4, 1.0)
    thr = np.sort(w)[::-1][399]
    w = np.where(w >= thr, w, 0.0)
    assert (w > 0).sum() == 400
    model = WNDModel(eng, plan, rows, ytr, 4, mn, mx)
    return dict(model=model, groups=groups, rows=rows, ytr=ytr, w=w, mn=mn, mx=mx,
                test=[imgs[i] for i in te], labels=labels[te])


def test_full_backward_matches_torch_autograd(full):
    import torch
    from wndcharm.grad import class_evidence_maps
    s = full
    # an image classified with a probability within ~1e-15 of 1 has
    # gradients below the forward pass's own rounding (every class's map is
    # then a difference of nearly equal terms): the check takes the 4 test
    # images the classifier is least sure of
    probs, _, _ = s["model"].run(s["test"], s["w"])
    pick = np.argsort(probs.max(1))[:4]
    print("checked images' largest probabilities:", probs.max(1)[pick])
    test = [s["test"][i] for i in pick]
    seed = np.random.default_rng(4).normal(size=(4, 4))
    _, gp, gw = s["model"].run(test, s["w"], seed=seed)
    Xn = torch.from_numpy(gref.normalize_train(s["rows"], s["mn"], s["mx"]))
    y = torch.from_numpy(s["ytr"])
    wt = torch.from_numpy(s["w"]).requires_grad_(True)
    # the seeded sum mixes the classes' maps, which cancel where one class's
    # probability is near 1 (the maps sum to zero): errors are measured
    # against the largest contributing class map
    maps = class_evidence_maps(s["model"], test, s["w"])
    worst = 0.0
    for i, img in enumerate(test):
        x = torch.from_numpy(img.copy()).requires_grad_(True)
        p = gref.wnd(gref.features(x, s["groups"]), Xn, y, 4, wt, torch.from_numpy(s["mn"]),
                     torch.from_numpy(s["mx"]))
        (torch.from_numpy(seed[i]) * p).sum().backward()
        g = x.grad.numpy()
        scale = max((np.abs(seed[i, c]) * np.abs(maps[i, c]).max() for c in range(4)))
        err = np.abs(gp[i] - g).max() / max(scale, 1e-300)
        worst = max(worst, err)
        assert err < 1e-7, (i, err, np.abs(g).max() / scale)
    gwt = wt.grad.numpy()
    np.testing.assert_allclose(gw, gwt, rtol=1e-7, atol=1e-9 * np.abs(gwt).max())
    print("256 x 256: pixel gradients within %.3g of torch autograd (relative to the largest class map)" % worst)


def test_full_backward_matches_central_differences(full):
    """Central differences of the GPU's forward pass on 64 random pixels of
    each of 8 test images, all 400 features.  At this size the pixels' values
    lie ~1e-5 apart, so a step of h = 1e-3 crosses kinks (order statistics
    change rank, fractal |I(p) - I(q)| change sign) on most pixels; those
    statistics are reported.  With h = 1e-6 few steps cross one, and the
    quotients agree with the derivative up to the forward pass's rounding.  The Zernike magnitudes off the
    Edge planes are smooth at any h: every sampled pixel agrees at h = 1e-3."""
    s = full
    rng_pix = np.random.default_rng(6)
    fd, an, gp, gm = _fd_check(s["model"], s["test"][:8], s["w"], 64, rng_pix)
    smooth, ok = _smooth_and_ok(fd, an, gp, gm)
    scale = np.abs(an).max()
    rel = np.abs(fd - an) / (np.abs(an) + 1e-6 * scale)
    print("256 x 256, h = 1e-3: %d of %d steps hold no kink, %d of them agree; relative error quantiles "
          "50/75/90/95/99%%: %s" % (smooth.sum(), smooth.size, (ok & smooth).sum(),
                                    np.array2string(np.quantile(rel, [0.5, 0.75, 0.9, 0.95, 0.99]), precision=3)))
    fd, an, gp, gm = _fd_check(s["model"], s["test"][:8], s["w"], 64, np.random.default_rng(6), h=1e-6)
    rel = np.abs(fd - an) / (np.abs(an) + 1e-6 * np.abs(an).max())
    q = np.quantile(rel, [0.5, 0.75, 0.9, 0.95, 0.99])
    print("256 x 256, h = 1e-6: relative error quantiles 50/75/90/95/99%%: %s; within 1e-3: %d of %d"
          % (np.array2string(q, precision=3), (rel < 1e-3).sum(), rel.size))
    # measured: the quotient's error grows with h on both sides of 1e-6 (rank
    # crossings of the Gini and order statistics over 65,536 pixels above it,
    # the forward pass's rounding over 2h below it); half the pixels agree to
    # ~1e-5, three quarters to ~1e-4
    assert q[0] < 1e-4 and q[1] < 1e-3, q
    names = s["model"].plan.feature_names()
    zern = np.array([nm.startswith("Zernike") and "Edge" not in nm for nm in names])
    wz = np.where(zern, s["w"], 0.0)
    assert (wz > 0).sum() >= 10
    fd, an, gp, gm = _fd_check(s["model"], s["test"][:8], wz, 16, np.random.default_rng(8))
    smooth, ok = _smooth_and_ok(fd, an, gp, gm)
    print("256 x 256, Zernike only, h = 1e-3: %d of %d steps hold no kink; %d of %d pixels agree"
          % (smooth.sum(), smooth.size, ok.sum(), ok.size))
    assert ok.mean() >= 0.98
