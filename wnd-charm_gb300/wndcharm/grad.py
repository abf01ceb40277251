"""Differentiable WND-5 marginal probabilities (wc_wnd_grad): the forward pass
is the engine's feature extraction of the test images followed by classify2
against fixed training rows; the backward pass is hand-written CUDA through
classify2, the smooth feature families (Zernike magnitudes, pixel statistics,
fractal, Gini) and the Fourier / Chebyshev / Wavelet / Edge transform chains
to the pixels, and to the Fisher weights.  Binned families are
piecewise-constant: their features contribute no gradient.

    model = WNDModel(engine, plan, train_rows, labels, n_classes, mins, maxs)
    probs = WNDProbability.apply(images, weights, model)   # images (n, H, W) float64
    probs[:, c].sum().backward()                            # images.grad, weights.grad
    maps = class_evidence_maps(model, images, weights)      # (n, C, H, W)
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib


# the transform chains of the long plan's groups (src/Tasks.cpp:354-400):
# group B (Zernike among them) on 8 of them, group C on all 12
LONG_CHAINS = ["()", "(Fourier ())", "(Wavelet ())", "(Chebyshev ())", "(Edge ())", "(Chebyshev (Fourier ()))",
               "(Wavelet (Fourier ()))", "(Fourier (Wavelet ()))", "(Fourier (Chebyshev ()))",
               "(Chebyshev (Wavelet ()))", "(Fourier (Edge ()))", "(Wavelet (Edge ()))"]
LONG_B_CHAINS = ["()", "(Fourier ())", "(Wavelet ())", "(Chebyshev ())", "(Fourier (Wavelet ()))", "(Edge ())",
                 "(Fourier (Edge ()))", "(Wavelet (Edge ()))"]


def continuous_groups():
    """The long plan's groups whose features are continuous functions of the
    pixels with a backward pass here: Zernike Coefficients on its 8 group-B
    chains, Fractal Features and Pixel Intensity Statistics on all 12, and
    the Gini Coefficient on the planes that take no negative values (the
    image, Fourier magnitudes, Edge maxima); on the others Gini jumps where a
    value crosses 0 (it counts the positive pixels).  882 features."""
    groups = ["Zernike Coefficients %s" % c for c in LONG_B_CHAINS]
    for c in LONG_CHAINS:
        groups += ["Fractal Features %s" % c, "Pixel Intensity Statistics %s" % c]
        if c == "()" or c.startswith("(Fourier") or c.startswith("(Edge"):
            groups.append("Gini Coefficient %s" % c)
    return groups


class WNDModel(object):
    """The fixed part of the classifier: engine, feature plan, training
    feature rows (N x plan features), their labels, the min / max the rows
    were normalised with."""

    def __init__(self, engine, plan, train, labels, n_classes, mins, maxs):
        self.engine = engine
        self.plan = plan
        self.train = np.ascontiguousarray(train, dtype=np.float64)
        self.labels = np.ascontiguousarray(labels, dtype=np.int32)
        self.C = int(n_classes)
        self.mins = np.ascontiguousarray(mins, dtype=np.float64)
        self.maxs = np.ascontiguousarray(maxs, dtype=np.float64)

    def run(self, images, weights, seed=None):
        """(probs (n, C), d loss / d pixels, d loss / d weights) for float images
        and weights.  seed: None (forward only: the gradients are None), (n, C)
        (one backward pass: a list of (H, W) maps and an (F,) vector), or
        (n, S, C) (S backward passes after one forward: a list of (S, H, W)
        maps and an (S, F) array)."""
        imgs = [np.ascontiguousarray(a, dtype=np.float64) for a in images]
        n = len(imgs)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        descs = (_lib.wc_image_desc * n)()
        for i, a in enumerate(imgs):
            descs[i] = _lib.wc_image_desc(a.ctypes.data, _lib.WC_F64, a.shape[1], a.shape[0], 16, 0)
        probs = np.zeros((n, self.C))
        D = _lib.D
        gp = gw = None
        sd = None
        S = 0
        if seed is not None:
            multi = np.ndim(seed) == 3
            sd = np.ascontiguousarray(seed, dtype=np.float64).reshape(n, -1, self.C)
            S = sd.shape[1]
            gp = np.zeros(sum(a.size for a in imgs) * S)
            gw = np.zeros(w.size * S)
        check(lib().wc_wnd_grad(self.engine._h, self.plan.handle, self.train.ctypes.data_as(D), self.train.shape[0],
                                self.labels.ctypes.data_as(_lib.I), self.C, w.ctypes.data_as(D),
                                self.mins.ctypes.data_as(D), self.maxs.ctypes.data_as(D), descs, n,
                                sd.ctypes.data_as(D) if sd is not None else None, S, probs.ctypes.data_as(D),
                                gp.ctypes.data_as(D) if gp is not None else None,
                                gw.ctypes.data_as(D) if gw is not None else None))
        grads = None
        if gp is not None:
            grads, o = [], 0
            for a in imgs:
                m = gp[o:o + a.size * S].reshape((S,) + a.shape)
                grads.append(m if multi else m[0])
                o += a.size * S
            gw = gw.reshape(S, -1) if multi else gw
        return probs, grads, gw


def _torch_function():
    import torch

    class WNDProbability(torch.autograd.Function):
        """probs = WNDProbability.apply(images (n, H, W) float64, weights (F,)
        float64, model): marginal probabilities (n, C); differentiable in the
        images and the weights through the hand-written backward kernels."""

        @staticmethod
        def forward(ctx, images, weights, model):
            probs, _, _ = model.run(list(images.detach().cpu().numpy()), weights.detach().cpu().numpy())
            ctx.save_for_backward(images, weights)
            ctx.model = model
            return torch.from_numpy(probs).to(images.device)

        @staticmethod
        def backward(ctx, grad_probs):
            images, weights = ctx.saved_tensors
            _, gp, gw = ctx.model.run(list(images.detach().cpu().numpy()), weights.detach().cpu().numpy(),
                                      seed=grad_probs.detach().cpu().numpy())
            gi = torch.from_numpy(np.stack(gp)).to(images.device) if ctx.needs_input_grad[0] else None
            gwt = torch.from_numpy(gw).to(weights.device) if ctx.needs_input_grad[1] else None
            return gi, gwt, None

    return WNDProbability


class _Lazy(object):
    def __init__(self):
        self.fn = None

    def __getattr__(self, k):
        if self.fn is None:
            self.fn = _torch_function()
        return getattr(self.fn, k)


WNDProbability = _Lazy()


def class_evidence_maps(model, images, weights):
    """Per image and class, d p_c / d pixel: (n, C, H, W) for same-size images
    (one forward pass, then one backward pass per class, seeded with that
    class's one-hot vector)."""
    imgs = [np.asarray(a, dtype=np.float64) for a in images]
    n = len(imgs)
    seed = np.tile(np.eye(model.C)[None], (n, 1, 1))  # (n, C seeds, C)
    _, gp, _ = model.run(imgs, weights, seed=seed)
    return np.stack(gp)
