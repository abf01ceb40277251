"""Seeded synthetic image and feature-vector generators for the benchmark
workloads and the tests.

Images: a Gaussian-noise background, K Gaussian blobs and a sinusoidal
grating, clipped to the pixel range.  For class c: K ~ U{5+5c .. 15+5c},
blob sigma ~ U[3, 3+2c] px, amplitude ~ U[80, 200] (times ``scale``), centres
uniform, grating period 8+4c px with a random orientation and amplitude 15
(times ``scale``).
"""
import numpy as np


def blob_image(rng, cls, width, height, mean=20.0, sd=5.0, scale=1.0, maxval=255):
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float64)
    img = rng.normal(mean, sd, size=(height, width))
    k = int(rng.integers(5 + 5 * cls, 15 + 5 * cls + 1))
    for _ in range(k):
        s = rng.uniform(3.0, 3.0 + 2.0 * cls)
        a = rng.uniform(80.0, 200.0) * scale
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        img += a * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2.0 * s * s))
    period = 8.0 + 4.0 * cls
    th = rng.uniform(0, np.pi)
    img += 15.0 * scale * np.sin(2.0 * np.pi * (xx * np.cos(th) + yy * np.sin(th)) / period)
    return np.clip(np.rint(img), 0, maxval)


def image_set(n_classes, per_class, width, height, seed, bits=8, sizes=None):
    """Returns (list of 2-D uint8/uint16 arrays, labels 1..C)."""
    rng = np.random.default_rng(seed)
    if bits == 8:
        kw = dict(mean=20.0, sd=5.0, scale=1.0, maxval=255)
        dt = np.uint8
    else:
        kw = dict(mean=320.0, sd=80.0, scale=16.0, maxval=4095)
        dt = np.uint16
    imgs, labels = [], []
    for c in range(n_classes):
        for i in range(per_class):
            w, h = (width, height) if sizes is None else sizes[len(imgs)]
            imgs.append(blob_image(rng, c, w, h, **kw).astype(dt))
            labels.append(c + 1)
    return imgs, np.array(labels, dtype=np.int32)


def config2(n_per_class=128, size=512, seed=1):
    """4 classes x n, uint16 12-bit, size x size (the long-set headline workload)."""
    return image_set(4, n_per_class, size, size, seed, bits=16)


def uneven_sizes(n, seed, lo=64, hi=1024, step=32):
    rng = np.random.default_rng(seed)
    sides = np.arange(lo, hi + 1, step)
    return [(int(rng.choice(sides)), int(rng.choice(sides))) for _ in range(n)]


def feature_vectors(n_train, n_test, n_features, n_classes, seed):
    """Per-feature values ~ N(mu_cf, 1), class means mu_cf ~ N(0, 0.5)."""
    rng = np.random.default_rng(seed)
    mu = rng.normal(0.0, 0.5, size=(n_classes, n_features))
    ytr = rng.integers(0, n_classes, size=n_train)
    yte = rng.integers(0, n_classes, size=n_test)
    xtr = mu[ytr] + rng.normal(size=(n_train, n_features))
    xte = mu[yte] + rng.normal(size=(n_test, n_features))
    return xtr, (ytr + 1).astype(np.int32), xte, (yte + 1).astype(np.int32)


def config4(n=256, size=256, n_classes=4, seed=3, dtype=np.float32):
    """The differentiation workload: float32 images in [0, 1] from the same
    blob + grating generator, not rounded (background N(0.08, 0.02), blob
    amplitudes U[0.3, 0.8], grating amplitude 0.06; shifted up when below 0 and
    scaled down when above 1), classes interleaved.
    Returns (list of 2-D float32 arrays, labels 1..C)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:size, 0:size].astype(np.float64)
    imgs, labels = [], []
    for i in range(n):
        c = i % n_classes
        img = rng.normal(0.08, 0.02, size=(size, size))
        k = int(rng.integers(5 + 5 * c, 15 + 5 * c + 1))
        for _ in range(k):
            s = rng.uniform(3.0, 3.0 + 2.0 * c) * size / 256.0
            a = rng.uniform(0.3, 0.8)
            cx, cy = rng.uniform(0, size), rng.uniform(0, size)
            img += a * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2.0 * s * s))
        period = (8.0 + 4.0 * c) * size / 256.0
        th = rng.uniform(0, np.pi)
        img += 0.06 * np.sin(2.0 * np.pi * (xx * np.cos(th) + yy * np.sin(th)) / period)
        # into [0, 1] by a shift and a scale rather than clipping, so that no
        # plateau of equal pixels (a kink of max / order statistics) appears
        img = img - min(0.0, img.min())
        img = img / max(1.0, img.max())
        imgs.append(img.astype(dtype))
        labels.append(c + 1)
    return imgs, np.array(labels, dtype=np.int32)
