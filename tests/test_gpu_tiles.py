"""Uneven batches of ROI tiles (the batched uneven-sizes workload, scaled down):
images with independent widths and heights from {64, 96, ..., 1024} cut into
4 x 4 tiles as wndchrm samples them, all tiles of all images in one batch;
tiles checked against the oracle and against single-tile extraction."""
import time

import numpy as np
import pytest

from conftest import golden_names, oracle_features, oracle_lib
from parity import compare
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


def test_uneven_tiles_one_batch():
    import wndcharm
    from wndcharm import synth
    rng = np.random.default_rng(2)
    sizes = [(int(rng.choice(np.arange(64, 1025, 32))), int(rng.choice(np.arange(64, 1025, 32)))) for _ in range(6)]
    imgs = [synth.blob_image(rng, i % 8, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
            for i, (w, h) in enumerate(sizes)]
    tl = [t for im in imgs for t in wndcharm.tiles(im, 4, 4)]
    assert len(tl) == 16 * len(imgs)
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    eng = wndcharm.Engine(0, "fp64")
    eng.extract(plan, tl[:4])
    t0 = time.perf_counter()
    got = eng.extract(plan, tl)
    dt = time.perf_counter() - t0
    print("%d tiles (%s) in one batch: %.2f s, %.1f tiles/s" % (len(tl), sorted({t.shape for t in tl})[:3], dt, len(tl) / dt))
    names = golden_names(1)
    lib = oracle_lib()
    for k in (0, 17, 42, len(tl) - 1):
        exp = oracle_features(lib, np.ascontiguousarray(tl[k]))
        fails = compare(got[k], exp, names, rtol=1e-7, atol=1e-9, count_moves=0, f14="exact")
        assert not fails, (k, tl[k].shape, list(fails.items())[:3])
        np.testing.assert_array_equal(eng.extract(plan, [np.ascontiguousarray(tl[k])])[0], got[k])


def test_device_tiles_equal_host_tiles():
    """Tiles cut on the GPU (wc_extract_samples) give the same rows, bit for
    bit, as the same tiles cut on the host and extracted as images."""
    import wndcharm
    from wndcharm import synth
    rng = np.random.default_rng(21)
    imgs = [synth.blob_image(rng, i, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
            for i, (w, h) in enumerate([(130, 97), (64, 200), (257, 66)])]
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    for prec in ("fp64", "mixed"):
        eng = wndcharm.Engine(0, prec)
        dev = eng.extract_samples(plan, imgs, wndcharm.Sampling(tiles_x=4, tiles_y=4))
        host = eng.extract(plan, [t for im in imgs for t in wndcharm.tiles(im, 4, 4)])
        assert dev.shape == host.shape == (48, 2919)
        np.testing.assert_array_equal(dev, host)
