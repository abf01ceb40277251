"""GPU parity per feature family and per transform chain, through the C ABI,
against the CPU oracle on seeded images of several (uneven) sizes."""
import numpy as np
import pytest

from gpu_helpers import CHAINS, images, oracle_group, oracle_transform
from parity import compare
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu

GROUP_C = ["Comb Moments", "Haralick Textures", "Multiscale Histograms", "Tamura Textures", "Radon Coefficients",
           "Fractal Features", "Pixel Intensity Statistics", "Gini Coefficient"]
GROUP_B = ["Chebyshev-Fourier Coefficients", "Chebyshev Coefficients", "Zernike Coefficients"]
GROUP_A = ["Edge Features", "Otsu Object Features", "Inverse-Otsu Object Features", "Gabor Textures"]
READY = {"Comb Moments", "Multiscale Histograms", "Radon Coefficients", "Fractal Features", "Zernike Coefficients",
         "Chebyshev-Fourier Coefficients", "Tamura Textures", "Haralick Textures", "Edge Features", "Otsu Object Features",
         "Inverse-Otsu Object Features", "Gabor Textures",
         "Pixel Intensity Statistics", "Gini Coefficient", "Chebyshev Coefficients"}


@pytest.fixture(scope="module")
def eng():
    import wndcharm
    return wndcharm.Engine(0, "fp64")


def _run(eng, alg, chains, imgs):
    import wndcharm
    plan = wndcharm.FeatureComputationPlan("t")
    for c in chains:
        plan.add("%s %s" % (alg, c))
    got = eng.extract(plan, imgs)
    names = plan.feature_names()
    fails = {}
    for i, img in enumerate(imgs):
        exp = np.concatenate([oracle_group("%s %s" % (alg, c), img) for c in chains])
        f = compare(got[i], exp, names, rtol=1e-7, atol=1e-9, count_moves=0, f14="exact")
        if f:
            fails[i] = f
    return fails


@pytest.mark.parametrize("alg", GROUP_C + GROUP_B)
def test_family_all_chains(eng, alg):
    if alg not in READY:
        pytest.skip("family not on the GPU yet")
    fails = _run(eng, alg, CHAINS, images())
    assert not fails, fails


@pytest.mark.parametrize("alg", GROUP_A)
def test_family_raw(eng, alg):
    if alg not in READY:
        pytest.skip("family not on the GPU yet")
    fails = _run(eng, alg, ["()"], images())
    assert not fails, fails


@pytest.mark.parametrize("name", ["Fourier", "Chebyshev", "Wavelet", "Edge"])
def test_transform(eng, name):
    for img in images():
        got = eng.transform(name, img)
        exp = oracle_transform(name, img)
        assert got.shape == exp.shape
        # all four are bit-identical (the oracle's DFT performs the GPU's Stockham
        # operations in the same order)
        np.testing.assert_array_equal(got, exp)
