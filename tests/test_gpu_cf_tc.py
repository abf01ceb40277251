"""Chebyshev-Fourier coefficients on the tensor cores (the mixed form, planes
of one size): against the oracle within the mixed form's stated rule for the
group (at most 2 single-count moves per 32-bin histogram), on whole 512 x 512
workload images and on 320 x 320 images (all their planes downsampled to
300 x 300, as the reference does); and the FP32 SIMT form (option cf_tensor_cores = 0) on the
same images under the same rule.  A batch of mixed sizes takes the SIMT form."""
import numpy as np
import pytest

from conftest import golden_names, oracle_features, oracle_lib
from gpu_helpers import images
from parity import compare_mixed
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu

CHAINS = ["()", "(Fourier ())", "(Wavelet ())", "(Chebyshev ())", "(Fourier (Wavelet ()))", "(Edge ())",
          "(Fourier (Edge ()))", "(Wavelet (Edge ()))"]


def _plan():
    import wndcharm
    p = wndcharm.FeatureComputationPlan("cf")
    for c in CHAINS:
        p.add("Chebyshev-Fourier Coefficients %s" % c)
    return p


def _check(eng, plan, imgs):
    names_all = golden_names(1)
    names = plan.feature_names()
    idx = np.array([names_all.index(n) for n in names])
    lib = oracle_lib()
    l0 = eng.launches
    got = eng.extract(plan, imgs)
    launches = eng.launches - l0
    moves = 0
    for i, img in enumerate(imgs):
        exp = oracle_features(lib, img)[idx]
        fails = compare_mixed(got[i], exp, names)
        assert not fails, (img.shape, list(fails.items())[:3])
        moves += int(np.abs(got[i] - exp).sum() // 2)
    return launches, moves


# square images of 300 x 300 or more: every plane (the Wavelet ones included)
# is downsampled to 300 x 300, one size for the whole batch
@pytest.mark.parametrize("sizes", [[(512, 512)] * 3, [(320, 320)] * 4])
def test_tensor_core_sums_within_the_rule(sizes):
    import wndcharm
    from wndcharm import synth
    if sizes[0] == (512, 512):
        imgs, _ = synth.config2(n_per_class=1, size=512, seed=1)
        imgs = imgs[:3]
    else:
        imgs = images(seed=5, sizes=sizes)
    plan = _plan()
    tc = wndcharm.Engine(0, "mixed")
    simt = wndcharm.Engine(0, "mixed")
    simt.set_option("cf_tensor_cores", 0)
    lt, mt = _check(tc, plan, imgs)
    ls, ms = _check(simt, plan, imgs)
    print("sizes %s: single-count moves against the oracle: tensor cores %d, FP32 SIMT %d" % (sizes[0], mt, ms))
    assert lt == ls + 4  # basis, scale, digits, products, chunk sums in place of the SIMT sums


def test_mixed_sizes_take_the_simt_form():
    import wndcharm
    plan = _plan()
    imgs = images(seed=6, sizes=[(96, 80), (64, 64), (50, 71)])
    a = wndcharm.Engine(0, "mixed")
    b = wndcharm.Engine(0, "mixed")
    b.set_option("cf_tensor_cores", 0)
    la, _ = _check(a, plan, imgs)
    lb, _ = _check(b, plan, imgs)
    assert la == lb
