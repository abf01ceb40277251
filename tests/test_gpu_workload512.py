"""The benchmark's own images (16 of the 512 x 512 uint16 workload, 4 classes,
seed 1) through both forms, against the unmodified reference build's rows
(tests/golden/reference_build_spread.npz, made by make_f14_spread.py).

Rules: every family at its form's rules with count groups exact (FP64 form;
the mixed form's FP32-binned families at their stated budgets), and Haralick
f14 bit-identical to the oracle's in both forms.  Against the reference build
itself f14 is checked on the entries that are reproducible at all: where the
reference built with and without fused multiply-adds and the oracle agree
(within 1e-6), the GPU must agree too.  The pairs-of-floats f14 chain (option
f14_exact = 0) is reported beside it."""
import hashlib

import numpy as np
import pytest

from conftest import golden, golden_names
from parity import compare, compare_mixed, f14_errors
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    from wndcharm import synth
    sp = golden("reference_build_spread.npz")
    n = int(sp["n_images"])
    per = (n + 3) // 4
    imgs, _ = synth.config2(n_per_class=per, size=512, seed=1)
    order = [c * per + i for i in range(per) for c in range(4)][:n]
    imgs = [imgs[k] for k in order]
    assert [hashlib.sha256(np.ascontiguousarray(im).tobytes()).hexdigest() for im in imgs] == list(sp["img_sha256"]), \
        "the generator no longer reproduces the fixture's images"
    return imgs, sp


def _close(x, y):
    return (np.isnan(x) & np.isnan(y)) | (np.abs(x - y) <= 1e-6 * np.maximum(np.abs(y), 1e-12))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_workload_512_vs_reference_build(prec, workload):
    import wndcharm
    imgs, sp = workload
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    got = wndcharm.Engine(0, prec).extract(plan, imgs)
    names = golden_names(1)
    cmp = compare if prec == "fp64" else compare_mixed
    for i in range(len(imgs)):
        fails = cmp(got[i], sp["ref_rows"][i], names, rtol=1e-7, atol=1e-9)
        assert not fails, (prec, i, list(fails.items())[:3])
    f14i = sp["f14_index"]
    a = got[:, f14i]
    # bit-identical to the oracle's f14 on every entry
    np.testing.assert_array_equal(a, sp["f14_oracle"])
    # and equal to the reference build wherever the reference is reproducible
    r, f, o = sp["f14_ref"], sp["f14_ref_fma"], sp["f14_oracle"]
    stable = _close(o, r) & _close(f, r)
    assert stable.sum() >= 300
    bad = stable & ~_close(a, r)
    assert not bad.any(), np.argwhere(bad)[:8]
    agree, dmax, rmax = f14_errors(a, r)
    print("%s f14 vs the reference build: %.3f agree within 1e-6 (the reference's own two builds: %.3f), max abs %.3g"
          % (prec, agree, f14_errors(f, r)[0], dmax))


def test_pairs_of_floats_f14_option(workload):
    """The mixed form with f14 in pairs of floats (f14_exact = 0): every other
    feature unchanged, f14 finite and in range; its agreement with the oracle
    and the reference builds is printed (it follows a different rounding, as a
    different build of the reference does)."""
    import wndcharm
    imgs, sp = workload
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    eng = wndcharm.Engine(0, "mixed")
    exact = eng.extract(plan, imgs[:4])
    eng.set_option("f14_exact", 0)
    got = eng.extract(plan, imgs[:4])
    f14i = sp["f14_index"]
    others = np.setdiff1d(np.arange(plan.n_features), f14i)
    np.testing.assert_array_equal(got[:, others], exact[:, others])
    a = got[:, f14i]
    assert np.all(np.isfinite(a)) and np.all((a >= 0) & (a <= 1.5))
    print("pairs-of-floats f14 on 4 images: %.3f agree with the oracle, %.3f with the reference build"
          % (f14_errors(a, sp["f14_oracle"][:4])[0], f14_errors(a, sp["f14_ref"][:4])[0]))
