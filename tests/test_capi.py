"""The C-ABI library: builds, loads, exports every entry point the header
declares, and its host-only plan functions reproduce the reference's feature
names and offsets (no GPU needed)."""
import os
import re
import subprocess

import pytest

from conftest import REPO, golden_names
import synth_loader  # noqa: F401


@pytest.fixture(scope="module")
def capi():
    import build as b  # wnd-charm_gb300/build.py
    b.build()
    import wndcharm
    return wndcharm


def test_exports_every_declared_symbol(capi):
    hdr = open(os.path.join(REPO, "include", "wndcharm_gb300.h")).read()
    declared = set(re.findall(r"^\s*(?:const\s+char\s*\*|int|void|long long)\s*(wc_\w+)\s*\(", hdr, re.M))
    assert len(declared) >= 18
    so = os.path.join(REPO, "wnd-charm_gb300", "build", "libwndcharm_gb300.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (wc_\w+)", out))
    assert declared <= exported, declared - exported
    L = capi.lib()
    for s in declared:
        getattr(L, s)


@pytest.mark.parametrize("kind", [0, 1])
def test_standard_plan_names(capi, kind):
    plan = (capi.StdFeatureComputationPlans.getFeatureSetLong() if kind else
            capi.StdFeatureComputationPlans.getFeatureSet())
    assert plan.feature_names() == golden_names(kind)


def test_plan_from_names_and_errors(capi):
    p = capi.FeatureComputationPlan("t")
    p.add("Zernike Coefficients (Fourier (Edge ()))")
    p.add("Gini Coefficient ()")
    assert p.n_features == 73
    assert p.getFeatureNameByIndex(72) == "Gini Coefficient () [0]"
    assert p.groups() == [("Zernike Coefficients (Fourier (Edge ()))", 0, 72), ("Gini Coefficient ()", 72, 1)]
    bad = capi.FeatureComputationPlan("bad")
    bad.add("No Such Algorithm ()")
    with pytest.raises(capi.WndcharmError):
        bad.finalize()
    dup = capi.FeatureComputationPlan("dup")
    dup.add("Gini Coefficient ()")
    dup.add("Gini Coefficient ()")
    with pytest.raises(capi.WndcharmError):
        dup.finalize()


def test_engine_without_gpu_fails_cleanly(capi):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.WndcharmError):
        capi.Engine(0, "fp64")


def test_output_buffers_are_checked(capi):
    """A caller's `out` array must hold exactly the rows the library writes
    (float64, C-contiguous, writable); anything else is refused before a call."""
    import numpy as np
    ob = capi._out_buffer
    assert ob(None, 3, 5).shape == (3, 5)
    good = np.zeros((3, 5))
    assert ob(good, 3, 5) is good
    ro = np.zeros((3, 5))
    ro.flags.writeable = False
    for bad in (np.zeros((3, 4)), np.zeros((5, 3)), np.zeros((3, 5), np.float32), np.zeros((5, 3)).T,
                np.zeros((3, 10))[:, ::2], ro, [[0.0] * 5] * 3):
        with pytest.raises(capi.WndcharmError):
            ob(bad, 3, 5)


def test_wnd_arguments_are_checked(capi):
    """WND-5 wrappers hand the library pointers it reads N x F, N, T x F and F
    values through: mismatched shapes are refused on the host, arrays that
    already have the layout pass through without a copy."""
    import numpy as np
    X = np.zeros((6, 4))
    y = np.arange(6, dtype=np.int32)
    T = np.zeros((3, 4))
    X2, y2, T2 = capi._wnd_rows(X, y, T)
    assert X2 is X and y2 is y and T2 is T
    assert capi._wnd_rows(X, list(range(6)))[1].dtype == np.int32
    assert capi._wnd_rows(X, y, np.zeros(4))[2].shape == (1, 4)  # one test row
    for args in ((X, y[:5]), (X, y.reshape(6, 1)), (np.zeros(6), y), (X, y, np.zeros((3, 5)))):
        with pytest.raises(capi.WndcharmError):
            capi._wnd_rows(*args)
    w = np.ones(4)
    assert capi._wnd_vecs(4, w, [0, 0, 0, 0])[0] is w
    with pytest.raises(capi.WndcharmError):
        capi._wnd_vecs(4, w, np.ones(3))
