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
