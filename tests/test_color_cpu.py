"""Colour images and the colour plans on the CPU: the oracle's RGB ingest (gray
and HSV planes), fuzzy colour classifier and colour-plan features against the
reference's own (its LoadTIFF and plans, with the terminator its fuzzy-colour
loader omits), and the C ABI's colour-plan names."""
import ctypes

import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features_rgb, oracle_lib
from parity import compare
import synth_loader  # noqa: F401

D = ctypes.POINTER(ctypes.c_double)
BITS = {"rgb8": 8, "rgb16": 16}


@pytest.mark.parametrize("key", ["rgb8", "rgb16"])
def test_oracle_rgb_ingest_matches_reference(key):
    g = golden("reference_colour.npz")
    img = g["img_" + key]
    h, w = img.shape[:2]
    gray, hsv = np.zeros(w * h), np.zeros(3 * w * h, dtype=np.uint8)
    oracle_lib().wco_load_rgb(ctypes.c_void_p(img.ctypes.data), w, h, BITS[key], gray.ctypes.data_as(D),
                              ctypes.c_void_p(hsv.ctypes.data))
    np.testing.assert_array_equal(gray.reshape(h, w), g["gray_" + key])
    np.testing.assert_array_equal(hsv.reshape(h, w, 3), g["hsv_" + key])


def test_oracle_find_colour_matches_reference():
    g = golden("reference_colour.npz")
    lib = oracle_lib()
    got = np.array([lib.wco_find_colour(int(a), int(b), int(c)) for a, b, c in g["fc_hsv"]])
    np.testing.assert_array_equal(got, g["fc_colour"])
    assert len(set(got.tolist())) >= 15  # the sample reaches most colours


@pytest.mark.parametrize("key,kind", [("rgb8", 2), ("rgb8", 3), ("rgb16", 2), ("rgb16", 3), ("grid", 2)])
def test_oracle_colour_plans_match_reference(key, kind):
    g = golden("reference_colour.npz")
    got = oracle_features_rgb(oracle_lib(), g["img_" + key], BITS.get(key, 8), kind)
    fails = compare(got, g["plan%d_%s" % (kind, key)], golden_names(kind))
    assert not fails, list(fails.items())[:3]


def test_color_transform_groups_are_the_root_groups():
    """The reference's plans name a "Color Transform" that resolves to a copy of
    the image: those groups repeat the root groups."""
    g = golden("reference_colour.npz")
    names = golden_names(3)
    f = g["plan3_rgb8"]
    idx = {n: i for i, n in enumerate(names)}
    for n in names:
        if "(Color Transform ())" in n:
            np.testing.assert_array_equal(f[idx[n]], f[idx[n.replace("(Color Transform ())", "()")]])


@pytest.mark.parametrize("kind", [2, 3])
def test_capi_colour_plan_names(kind):
    import build as b  # wnd-charm_gb300/build.py
    b.build()
    import wndcharm
    plan = (wndcharm.StdFeatureComputationPlans.getFeatureSetColor() if kind == 2 else
            wndcharm.StdFeatureComputationPlans.getFeatureSetLongColor())
    assert plan.feature_names() == golden_names(kind)
    p = wndcharm.FeatureComputationPlan("c")
    p.add("Zernike Coefficients (Fourier (Hue ()))")
    p.add("Color Histogram ()")
    p.add("Haralick Textures (Color ())")
    p.add("Gini Coefficient (Color Transform ())")
    assert p.n_features == 72 + 20 + 28 + 1
