"""Colour images on the GPU: the colour plans (2199 and 4059 features) in both
forms against the reference's features and the oracle's, the fuzzy colour
classifier through the Color Histogram of an image of 65,536 distinct colours
(exact counts), custom plans on the Color transform, and the grayscale plans
on RGB input (the gray plane LoadTIFF makes)."""
import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_features_rgb, oracle_lib
from parity import compare, compare_mixed
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu
BITS = {"rgb8": 8, "rgb16": 16, "grid": 8}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_colour_plans_vs_reference_and_oracle(prec):
    import wndcharm
    g = golden("reference_colour.npz")
    eng = wndcharm.Engine(0, prec)
    cmp = compare if prec == "fp64" else compare_mixed
    lib = oracle_lib()
    for kind in (2, 3):
        plan = (wndcharm.StdFeatureComputationPlans.getFeatureSetColor() if kind == 2 else
                wndcharm.StdFeatureComputationPlans.getFeatureSetLongColor())
        names = golden_names(kind)
        for key in ("rgb8", "rgb16"):
            got = eng.extract(plan, [g["img_" + key]], bits=BITS[key])[0]
            fails = cmp(got, g["plan%d_%s" % (kind, key)], names)
            assert not fails, (prec, kind, key, "reference", list(fails.items())[:3])
            fails = cmp(got, oracle_features_rgb(lib, g["img_" + key], BITS[key], kind), names)
            assert not fails, (prec, kind, key, "oracle", list(fails.items())[:3])


def test_colour_histogram_of_many_colours_is_exact():
    import wndcharm
    g = golden("reference_colour.npz")
    eng = wndcharm.Engine(0, "fp64")
    p = wndcharm.FeatureComputationPlan("hist")
    p.add("Color Histogram ()")
    got = eng.extract(p, [g["img_grid"]], bits=8)[0]
    names = golden_names(2)
    ref = g["plan2_grid"][[i for i, n in enumerate(names) if n.startswith("Color Histogram ()")]]
    np.testing.assert_array_equal(got, ref)


def test_custom_colour_groups_and_batches():
    """The Color transform (fuzzy colour index as a level), Hue chains and a
    mixed batch of RGB images of different sizes and depths, against the oracle."""
    import wndcharm
    g = golden("reference_colour.npz")
    groups = ["Multiscale Histograms (Color ())", "Pixel Intensity Statistics (Color ())",
              "Haralick Textures (Color ())", "Zernike Coefficients (Fourier (Hue ()))", "Color Histogram ()",
              "Gini Coefficient (Color Transform ())"]
    p = wndcharm.FeatureComputationPlan("custom")
    for n in groups:
        p.add(n)
    eng = wndcharm.Engine(0, "fp64")
    imgs = [g["img_rgb8"], g["img_grid"][:100, :77].copy(), g["img_rgb16"]]
    bits = [8, 8, 16]
    got = np.stack([eng.extract(p, [im], bits=b)[0] for im, b in zip(imgs, bits)])
    lib = oracle_lib()
    names = p.feature_names()
    for i, (im, b) in enumerate(zip(imgs, bits)):
        exp = np.zeros(p.n_features)
        off = 0
        for n in groups:
            one = wndcharm.FeatureComputationPlan("one")
            one.add(n)
            k = one.n_features
            exp[off:off + k] = _oracle_group_rgb(lib, n, im, b)
            off += k
        fails = compare(got[i], exp, names, f14="exact")
        assert not fails, (i, list(fails.items())[:3])


def _oracle_group_rgb(lib, group, img, bits):
    """One group on an RGB image through the oracle's long colour plan (groups
    it contains) or its custom-group entry on the Color transform's plane."""
    names3 = golden_names(3)
    idx = [i for i, n in enumerate(names3) if n.rsplit(" [", 1)[0] == group]
    if idx:
        return oracle_features_rgb(lib, img, bits, 3)[idx]
    # a group on the Color transform: the oracle's transform, then the group on its plane
    import ctypes
    a = np.ascontiguousarray(img)
    h, w = a.shape[:2]
    gray, hsv = np.zeros(w * h), np.zeros(3 * w * h, dtype=np.uint8)
    lib.wco_load_rgb(ctypes.c_void_p(a.ctypes.data), w, h, bits, gray.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                     ctypes.c_void_p(hsv.ctypes.data))
    levels = np.array([int((255.0 * lib.wco_find_colour(int(x), int(y), int(z))) / 19) for x, y, z in
                       hsv.reshape(-1, 3)], dtype=np.float64).reshape(h, w)
    alg = group.split(" (")[0] + " ()"
    D = ctypes.POINTER(ctypes.c_double)
    one = np.zeros(200)
    k = lib.wco_extract_group(alg.encode(), np.ascontiguousarray(levels).ctypes.data_as(D), w, h, 8,
                              one.ctypes.data_as(D))
    return one[:k]


def test_gray_plans_on_rgb_input_read_the_gray_plane():
    import wndcharm
    g = golden("reference_colour.npz")
    eng = wndcharm.Engine(0, "fp64")
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    got = eng.extract(plan, [g["img_rgb8"]], bits=8)[0]
    exp = oracle_features(oracle_lib(), g["gray_rgb8"], bits=8)
    fails = compare(got, exp, golden_names(1), f14="exact")
    assert not fails, list(fails.items())[:3]


def test_colour_plan_needs_rgb():
    import wndcharm
    eng = wndcharm.Engine(0, "fp64")
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetColor()
    with pytest.raises(wndcharm.WndcharmError):
        eng.extract(plan, [np.zeros((32, 32), dtype=np.uint16)])
    p = wndcharm.FeatureComputationPlan("bad")
    p.add("Zernike Coefficients (Hue (Fourier ()))")
    with pytest.raises(wndcharm.WndcharmError):
        eng.extract(p, [golden("reference_colour.npz")["img_rgb8"]], bits=8)
