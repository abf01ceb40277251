"""Pins the CPU oracle (oracle/wc_oracle.cpp) to the reference: its feature
names, feature values, transform images and WND-5 results against the golden
fixtures (reference fixtures + outputs of the unmodified reference build)."""
import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_wnd
from parity import F14, compare, index_of, group_of
import synth_loader  # noqa: F401  (puts the package on sys.path)
from wndcharm import synth


def test_names_match_reference(oracle):
    import ctypes
    buf = ctypes.create_string_buffer(512)
    for kind in (0, 1):
        ref = golden_names(kind)
        assert oracle.wco_plan_n_features(kind) == len(ref) == (2919 if kind else 1059)
        for i, n in enumerate(ref):
            oracle.wco_plan_feature_name(kind, i, buf, 512)
            assert buf.value.decode() == n


@pytest.mark.parametrize("key", ["t1_s01_c05_ij", "binuc1", "010067_301x300"])
def test_golden_images(oracle, key):
    g = golden("reference_images.npz")
    names = golden_names(1)
    img, bits = g["img_" + key], int(g["bits_" + key])
    got = oracle_features(oracle, img, bits)
    # against the reference build (current f14): same arithmetic, tight
    assert not compare(got, g["ref_" + key], names, rtol=1e-9, atol=1e-12, count_moves=0)
    # against the reference's precalculated signatures (%.8g text, pre-2017 f14)
    f14 = np.array([group_of(n).startswith("Haralick") and index_of(n) in F14 for n in names])
    sig = g["sig_" + key]
    rel = np.abs(got - sig) / np.maximum(np.abs(sig), 1e-300)
    bad = (rel > 1e-6) & (np.abs(got - sig) > 1e-7) & ~f14
    assert not bad.any(), np.nonzero(bad)[0][:10]


@pytest.mark.parametrize("i", range(6))
def test_synthetic_long_and_short(oracle, i):
    g = golden("reference_synthetic.npz")
    img = g["img_%d" % i]
    for kind, key in ((1, "long_%d" % i), (0, "short_%d" % i)):
        got = oracle_features(oracle, img, 16, kind)
        assert not compare(got, g[key], golden_names(kind), rtol=1e-9, atol=1e-12, count_moves=0)


def test_uint8_image(oracle):
    g = golden("reference_synthetic.npz")
    got = oracle_features(oracle, g["img_u8"], 8, 1)
    assert not compare(got, g["long_u8"], golden_names(1), rtol=1e-9, atol=1e-12, count_moves=0)


@pytest.mark.parametrize("name", ["Fourier", "Chebyshev", "Wavelet", "Edge"])
def test_transforms(oracle, name):
    import ctypes
    from conftest import D
    g = golden("reference_transforms.npz")
    for i in range(2):
        img = np.ascontiguousarray(g["img_%d" % i], dtype=np.float64)
        exp = g["%s_%d" % (name, i)]
        out = np.zeros(4 * img.size + 4096)
        ow, oh = ctypes.c_int(), ctypes.c_int()
        assert oracle.wco_transform(name.encode(), img.ctypes.data_as(D), img.shape[1], img.shape[0],
                                    out.ctypes.data_as(D), ctypes.byref(ow), ctypes.byref(oh)) == 0
        got = out[: ow.value * oh.value].reshape(oh.value, ow.value)
        assert got.shape == exp.shape
        np.testing.assert_allclose(got, exp, rtol=1e-11, atol=1e-9 * np.abs(exp).max())


@pytest.mark.parametrize("h,w", [(64, 64), (48, 40), (37, 53), (60, 70), (30, 29)])
def test_fourier_against_numpy(oracle, h, w):
    """The oracle's DFT (radix-2/4/8 butterflies, odd primes direct; the GPU's
    Fourier node reproduces it bit for bit): |DFT| equals numpy's |fft2| to
    FP64 accuracy, for power-of-two, odd and prime sides."""
    import ctypes
    from conftest import D
    rng = np.random.default_rng(h * 100 + w)
    img = np.ascontiguousarray(rng.integers(0, 4096, size=(h, w)), dtype=np.float64)
    out = np.zeros(4 * img.size + 4096)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    assert oracle.wco_transform(b"Fourier", img.ctypes.data_as(D), w, h, out.ctypes.data_as(D),
                                ctypes.byref(ow), ctypes.byref(oh)) == 0
    got = out[: ow.value * oh.value].reshape(oh.value, ow.value)
    exp = np.abs(np.fft.fft2(img))
    assert got.shape == exp.shape
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-12 * exp.max())


def test_wnd_classify_fixture(oracle):
    """test01-classify.pl: classify -l test-l.fit test-l.fit (3-decimal table)."""
    g = golden("reference_wnd.npz")
    X, y = g["fit_X"], g["fit_y"]
    w, mn, mx, p, pred = oracle_wnd(oracle, X, y, X, 2, 0.15)
    np.testing.assert_array_equal(pred, g["classify_pred"])
    np.testing.assert_allclose(p, g["classify_table"][:, 1:3], atol=5e-4 + 1e-12)
    np.testing.assert_array_equal(w, g["ref_w"])
    np.testing.assert_array_equal(p, g["ref_p"])
    np.testing.assert_array_equal(pred, g["ref_pred"])


def test_wnd_fisher_weights_fixture(oracle):
    """test_fit-l.weights: wndchrm classify -l -f1.0 on test-l.fit (printed %f)."""
    g = golden("reference_wnd.npz")
    X, y = g["fit_X"], g["fit_y"]
    w, *_ = oracle_wnd(oracle, X, y, X[:1], 2, 1.0)
    np.testing.assert_allclose(w, g["weights_f1"], atol=1e-5)


def test_wnd_synthetic(oracle):
    g = golden("reference_wnd.npz")
    xtr, ytr, xte, _ = synth.feature_vectors(300, 40, 2919, 10, 4)
    w, mn, mx, p, pred = oracle_wnd(oracle, xtr, ytr, xte, 10, 0.15)
    np.testing.assert_array_equal(w, g["syn_w"])
    np.testing.assert_array_equal(pred, g["syn_pred"])
    np.testing.assert_allclose(p, g["syn_p"], rtol=1e-12, atol=0)
