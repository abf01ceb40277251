"""The .sig and .fit text files: parsing the reference's own files, and writing
them back byte for byte."""
import numpy as np

from conftest import golden
import synth_loader  # noqa: F401
from wndcharm import sigfile


def _text(key):
    return str(golden("reference_text.npz")[key])


def test_sig_parse_matches_reference_values():
    imgs = golden("reference_images.npz")
    for key, img in (("sig_010067", "010067_301x300"), ("sig_t1", "t1_s01_c05_ij")):
        s = sigfile.parse_sig(_text(key))
        assert s["version"] == 4 and s["fv_type"] == sigfile.FV_LONG
        assert len(s["values"]) == 2919 and len(s["names"]) == 2919
        np.testing.assert_array_equal(s["values"], imgs["sig_" + img])
        assert s["names"][0] == "Edge Features () [0]"


def test_sig_write_is_byte_identical():
    for key in ("sig_010067", "sig_t1"):
        text = _text(key)
        s = sigfile.parse_sig(text)
        out = sigfile.format_sig(s["values"], s["names"], s["sample_class"], s["full_path"], s["version"], s["fv_type"])
        assert out == text


def test_fit_roundtrip_is_byte_identical():
    text = _text("fit_unbalanced")
    f = sigfile.parse_fit(text)
    assert f["X"].shape == (8, 2919)
    assert f["class_labels"][1:] == sorted(set(f["class_labels"][1:]), key=f["class_labels"].index)
    out = sigfile.format_fit(f["X"], f["classes"], f["names"], f["class_labels"], f["paths"], f["version"], f["fv_type"])
    assert out == text


def test_sig_roundtrip_of_computed_row(tmp_path):
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(size=50) * 10.0 ** rng.integers(-8, 8, size=50), [0.0, -0.0, 7.0, np.nan]])
    names = ["f [%d]" % i for i in range(len(v))]
    p = tmp_path / "x.sig"
    sigfile.write_sig(p, v, names, sample_class=3, full_path="a/b.tif")
    s = sigfile.read_sig(p)
    assert s["sample_class"] == 3 and s["full_path"] == "a/b.tif" and s["names"] == names
    fin = np.isfinite(v)
    np.testing.assert_allclose(s["values"][fin], v[fin], rtol=6e-8, atol=0)  # 8 significant digits
    assert np.isnan(s["values"][~fin]).all()
