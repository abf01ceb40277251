"""Preprocessing and sampling on the GPU (wc_preprocess, wc_extract_samples)
against the reference's outputs and the oracle: crop, Downsample,
normalisation (the reference's sequential Welford mean and standard
deviation), rotations and tiles bit for bit; features of every sample against
the oracle's, and of two samples against the reference's."""
import ctypes

import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_lib
from parity import compare, compare_mixed
import synth_loader  # noqa: F401
from test_preproc_cpu import BITS, CASES, oracle_preprocess, sampling_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import wndcharm
    return wndcharm.Engine(0, "fp64")


@pytest.mark.parametrize("case", CASES)
def test_preprocess_matches_reference(eng, case):
    import wndcharm
    g = golden("reference_preproc.npz")
    src = str(g["src_" + case])
    img, opt, ok = g["img_" + src], g["opt_" + case], g["ok_" + case]
    s = sampling_of(opt)
    for k in range(len(ok)):
        if not ok[k]:
            with pytest.raises(wndcharm.WndcharmError):
                eng.preprocess(img, s, k, BITS[src])
            continue
        got = eng.preprocess(img, s, k, BITS[src])
        ref = g["%s_%d" % (case, k)]
        assert got.shape == ref.shape
        np.testing.assert_array_equal(got, ref, err_msg="%s sample %d" % (case, k))


def test_preprocess_device_input_and_output(eng):
    """On-device input image and on-device output plane (torch buffers)."""
    import torch
    import wndcharm
    from wndcharm import _lib
    g = golden("reference_preproc.npz")
    img, opt, ok = g["img_a"], g["opt_tiles"], g["ok_tiles"]
    s = sampling_of(opt)
    dev = torch.from_numpy(img.astype(np.int32)).to(torch.int16).cuda()  # 12-bit values fit int16
    k = [j for j in range(6, len(ok)) if ok[j]][0]  # a tile of a rotated plane
    w, h = s.sample_size(img.shape[1], img.shape[0], k)
    out = torch.zeros(h * w, dtype=torch.float64, device="cuda")
    d = _lib.wc_image_desc(dev.data_ptr(), _lib.WC_U16, img.shape[1], img.shape[0], 16, 1)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    st = s.struct()
    wndcharm.check(_lib.lib().wc_preprocess(eng._h, ctypes.byref(d), ctypes.byref(st), k, out.data_ptr(), out.numel(),
                                            ctypes.byref(ow), ctypes.byref(oh), 1))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().reshape(h, w), g["tiles_%d" % k])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_extract_samples_vs_oracle_and_reference(prec):
    """All 16 samples (4 rotations x 2 x 2 tiles) of a cropped, downsampled,
    normalised reference image in one call: every row against the oracle's
    features of the oracle's sample; rows 0 and 5 against the reference's."""
    import wndcharm
    g = golden("reference_preproc.npz")
    img, opt = g["img_c"], g["opt_full"]
    s = sampling_of(opt)
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    eng = wndcharm.Engine(0, prec)
    rows = eng.extract_samples(plan, [img, img[::-1].copy()], s, bits=16)
    assert rows.shape == (32, 2919)
    names = golden_names(1)
    lib = oracle_lib()
    cmp = compare if prec == "fp64" else compare_mixed
    for i, im in enumerate((img, img[::-1].copy())):
        for k in range(16):
            plane = oracle_preprocess(lib, im, 16, opt, k)
            exp = oracle_features(lib, plane, bits=16)
            fails = cmp(rows[16 * i + k], exp, names)
            assert not fails, (prec, i, k, list(fails.items())[:3])
    for k in (0, 5):
        fails = cmp(rows[k], g["full_%d_long" % k], names)
        assert not fails, (prec, "reference", k, list(fails.items())[:3])


def test_extract_samples_refuses_a_tile_outside(eng):
    import wndcharm
    g = golden("reference_preproc.npz")
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSet()
    with pytest.raises(wndcharm.WndcharmError):
        eng.extract_samples(plan, [g["img_a"]], sampling_of(g["opt_tiles"]))
    # the engine stays usable
    out = eng.extract_samples(plan, [g["img_a"]], wndcharm.Sampling(downsample=50))
    assert out.shape == (1, 1059) and np.isfinite(out).sum() > 1000


def test_image_matrix_methods(tmp_path):
    """ImageMatrix.OpenImage with downsampling and normalisation, submatrix,
    Downsample, normalize and Rotate: same planes as the oracle's chain."""
    import wndcharm
    t = golden("reference_tiff.npz")
    p = tmp_path / "t1.tif"
    p.write_bytes(t["t1_s01_c05_ij"].tobytes())
    lib = oracle_lib()
    pix, bits = wndcharm.read_tiff(str(p))
    im = wndcharm.ImageMatrix()
    assert im.OpenImage(str(p), downsample=60, bounding_rect=(3, 4, 90, 80), mean=1500, stddev=400) == 1
    opt = np.array([3, 4, 90, 80, 0.6, 0.6, -1, -1, -1, 1500, 400, 1, 1, 1], dtype=np.float64)
    np.testing.assert_array_equal(im.pix_plane, oracle_preprocess(lib, pix, bits, opt, 0))
    r = wndcharm.ImageMatrix()
    r.Rotate(im, 90)
    np.testing.assert_array_equal(r.pix_plane, np.rot90(im.pix_plane, -1))
    r.Rotate(im, 270)
    np.testing.assert_array_equal(r.pix_plane, im.pix_plane.T)
    sub = wndcharm.ImageMatrix()
    assert sub.submatrix(im, 5, 6, 30, 40) == 1
    np.testing.assert_array_equal(sub.pix_plane, im.pix_plane[6:41, 5:31])
    assert sub.submatrix(im, 5, 6, 300, 40) == 0
    ds = wndcharm.ImageMatrix()
    ds.Downsample(sub, 0.5, 0.7)
    opt = np.array([-1, -1, -1, -1, 0.5, 0.7, -1, -1, -1, -1, -1, 1, 1, 1], dtype=np.float64)
    np.testing.assert_array_equal(ds.pix_plane, oracle_preprocess(lib, sub.pix_plane, 16, opt, 0))
    ds.normalize(100, 2000, 255, -1, -1)
    opt = np.array([-1, -1, -1, -1, 1, 1, 100, 2000, 255, -1, -1, 1, 1, 1], dtype=np.float64)
    prev = oracle_preprocess(lib, sub.pix_plane, 16, np.array([-1, -1, -1, -1, 0.5, 0.7, -1, -1, -1, -1, -1, 1, 1, 1.0]), 0)
    np.testing.assert_array_equal(ds.pix_plane, oracle_preprocess(lib, prev, 16, opt, 0))
