"""Preprocessing and sampling (crop, Downsample, normalize, Rotate, tiles) on
the CPU: the oracle against the reference's own outputs (bit for bit), the C
ABI's host-side sample geometry against the reference's sizes and refusals,
and the oracle's features of the reference's samples."""
import ctypes

import numpy as np
import pytest

from conftest import golden, golden_names, oracle_features, oracle_lib
from parity import compare
import synth_loader  # noqa: F401

D = ctypes.POINTER(ctypes.c_double)
CASES = ["crop", "ds50", "ds37", "ds_xy", "norm_ms", "norm_m", "norm_mm", "norm_both", "rot4", "tiles", "u8", "full",
         "crop_bad"]
BITS = {"a": 16, "b": 8, "c": 16}


def oracle_preprocess(lib, img, bits, opt, sample):
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(pix.size + 64)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    o = np.ascontiguousarray(opt, dtype=np.float64)
    r = lib.wco_preprocess(pix.ctypes.data_as(D), img.shape[1], img.shape[0], bits, o.ctypes.data_as(D), sample,
                           out.ctypes.data_as(D), ctypes.c_long(out.size), ctypes.byref(ow), ctypes.byref(oh))
    if r:
        return None
    return out[: ow.value * oh.value].reshape(oh.value, ow.value)


def sampling_of(opt):
    import wndcharm
    return wndcharm.Sampling(bounding_rect=tuple(int(v) for v in opt[:4]) if opt[0] >= 0 else None,
                             ratio_x=opt[4], ratio_y=opt[5], norm_min=opt[6], norm_max=opt[7], norm_range=int(opt[8]),
                             mean=opt[9], stddev=opt[10], rotations=int(opt[11]), tiles_x=int(opt[12]),
                             tiles_y=int(opt[13]))


@pytest.mark.parametrize("case", CASES)
def test_oracle_preprocess_matches_reference(case):
    g = golden("reference_preproc.npz")
    lib = oracle_lib()
    src = str(g["src_" + case])
    img, opt, ok = g["img_" + src], g["opt_" + case], g["ok_" + case]
    for k in range(len(ok)):
        got = oracle_preprocess(lib, img, BITS[src], opt, k)
        assert (got is not None) == bool(ok[k]), (case, k)
        if ok[k]:
            np.testing.assert_array_equal(got, g["%s_%d" % (case, k)], err_msg="%s sample %d" % (case, k))


@pytest.mark.parametrize("case", CASES)
def test_capi_sample_geometry_matches_reference(case):
    """wc_sample_size (host code of the C ABI, no GPU): sizes and refusals."""
    import build as b  # wnd-charm_gb300/build.py
    b.build()
    import wndcharm
    g = golden("reference_preproc.npz")
    src = str(g["src_" + case])
    img, opt, ok = g["img_" + src], g["opt_" + case], g["ok_" + case]
    s = sampling_of(opt)
    assert s.count == len(ok)
    for k in range(len(ok)):
        if ok[k]:
            ref = g["%s_%d" % (case, k)]
            assert s.sample_size(img.shape[1], img.shape[0], k) == (ref.shape[1], ref.shape[0]), (case, k)
        else:
            with pytest.raises(wndcharm.WndcharmError):
                s.sample_size(img.shape[1], img.shape[0], k)


def test_sampling_options_are_checked():
    import build as b
    b.build()
    import wndcharm
    for bad in (dict(rotations=0), dict(rotations=5), dict(tiles_x=0), dict(ratio_x=0.0), dict(ratio_y=-1.0),
                dict(ratio_x=float("nan"))):
        with pytest.raises(wndcharm.WndcharmError):
            wndcharm.Sampling(**bad).sample_size(64, 64)
    # a rectangle outside the image, and downsampling to nothing
    with pytest.raises(wndcharm.WndcharmError):
        wndcharm.Sampling(bounding_rect=(10, 10, 60, 10)).sample_size(64, 64)
    with pytest.raises(wndcharm.WndcharmError):
        wndcharm.Sampling(ratio_x=0.01).sample_size(64, 64)
    # OpenImage's percentage form: 100 (and 0) means no downsampling
    assert wndcharm.Sampling(downsample=100).sample_size(64, 50) == (64, 50)
    assert wndcharm.Sampling(downsample=50).sample_size(64, 50) == (32, 25)


def test_oracle_features_of_reference_samples():
    """The oracle's long-plan features of the reference's preprocessed samples
    against the reference's own features of the same samples."""
    g = golden("reference_preproc.npz")
    lib = oracle_lib()
    names = golden_names(1)
    for k in (0, 5):
        plane = g["full_%d" % k]
        fails = compare(oracle_features(lib, plane, bits=16), g["full_%d_long" % k], names)
        assert not fails, (k, list(fails.items())[:3])
