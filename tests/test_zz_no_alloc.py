"""The allocation-free Wavelet entry point (wc_wavelet_noalloc), for callers
that may not allocate device memory (a fixed device-memory budget handed to
the library, a host that owns every allocation, a loop that must not meet the
synchronisation an allocation can bring).  It must give the same output as the
ordinary transform entry point (wc_transform "Wavelet") on calls in a row of
different sizes (odd, at the 1024 x 1024 limit, tall and thin, wide), so stale
scratch contents would show, and
reject inputs larger than its static scratch.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


def test_wavelet_noalloc_matches_wc_transform():
    import torch
    import wndcharm
    from wndcharm import synth
    L = wndcharm.lib()
    eng = wndcharm.Engine(0, "fp64")
    rng = np.random.default_rng(17)
    stream = torch.cuda.current_stream().cuda_stream
    # sizes in a row: ordinary, odd, at the scratch's 1024 x 1024 limit, tall and
    # thin (more output rows than one grid's y extent covers per pass), wide
    for (w, h) in [(64, 48), (37, 53), (1024, 1024), (3, 3000), (1023, 1025), (2100, 5)]:
        img = synth.blob_image(rng, 1, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.float64)
        exp = eng.transform("Wavelet", img)
        d_in = torch.from_numpy(np.ascontiguousarray(img)).cuda()
        d_out = torch.full(exp.shape, np.nan, dtype=torch.float64, device="cuda")
        rc = L.wc_wavelet_noalloc(ctypes.c_void_p(d_in.data_ptr()), w, h, ctypes.c_void_p(d_out.data_ptr()),
                                  ctypes.c_void_p(stream))
        assert rc == 0, L.wc_last_error()
        torch.cuda.synchronize()
        # same arithmetic as the Wavelet transform tests: exact agreement
        np.testing.assert_array_equal(d_out.cpu().numpy(), exp)


def test_wavelet_noalloc_rejects_oversize():
    import torch
    import wndcharm
    L = wndcharm.lib()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.wc_wavelet_noalloc(ctypes.c_void_p(d.data_ptr()), 2048, 2048, ctypes.c_void_p(d.data_ptr()), None)
    assert rc == -1
    assert b"static scratch" in L.wc_last_error()


def test_wavelet_noalloc_one_column_at_the_scratch_limit():
    """A 1 x 1,081,335 input fills the scratch exactly and needs 540,672
    output rows, more than one grid's y extent (65,535 x 8) covers: the rows
    are strided over the grid.  Checked against the oracle's Wavelet (the
    engine's transform entry point takes sides up to 32,768)."""
    import torch
    import wndcharm
    from conftest import oracle_lib
    L = wndcharm.lib()
    h = 1081335
    img = np.random.default_rng(3).uniform(0, 4095, size=(h, 1)).round()
    ow, oh = 2 * ((1 + 9) // 2), 2 * ((h + 9) // 2)  # the transform's output size
    out = np.zeros(ow * oh + 4096)
    cw, ch = ctypes.c_int(), ctypes.c_int()
    D = ctypes.POINTER(ctypes.c_double)
    assert oracle_lib().wco_transform(b"Wavelet", img.ctypes.data_as(D), 1, h, out.ctypes.data_as(D),
                                      ctypes.byref(cw), ctypes.byref(ch)) == 0
    assert (cw.value, ch.value) == (ow, oh)
    exp = out[:ow * oh].reshape(oh, ow)
    d_in = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    d_out = torch.full(exp.shape, np.nan, dtype=torch.float64, device="cuda")
    rc = L.wc_wavelet_noalloc(ctypes.c_void_p(d_in.data_ptr()), 1, h, ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == 0, L.wc_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy(), exp)
    rc = L.wc_wavelet_noalloc(ctypes.c_void_p(d_in.data_ptr()), 1, h + 2, ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == -1  # one row pair more than the scratch holds
