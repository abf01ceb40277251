"""The allocation-free Wavelet entry point (wc_wavelet_noalloc), for callers
that may not allocate device memory (a fixed device-memory budget handed to
the library, a host that owns every allocation, a loop that must not meet the
synchronisation an allocation can bring).  It must give the same output as the
ordinary transform entry point (wc_transform "Wavelet") on two calls in a row
(the second with a different size, so stale scratch contents would show), and
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
    for (w, h) in [(64, 48), (37, 53)]:
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
