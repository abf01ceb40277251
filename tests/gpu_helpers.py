"""Helpers for the GPU parity tests: engine, oracle calls, seeded images."""
import ctypes

import numpy as np

from conftest import D, oracle_lib
import synth_loader  # noqa: F401
from wndcharm import synth

CHAINS = ["()", "(Fourier ())", "(Wavelet ())", "(Chebyshev ())", "(Edge ())", "(Chebyshev (Fourier ()))",
          "(Wavelet (Fourier ()))", "(Fourier (Wavelet ()))", "(Fourier (Chebyshev ()))", "(Chebyshev (Wavelet ()))",
          "(Fourier (Edge ()))", "(Wavelet (Edge ()))"]
SIZES = [(64, 64), (48, 37), (17, 23), (100, 71)]


def images(seed=11, sizes=SIZES, bits=16):
    rng = np.random.default_rng(seed)
    out = []
    for i, (w, h) in enumerate(sizes):
        if bits == 16:
            out.append(synth.blob_image(rng, i % 3, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16))
        else:
            out.append(synth.blob_image(rng, i % 3, w, h).astype(np.uint8))
    return out


def oracle_group(group, img):
    lib = oracle_lib()
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(256)
    n = lib.wco_extract_group(group.encode(), pix.ctypes.data_as(D), img.shape[1], img.shape[0], 16,
                              out.ctypes.data_as(D))
    assert n > 0, group
    return out[:n]


def oracle_transform(name, img):
    lib = oracle_lib()
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(4 * pix.size + 4096)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    assert lib.wco_transform(name.encode(), pix.ctypes.data_as(D), img.shape[1], img.shape[0],
                             out.ctypes.data_as(D), ctypes.byref(ow), ctypes.byref(oh)) == 0
    return out[: ow.value * oh.value].reshape(oh.value, ow.value)
