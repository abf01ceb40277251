import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
PKG = os.path.join(REPO, "wnd-charm_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_ORACLE = None


def oracle_lib():
    """The CPU oracle (test infrastructure), built with make on first use."""
    global _ORACLE
    if _ORACLE is None:
        so = os.path.join(REPO, "oracle", "build", "libwc_oracle.so")
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
        _ORACLE = ctypes.CDLL(so)
    return _ORACLE


@pytest.fixture(scope="session")
def oracle():
    return oracle_lib()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_names(kind):
    fn = {0: "names_short.txt", 1: "names_long.txt", 2: "names_color_short.txt", 3: "names_color_long.txt"}[kind]
    return open(os.path.join(GOLDEN, fn)).read().splitlines()


def oracle_features_rgb(lib, img, bits, kind):
    """The oracle's plan `kind` on an RGB image ((h, w, 3) uint8 / uint16)."""
    a = np.ascontiguousarray(img)
    out = np.zeros(lib.wco_plan_n_features(kind))
    lib.wco_extract_rgb(kind, ctypes.c_void_p(a.ctypes.data), a.shape[1], a.shape[0], bits, out.ctypes.data_as(D))
    return out


def oracle_features(lib, img, bits=16, kind=1):
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(lib.wco_plan_n_features(kind))
    lib.wco_extract_std(kind, pix.ctypes.data_as(D), img.shape[1], img.shape[0], bits, out.ctypes.data_as(D))
    return out


def oracle_wnd(lib, xtr, ytr, xte, C, frac):
    N, F = xtr.shape
    T = xte.shape[0]
    w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
    p, pr = np.zeros((T, C)), np.zeros(T, dtype=np.int32)
    lib.wco_wnd(np.ascontiguousarray(xtr, dtype=np.float64).ctypes.data_as(D), N, F,
                np.ascontiguousarray(ytr, dtype=np.int32).ctypes.data_as(I), C, ctypes.c_double(frac),
                np.ascontiguousarray(xte, dtype=np.float64).ctypes.data_as(D), T, w.ctypes.data_as(D),
                mn.ctypes.data_as(D), mx.ctypes.data_as(D), p.ctypes.data_as(D), pr.ctypes.data_as(I))
    return w, mn, mx, p, pr
