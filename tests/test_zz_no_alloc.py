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


RESET_PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include "wndcharm_gb300.h"
// wc_wavelet_noalloc before and after cudaDeviceReset (a new primary context:
// the library's device code is loaded again and its static scratch may move)
static int run(const std::vector<double> &in, int w, int h, std::vector<double> &out) {
    double *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, in.size() * 8) != cudaSuccess || cudaMalloc(&dout, out.size() * 8) != cudaSuccess) return 1;
    cudaMemcpy(din, in.data(), in.size() * 8, cudaMemcpyHostToDevice);
    if (wc_wavelet_noalloc(din, w, h, dout, nullptr) != 0) { printf("rc: %s\n", wc_last_error()); return 2; }
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    cudaMemcpy(out.data(), dout, out.size() * 8, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    return 0;
}
int main() {
    const int w = 64, h = 48, ow = 2 * ((w + 9) / 2), oh = 2 * ((h + 9) / 2);
    std::vector<double> in((size_t)w * h), a((size_t)ow * oh), b((size_t)ow * oh, -1.0);
    for (int i = 0; i < w * h; i++) in[i] = (i * 37) % 4096;
    int rc = run(in, w, h, a);
    if (rc) return rc;
    if (cudaDeviceReset() != cudaSuccess) return 4;
    rc = run(in, w, h, b);
    if (rc) return 10 + rc;
    if (memcmp(a.data(), b.data(), a.size() * 8) != 0) { printf("differ\n"); return 20; }
    printf("same after reset\n");
    return 0;
}
"""


def test_wavelet_noalloc_after_device_reset(tmp_path):
    """A process calls the entry point, resets the device (cudaDeviceReset:
    the primary context and the library's loaded device code are recreated,
    so the static scratch's address may change), and calls it again: the
    scratch is looked up on every call, and the output is the same."""
    import os
    import shutil
    import subprocess
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = os.path.join(repo, "wnd-charm_gb300", "build")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "reset.cu"
    src.write_text(RESET_PROGRAM)
    exe = tmp_path / "reset"
    b = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-I" + os.path.join(repo, "include"),
                        str(src), "-o", str(exe), "-L" + lib, "-lwndcharm_gb300", "-Xlinker", "-rpath=" + lib],
                       capture_output=True, text=True, timeout=600)
    assert b.returncode == 0, b.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "same after reset" in r.stdout, (r.returncode, r.stdout, r.stderr)
