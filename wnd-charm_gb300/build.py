"""Builds the CUDA library libwndcharm_gb300.so (C ABI of include/wndcharm_gb300.h)
in-tree under wnd-charm_gb300/build/, for sm_103a only.

    python wnd-charm_gb300/build.py [--force]

Translation units compile in parallel; only changed ones are rebuilt.
"""
import concurrent.futures
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "build")
LIB = os.path.join(OUT, "libwndcharm_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# files whose arithmetic restates a CPU order of operations bit for bit: no
# multiply-add contraction anywhere in them
EXTRA = {"k_haralick.cu": ["-fmad=false"], "k_groupa.cu": ["-fmad=false"], "k_fft.cu": ["-fmad=false"],
         "k_pre.cu": ["-fmad=false"], "k_color.cu": ["-fmad=false"]}
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + CSRC, "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _deps_newer(src, obj):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    heads = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(os.path.dirname(HERE), "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in [src] + heads)


def _compile(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not force and not _deps_newer(src, obj):
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + EXTRA.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, p.stdout + p.stderr
    return obj, None


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        res = list(ex.map(lambda s: _compile(s, force), srcs))
    errs = [e for _, e in res if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in res]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
