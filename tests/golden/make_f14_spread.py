"""Measures the reference's own build-to-build spread on the long plan and
writes tests/golden/reference_build_spread.npz (run in the container that has
the reference checkout; the GPU host never runs this).

Two builds of the UNMODIFIED reference library (oracle/build_ref.sh):
  * oracle/_ref      : g++ -O2, no fused multiply-add (the default x86-64 build);
  * oracle/_ref_fma  : the same sources with contraction into fused
                       multiply-adds (VARIANT=fma), as a contracting compiler
                       (or the aarch64 default) builds them.
Both run the long plan (2919 features) on the first N images of the 512 x 512
benchmark workload (4 classes, seed 1, classes interleaved), one process per
image.  The oracle (oracle/build/libwc_oracle.so) runs on the same images.

The fixture keeps, per image: the default build's 2919 features, the 24
Haralick f14 entries (in-group [16], [17]
of the 12 Haralick groups) of both builds and of the oracle, and, for every
feature, the absolute difference between the two builds.  The tests gate the
GPU's f14 on the entries the two builds agree on and read the spread of the
binned families from it.

Usage: python tests/golden/make_f14_spread.py [N_IMAGES]   (default 16)
"""
import ctypes
import hashlib
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "wnd-charm_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

LIBS = {"ref": os.path.join(REPO, "oracle", "_ref", "libwndref.so"),
        "ref_fma": os.path.join(REPO, "oracle", "_ref_fma", "libwndref.so"),
        "oracle": os.path.join(REPO, "oracle", "build", "libwc_oracle.so")}
D = ctypes.POINTER(ctypes.c_double)


def workload(n):
    """The benchmark's images: config-2 generator, seed 1, classes interleaved."""
    from wndcharm import synth
    per = (n + 3) // 4
    imgs, _ = synth.config2(n_per_class=per, size=512, seed=1)
    order = [c * per + i for i in range(per) for c in range(4)][:n]
    return [imgs[k] for k in order]


def _run(job):
    which, img = job
    lib = ctypes.CDLL(LIBS[which])
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(2919)
    fn = lib.wco_extract_std if which == "oracle" else lib.wcref_extract_std
    fn(1, pix.ctypes.data_as(D), img.shape[1], img.shape[0], 16, out.ctypes.data_as(D))
    return out


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    for k, p in LIBS.items():
        if not os.path.exists(p):
            raise SystemExit("missing %s (oracle/build_ref.sh, VARIANT=fma oracle/build_ref.sh, make -C oracle)" % p)
    imgs = workload(n)
    jobs = [(w, im) for w in ("ref", "ref_fma", "oracle") for im in imgs]
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        rows = pool.map(_run, jobs, chunksize=1)
    ref, fma, ora = (np.array(rows[i * n:(i + 1) * n]) for i in range(3))
    from parity import F14, group_of, index_of
    names = open(os.path.join(HERE, "names_long.txt")).read().splitlines()
    f14i = np.array([i for i, nm in enumerate(names) if group_of(nm).startswith("Haralick") and index_of(nm) in F14])
    np.savez_compressed(os.path.join(HERE, "reference_build_spread.npz"), f14_index=f14i, f14_ref=ref[:, f14i],
                        f14_ref_fma=fma[:, f14i], f14_oracle=ora[:, f14i], build_absdiff=np.abs(ref - fma),
                        oracle_absdiff=np.abs(ora - ref), ref_rows=ref, n_images=n,
                        img_sha256=np.array([hashlib.sha256(np.ascontiguousarray(im).tobytes()).hexdigest()
                                             for im in imgs]))
    a, b = ref[:, f14i], fma[:, f14i]
    agree = np.abs(a - b) <= 1e-6 * np.maximum(np.abs(a), 1e-12)
    print("f14: the two reference builds agree within 1e-6 on %d of %d entries; max |diff| %.3g"
          % (agree.sum(), agree.size, np.nanmax(np.abs(a - b))))
    o = ora[:, f14i]
    agree_o = np.abs(o - a) <= 1e-6 * np.maximum(np.abs(a), 1e-12)
    print("f14: the oracle agrees with the default build on %d of %d entries" % (agree_o.sum(), agree_o.size))


if __name__ == "__main__":
    main()
