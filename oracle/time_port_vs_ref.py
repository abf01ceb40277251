"""Times the oracle port (oracle/build/libwc_oracle.so) against the reference
library built from the reference's own sources (oracle/_ref/libwndref.so) on
the same synthetic 512 x 512 12-bit images, one image at a time on one core,
long plan: the ratio says how well the port's time stands for the reference's
when the port is timed as the CPU baseline.  Run where oracle/build_ref.sh has
built oracle/_ref:  python oracle/time_port_vs_ref.py [n_images]"""
import ctypes
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "wnd-charm_gb300"))
from wndcharm import synth  # noqa: E402

D = ctypes.POINTER(ctypes.c_double)


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 3
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    ora = ctypes.CDLL(os.path.join(REPO, "oracle", "build", "libwc_oracle.so"))
    ref = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libwndref.so"))
    imgs, _ = synth.config2(n_per_class=1, size=512, seed=1)
    imgs = imgs[:n]
    tp, tr, worst = [], [], 0.0
    for img in imgs:
        pix = np.ascontiguousarray(img, dtype=np.float64)
        a = np.zeros(2919)
        b = np.zeros(2919)
        offs = np.zeros(1, dtype=np.int64)
        w = np.array([512], dtype=np.int32)
        h = np.array([512], dtype=np.int32)
        t0 = time.perf_counter()
        ora.wco_extract_std_batch(1, pix.ctypes.data_as(D), offs.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                  w.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                  h.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 1, 16, a.ctypes.data_as(D), 1)
        tp.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        ref.wcref_extract_std(1, pix.ctypes.data_as(D), 512, 512, 16, b.ctypes.data_as(D))
        tr.append(time.perf_counter() - t0)
        ok = np.isfinite(a) & np.isfinite(b)
        worst = max(worst, float(np.median(np.abs(a[ok] - b[ok]) / (np.abs(b[ok]) + 1e-9))))
    print("images: %d of 512x512, long plan, one core each" % n)
    print("oracle port    : %.2f s/image (%s)" % (np.mean(tp), " ".join("%.2f" % t for t in tp)))
    print("reference build: %.2f s/image (%s)" % (np.mean(tr), " ".join("%.2f" % t for t in tr)))
    print("port / reference time: %.3f" % (np.mean(tp) / np.mean(tr)))
    print("median relative feature difference (worst image): %.2g" % worst)


if __name__ == "__main__":
    main()
