"""Regenerates the golden fixtures under tests/golden/ (run in the container
that has the reference checkout; the GPU host never runs this).

Sources:
  * the reference's own fixtures (tests/wndchrm_tests/*.tif, *.sig, *.fit,
    *.weights and the expected table of test01-classify.pl), decoded here;
  * the unmodified reference library built by oracle/build_ref.sh
    (oracle/_ref/libwndref.so), run on those images and on small seeded
    synthetic images, for feature vectors, transform outputs and WND-5.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import ctypes
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "wnd-charm_gb300"))
from tiffread import read_tiff  # noqa: E402
from wndcharm import synth  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
T = os.path.join(REF, "tests", "wndchrm_tests")
LIB = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libwndref.so"))
D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)


def names(kind):
    buf = ctypes.create_string_buffer(512)
    out = []
    for i in range(LIB.wcref_plan_n_features(kind)):
        LIB.wcref_plan_feature_name(kind, i, buf, 512)
        out.append(buf.value.decode())
    return out


def ref_features(img, bits, kind):
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(LIB.wcref_plan_n_features(kind))
    LIB.wcref_extract_std(kind, pix.ctypes.data_as(D), img.shape[1], img.shape[0], bits, out.ctypes.data_as(D))
    return out


def ref_transform(name, img):
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(4 * pix.size + 4096)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    LIB.wcref_transform(name.encode(), pix.ctypes.data_as(D), img.shape[1], img.shape[0], 16,
                        out.ctypes.data_as(D), ctypes.byref(ow), ctypes.byref(oh))
    return out[: ow.value * oh.value].reshape(oh.value, ow.value)


def ref_wnd(xtr, ytr, xte, C, frac):
    N, F = xtr.shape
    Tn = xte.shape[0]
    w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
    p, pr = np.zeros((Tn, C)), np.zeros(Tn, dtype=np.int32)
    LIB.wcref_wnd(np.ascontiguousarray(xtr).ctypes.data_as(D), N, F,
                  np.ascontiguousarray(ytr, dtype=np.int32).ctypes.data_as(I), C, ctypes.c_double(frac),
                  np.ascontiguousarray(xte).ctypes.data_as(D), Tn, w.ctypes.data_as(D), mn.ctypes.data_as(D),
                  mx.ctypes.data_as(D), p.ctypes.data_as(D), pr.ctypes.data_as(I))
    return w, mn, mx, p, pr


def read_sig(path):
    lines = open(path).read().splitlines()[2:]
    return np.array([float(l.split("\t")[0]) for l in lines])


def read_fit(path):
    lines = open(path).read().splitlines()
    ncls, nf, ns = int(lines[0].split()[0]), int(lines[1]), int(lines[2])
    k = 3 + nf
    while not lines[k].strip():
        k += 1
    labels = lines[k:k + ncls]
    k += ncls
    rows, paths = [], []
    for s in range(ns):
        rows.append([float(v) for v in lines[k].split()])
        paths.append(lines[k + 1])
        k += 2
    a = np.array(rows)
    return a[:, :nf], a[:, nf].astype(np.int32), labels, paths


def main():
    with open(os.path.join(HERE, "names_long.txt"), "w") as fh:
        fh.write("\n".join(names(1)) + "\n")
    with open(os.path.join(HERE, "names_short.txt"), "w") as fh:
        fh.write("\n".join(names(0)) + "\n")

    # 1. the reference's golden TIFFs with their precalculated signatures
    imgs = {}
    for base in ["010067_301x300", "t1_s01_c05_ij"]:
        img, bits = read_tiff(os.path.join(T, base + ".tif"))
        imgs[base] = (img, bits, read_sig(os.path.join(T, base + "-l_precalculated.sig")))
    ufit, ucls, _, upaths = read_fit(os.path.join(T, "unbalanced.fit"))
    for keep in ["images/binuc/binuc1.tiff", "images/norm/norm1.tiff"]:
        i = upaths.index(keep)
        img, bits = read_tiff(os.path.join(T, keep))
        imgs[os.path.basename(keep).split(".")[0]] = (img, bits, ufit[i])
    arrays = {}
    for k, (img, bits, sig) in imgs.items():
        arrays["img_" + k] = img
        arrays["bits_" + k] = np.int32(bits)
        arrays["sig_" + k] = sig
        arrays["ref_" + k] = ref_features(img, bits, 1)
        print(k, img.shape, "ref done", flush=True)
    np.savez_compressed(os.path.join(HERE, "reference_images.npz"), **arrays)

    # 2. seeded synthetic images (uint16 12-bit, uneven sizes) through both plans
    rng = np.random.default_rng(20240)
    sizes = [(64, 64), (48, 37), (100, 71), (17, 23), (128, 96), (33, 90)]
    syn = {}
    for i, (w, h) in enumerate(sizes):
        img = synth.blob_image(rng, i % 3, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
        syn["img_%d" % i] = img
        syn["long_%d" % i] = ref_features(img, 16, 1)
        syn["short_%d" % i] = ref_features(img, 16, 0)
        print("synthetic", (w, h), flush=True)
    img8 = synth.blob_image(rng, 1, 96, 96).astype(np.uint8)
    syn["img_u8"] = img8
    syn["long_u8"] = ref_features(img8, 8, 1)
    syn["short_u8"] = ref_features(img8, 8, 0)
    np.savez_compressed(os.path.join(HERE, "reference_synthetic.npz"), **syn)

    # 3. single transforms on two small images
    tr = {}
    for i, (w, h) in enumerate([(40, 33), (64, 64)]):
        img = synth.blob_image(rng, 2, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
        tr["img_%d" % i] = img
        for name in ["Fourier", "Chebyshev", "Wavelet", "Edge"]:
            tr["%s_%d" % (name, i)] = ref_transform(name, img)
    np.savez_compressed(os.path.join(HERE, "reference_transforms.npz"), **tr)

    # 4. WND-5: test-l.fit (the CLI classify fixture), its Fisher weights, the
    #    expected classify table of test01-classify.pl, and a synthetic case.
    X, y, labels, paths = read_fit(os.path.join(T, "test-l.fit"))
    wts = np.array([float(l.split()[0]) for l in open(os.path.join(T, "test_fit-l.weights")).read().splitlines()])
    src = open(os.path.join(T, "test01-classify.pl")).read()
    block = re.search(r"<<END;\n(.*?)\nEND", src, re.S).group(1).splitlines()
    table = np.array([[float(t) for t in l.split("\t")[1:4]] for l in block])
    pred_cls = np.array([labels.index(l.split("\t")[4]) + 1 for l in block], dtype=np.int32)
    w, mn, mx, p, pr = ref_wnd(X, y, X, len(labels), 0.15)
    # inputs are regenerated from the seed by the tests: synth.feature_vectors(300, 40, 2919, 10, 4)
    xtr, ytr, xte, yte = synth.feature_vectors(300, 40, 2919, 10, 4)
    sw, smn, smx, sp, spr = ref_wnd(xtr, ytr, xte, 10, 0.15)
    np.savez_compressed(os.path.join(HERE, "reference_wnd.npz"),
                        fit_X=X, fit_y=y, weights_f1=wts, classify_table=table, classify_pred=pred_cls,
                        ref_w=w, ref_min=mn, ref_max=mx, ref_p=p, ref_pred=pr,
                        syn_w=sw, syn_min=smn, syn_max=smx,
                        syn_p=sp, syn_pred=spr)
    # the reference's signature and training-set files as text, for the .sig/.fit writers and readers
    texts = {}
    for key, fn in (("sig_010067", "010067_301x300-l_precalculated.sig"), ("sig_t1", "t1_s01_c05_ij-l_precalculated.sig"),
                    ("fit_unbalanced", "unbalanced.fit")):
        texts[key] = np.array(open(os.path.join(T, fn)).read())
    np.savez_compressed(os.path.join(HERE, "reference_text.npz"), **texts)
    # the reference's test TIFFs as bytes (uncompressed and LZW, big-endian), for the TIFF reader
    tifs = {}
    for key, fn in (("t1_s01_c05_ij", "t1_s01_c05_ij.tif"), ("010067_301x300", "010067_301x300.tif"),
                    ("binuc1", "images/binuc/binuc1.tiff"), ("norm1", "images/norm/norm1.tiff")):
        tifs[key] = np.frombuffer(open(os.path.join(T, fn), "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "reference_tiff.npz"), **tifs)
    print("done")


if __name__ == "__main__":
    main()
