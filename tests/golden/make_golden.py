"""Regenerates the golden fixtures under tests/golden/ (run in the container
that has the reference checkout; the GPU host never runs this).

Sources:
  * the reference's own fixtures (tests/wndchrm_tests/*.tif, *.sig, *.fit,
    *.weights and the expected table of test01-classify.pl), decoded here;
  * the unmodified reference library built by oracle/build_ref.sh
    (oracle/_ref/libwndref.so), run on those images and on small seeded
    synthetic images, for feature vectors, transform outputs and WND-5.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT] [--only preproc|wnd_images|colour]
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

ARGS = [a for i, a in enumerate(sys.argv[1:]) if not a.startswith("--") and sys.argv[i] != "--only"]
REF = ARGS[0] if ARGS else "/root/reference"
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


def ref_preprocess(img, bits, opt, sample, feat_kind=-1):
    """The reference's OpenImage preprocessing + AddImageFile sample cut (oracle/ref_shim/ref_capi.cpp)."""
    pix = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros(pix.size + 64)
    ow, oh = ctypes.c_int(), ctypes.c_int()
    feat = np.zeros(LIB.wcref_plan_n_features(max(feat_kind, 0)))
    o = np.ascontiguousarray(opt, dtype=np.float64)
    r = LIB.wcref_preprocess(pix.ctypes.data_as(D), img.shape[1], img.shape[0], bits, o.ctypes.data_as(D), sample,
                             out.ctypes.data_as(D), ctypes.c_long(out.size), ctypes.byref(ow), ctypes.byref(oh),
                             feat_kind, feat.ctypes.data_as(D))
    if r:
        return None, None
    plane = out[: ow.value * oh.value].reshape(oh.value, ow.value).copy()
    return plane, (feat if feat_kind >= 0 else None)


# opt: crop x, y, w, h; downsample x, y; normalize min, max, range, mean, std; rotations; tiles x, y
NONE_OPT = [-1, -1, -1, -1, 1, 1, -1, -1, -1, -1, -1, 1, 1, 1]


def _opt(**kw):
    o = list(NONE_OPT)
    keys = ["cx", "cy", "cw", "ch", "dsx", "dsy", "nmin", "nmax", "nrange", "nmean", "nstd", "rot", "tx", "ty"]
    for k, v in kw.items():
        o[keys.index(k)] = v
    return np.array(o, dtype=np.float64)


def preproc_fixtures():
    """Preprocessing and sampling (crop, Downsample, normalize, Rotate, tiles) by
    the reference, on a seeded 12-bit image, an 8-bit image and a crop of one of
    the reference's test images; features for a few samples."""
    rng = np.random.default_rng(31337)
    a = synth.blob_image(rng, 0, 61, 83, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
    b = synth.blob_image(rng, 1, 64, 48).astype(np.uint8)
    c = read_tiff(os.path.join(T, "t1_s01_c05_ij.tif"))[0]
    images = {"a": (a, 16), "b": (b, 8), "c": (c, 16)}
    cases = [
        ("crop", "a", _opt(cx=10, cy=7, cw=40, ch=70), []),
        ("ds50", "a", _opt(dsx=0.5, dsy=0.5), []),
        ("ds37", "a", _opt(dsx=0.37, dsy=0.37), []),
        ("ds_xy", "a", _opt(dsx=0.8, dsy=0.45), []),
        ("norm_ms", "a", _opt(nmean=1000, nstd=300), []),
        ("norm_m", "a", _opt(nmean=500, nstd=0), []),
        ("norm_mm", "a", _opt(nmin=200, nmax=3000, nrange=255), []),
        ("norm_both", "a", _opt(nmin=200, nmax=3000, nrange=4000, nmean=1500, nstd=200), []),
        ("rot4", "a", _opt(rot=4), []),
        ("tiles", "a", _opt(rot=4, tx=2, ty=3), []),
        ("u8", "b", _opt(dsx=0.6, dsy=0.6, nmean=100, nstd=30), []),
        ("full", "c", _opt(cx=5, cy=9, cw=96, ch=96, dsx=0.75, dsy=0.75, nmean=2000, nstd=500, rot=4, tx=2, ty=2),
         [0, 5]),
        ("crop_bad", "a", _opt(cx=30, cy=0, cw=40, ch=10), []),
    ]
    out = {"img_a": a, "img_b": b, "img_c": c}
    for name, im, opt, feats in cases:
        img, bits = images[im]
        out["opt_" + name] = opt
        out["src_" + name] = np.array(im)
        n = int(opt[11] * opt[12] * opt[13])
        ok = []
        for k in range(n):
            plane, f = ref_preprocess(img, bits, opt, k, 1 if k in feats else -1)
            ok.append(plane is not None)
            if plane is not None:
                out["%s_%d" % (name, k)] = plane
            if f is not None:
                out["%s_%d_long" % (name, k)] = f
        out["ok_" + name] = np.array(ok)
        print("preproc", name, sum(ok), "/", n, flush=True)
    np.savez_compressed(os.path.join(HERE, "reference_preproc.npz"), **out)


def wnd_image_fixtures():
    """TrainingSet::ClassifyImage (WND-5, tiles averaged, and the most-similar-tile
    rule) by the reference on seeded feature vectors: 12 test images of 4 tiles.
    Inputs are regenerated by the tests: synth.feature_vectors(200, 48, 2919, 6, 7)."""
    xtr, ytr, xte, yte = synth.feature_vectors(200, 48, 2919, 6, 7)
    out = {}
    for mt in (0, 1):
        probs = np.zeros((12, 6))
        pred = np.zeros(12, dtype=np.int32)
        LIB.wcref_wnd_images(np.ascontiguousarray(xtr).ctypes.data_as(D), 200, 2919,
                             np.ascontiguousarray(ytr, dtype=np.int32).ctypes.data_as(I), 6, ctypes.c_double(0.15),
                             np.ascontiguousarray(xte).ctypes.data_as(D), 12, 4, mt, probs.ctypes.data_as(D),
                             pred.ctypes.data_as(I))
        out["probs_max_tile%d" % mt] = probs
        out["pred_max_tile%d" % mt] = pred
        print("wnd images, max_tile", mt, pred, flush=True)
    np.savez_compressed(os.path.join(HERE, "reference_wnd_images.npz"), **out)


def colour_image(rng, w, h, bits):
    """Seeded synthetic RGB image: three blob images (different classes) as
    the channels; 8-bit, or 12-bit values in 16-bit samples."""
    ch = [synth.blob_image(rng, c, w, h, mean=60 + 40 * c, sd=30, scale=1 if bits == 8 else 16,
                           maxval=255 if bits == 8 else 4095) for c in range(3)]
    return np.ascontiguousarray(np.stack(ch, axis=-1).astype(np.uint8 if bits == 8 else np.uint16))


def colour_fixtures():
    """Colour images through the reference's LoadTIFF (gray + HSV planes) and
    its colour plans (with the terminator its fuzzy-colour loader omits,
    supplied by oracle/ref_shim/ref_capi.cpp); FindColor on random h, s, v."""
    rng = np.random.default_rng(4242)
    rgb8 = colour_image(rng, 64, 48, 8)
    rgb16 = colour_image(rng, 40, 56, 16)
    y, x = np.mgrid[0:256, 0:256]
    grid = np.ascontiguousarray(np.stack([x, y, (7 * x + 13 * y) % 256], axis=-1).astype(np.uint8))
    out = {"img_rgb8": rgb8, "img_rgb16": rgb16, "img_grid": grid}
    for key, img, bits in (("rgb8", rgb8, 8), ("rgb16", rgb16, 16)):
        h, w = img.shape[:2]
        gray, hsv = np.zeros(w * h), np.zeros(3 * w * h, dtype=np.uint8)
        LIB.wcref_load_rgb(img.ctypes.data, w, h, bits, gray.ctypes.data_as(D), hsv.ctypes.data)
        out["gray_" + key] = gray.reshape(h, w)
        out["hsv_" + key] = hsv.reshape(h, w, 3)
        for kind in (2, 3):
            f = np.zeros(LIB.wcref_plan_n_features(kind))
            LIB.wcref_extract_image(kind, img.ctypes.data, w, h, bits, 3, f.ctypes.data_as(D))
            out["plan%d_%s" % (kind, key)] = f
        print("colour", key, flush=True)
    f = np.zeros(LIB.wcref_plan_n_features(2))
    LIB.wcref_extract_image(2, grid.ctypes.data, 256, 256, 8, 3, f.ctypes.data_as(D))
    out["plan2_grid"] = f
    hsv = rng.integers(0, 256, size=(20000, 3)).astype(np.int32)
    out["fc_hsv"] = hsv
    out["fc_colour"] = np.array([LIB.wcref_find_colour(int(a), int(b), int(c)) for a, b, c in hsv], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "reference_colour.npz"), **out)
    for kind, fn in ((2, "names_color_short.txt"), (3, "names_color_long.txt")):
        with open(os.path.join(HERE, fn), "w") as fh:
            fh.write("\n".join(names(kind)) + "\n")


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
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "preproc":
        preproc_fixtures()
    elif only == "wnd_images":
        wnd_image_fixtures()
    elif only == "colour":
        colour_fixtures()
    else:
        main()
        preproc_fixtures()
        wnd_image_fixtures()
        colour_fixtures()
