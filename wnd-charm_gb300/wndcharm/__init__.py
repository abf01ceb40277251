"""GB300 (sm_103a) implementation of WND-CHARM's feature-extraction and WND-5
hot path, with the reference's Python/SWIG names for that path.

Reference interface mirrored (paths in the wnd-charm source tree):
  * StdFeatureComputationPlans.getFeatureSet / getFeatureSetLong   src/Tasks.h:355-377
  * FeatureComputationPlan(name).add(group_name), n_features,
    getFeatureNameByIndex(i)                                        src/Tasks.h:272-316
  * FeatureComputationPlanExecutor(plan).run(image, feature_vec, row)
                                                                    src/Tasks.h:318-348
  * ImageMatrix: a pixel plane with bits/width/height               src/cmatrix.h:164-339
  * WND-5 (CLI semantics): normalize, Fisher scores, classify2      src/wndchrm_src/TrainingSet.cpp

Every computation runs in the CUDA library (libwndcharm_gb300.so) through its
C ABI; importing works without a GPU, computing does not.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import WndcharmError, check, lib

__all__ = ["ImageMatrix", "FeatureComputationPlan", "StdFeatureComputationPlans", "FeatureComputationPlanExecutor",
           "Engine", "extract_batch", "wnd_fit", "wnd_classify", "WndcharmError"]


class FeatureComputationPlan(object):
    """A feature plan: feature groups in order, their columns and names."""

    def __init__(self, name="plan", _handle=None, _owned=False):
        self.name = name
        self._groups = []
        self._h = _handle
        self._owned = _owned

    @classmethod
    def _standard(cls, kind, name):
        h = ctypes.c_void_p()
        check(lib().wc_plan_get(kind, ctypes.byref(h)))
        return cls(name, h, False)

    def add(self, group_name):
        if self._h is not None:
            raise WndcharmError("plan is finalized")
        self._groups.append(group_name)

    def finalize(self):
        if self._h is None:
            arr = (ctypes.c_char_p * len(self._groups))(*[g.encode() for g in self._groups])
            h = ctypes.c_void_p()
            check(lib().wc_plan_from_names(arr, len(self._groups), ctypes.byref(h)))
            self._h, self._owned = h, True
        return self

    @property
    def handle(self):
        return self.finalize()._h

    @property
    def n_features(self):
        return check(lib().wc_plan_n_features(self.handle))

    def getFeatureNameByIndex(self, i):
        buf = ctypes.create_string_buffer(512)
        check(lib().wc_plan_feature_name(self.handle, int(i), buf, 512))
        return buf.value.decode()

    def feature_names(self):
        return [self.getFeatureNameByIndex(i) for i in range(self.n_features)]

    def groups(self):
        out = []
        buf = ctypes.create_string_buffer(512)
        off, nf = ctypes.c_int(), ctypes.c_int()
        for g in range(check(lib().wc_plan_n_groups(self.handle))):
            check(lib().wc_plan_group(self.handle, g, buf, 512, ctypes.byref(off), ctypes.byref(nf)))
            out.append((buf.value.decode(), off.value, nf.value))
        return out

    def __del__(self):
        try:
            if self._owned and self._h is not None:
                lib().wc_plan_free(self._h)
        except Exception:
            pass


class StdFeatureComputationPlans(object):
    @staticmethod
    def getFeatureSet():
        return FeatureComputationPlan._standard(_lib.WC_PLAN_SHORT, "Standard Feature Set")

    @staticmethod
    def getFeatureSetLong():
        return FeatureComputationPlan._standard(_lib.WC_PLAN_LONG, "Long Feature Set")


class ImageMatrix(object):
    """Grayscale pixel plane (row-major, height x width) with its bit depth."""

    def __init__(self, pixels=None, bits=16):
        self.pix_plane = None
        self.bits = bits
        if pixels is not None:
            self.set(pixels, bits)

    def set(self, pixels, bits=None):
        a = np.asarray(pixels)
        if a.ndim != 2:
            raise WndcharmError("ImageMatrix needs a 2-D array")
        self.pix_plane = a
        if bits is not None:
            self.bits = bits
        return self

    def OpenImage(self, path, downsample=0, bounding_rect=None, mean=0, stddev=0):
        """Read a grayscale 8/16-bit TIFF as ImageMatrix::OpenImage does
        (src/cmatrix.cpp:252-294): optional crop to bounding_rect = (x, y, w, h).
        Returns 1 on success, 0 when the file name has no ".tif"/".TIF" (as
        the reference); downsampling and mean/stddev normalisation are not
        supported here (WndcharmError)."""
        if ".tif" not in path and ".TIF" not in path:
            return 0
        if (downsample and 0 < downsample < 100) or mean > 0:
            raise WndcharmError("OpenImage: downsample / normalisation are not supported")
        pix, bits = read_tiff(path)
        if bounding_rect is not None and bounding_rect[0] >= 0:
            x, y, w, h = bounding_rect
            if x + w > pix.shape[1] or y + h > pix.shape[0]:
                raise WndcharmError("OpenImage: bounding_rect outside the image")
            pix = pix[y:y + h, x:x + w]
        self.set(np.ascontiguousarray(pix), bits)
        return 1

    @property
    def width(self):
        return self.pix_plane.shape[1]

    @property
    def height(self):
        return self.pix_plane.shape[0]


_DT = {np.dtype(np.uint8): _lib.WC_U8, np.dtype(np.uint16): _lib.WC_U16, np.dtype(np.float32): _lib.WC_F32,
       np.dtype(np.float64): _lib.WC_F64}


def _as_input(a):
    a = np.asarray(a)
    if a.dtype not in _DT:
        a = a.astype(np.float64)
    return np.ascontiguousarray(a)


class Engine(object):
    """One GPU with its device memory pools.  precision: 'fp64' or 'mixed'."""

    def __init__(self, device=0, precision="fp64"):
        p = {"fp64": _lib.WC_PREC_FP64, "mixed": _lib.WC_PREC_MIXED}[precision]
        h = ctypes.c_void_p()
        check(lib().wc_engine_create(int(device), p, ctypes.byref(h)))
        self._h = h
        self.precision = precision

    @property
    def launches(self):
        return lib().wc_engine_launch_count(self._h)

    def profile(self, on=True):
        check(lib().wc_engine_profile(self._h, 1 if on else 0))

    def profile_report(self):
        buf = ctypes.create_string_buffer(1 << 16)
        check(lib().wc_engine_profile_report(self._h, buf, 1 << 16))
        out = []
        for line in buf.value.decode().splitlines():
            f = line.split("\t")
            out.append((f[0], float(f[1]), int(f[2])))
        return out

    def profile_timeline(self):
        """Per stage: (name, start_ms, end_ms) after the profiled batch's first
        stage started (stages on different lanes overlap)."""
        buf = ctypes.create_string_buffer(1 << 16)
        check(lib().wc_engine_profile_report(self._h, buf, 1 << 16))
        out = []
        for line in buf.value.decode().splitlines():
            f = line.split("\t")
            out.append((f[0], float(f[3]), float(f[4])))
        return out

    def set_stream(self, stream_ptr):
        check(lib().wc_engine_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def extract(self, plan, images, bits=16, out=None):
        """Features of a list of 2-D arrays (any sizes): (n, n_features) float64."""
        imgs = [_as_input(a) for a in images]
        n = len(imgs)
        descs = (_lib.wc_image_desc * n)()
        for i, a in enumerate(imgs):
            descs[i] = _lib.wc_image_desc(a.ctypes.data, _DT[a.dtype], a.shape[1], a.shape[0], bits, 0)
        if out is None:
            out = np.zeros((n, plan.n_features))
        check(lib().wc_extract_batch(self._h, plan.handle, descs, n, out.ctypes.data, 0))
        return out

    def extract_device(self, plan, descs, n, out_dev_ptr):
        """Device-resident form: descs is a wc_image_desc array with on_device set;
        features land at out_dev_ptr (device); returns once queued."""
        check(lib().wc_extract_batch(self._h, plan.handle, descs, n, ctypes.c_void_p(out_dev_ptr), 1))

    def transform(self, name, pixels):
        a = np.ascontiguousarray(pixels, dtype=np.float64)
        cap = 4 * a.size + 8192
        out = np.zeros(cap)
        ow, oh = ctypes.c_int(), ctypes.c_int()
        check(lib().wc_transform(self._h, name.encode(), a.ctypes.data_as(_lib.D), a.shape[1], a.shape[0],
                                 out.ctypes.data_as(_lib.D), cap, ctypes.byref(ow), ctypes.byref(oh)))
        return out[: ow.value * oh.value].reshape(oh.value, ow.value).copy()

    def wnd_fit(self, train, labels, n_classes, frac=0.15):
        X = np.ascontiguousarray(train, dtype=np.float64)
        y = np.ascontiguousarray(labels, dtype=np.int32)
        N, F = X.shape
        w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
        check(lib().wc_wnd_fit(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I), int(n_classes),
                               float(frac), w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D),
                               mx.ctypes.data_as(_lib.D)))
        return w, mn, mx

    def wnd_classify(self, train, labels, n_classes, weights, mins, maxs, test):
        X = np.ascontiguousarray(train, dtype=np.float64)
        y = np.ascontiguousarray(labels, dtype=np.int32)
        T = np.ascontiguousarray(test, dtype=np.float64)
        N, F = X.shape
        nt = T.shape[0]
        w, mn, mx = (np.ascontiguousarray(v, dtype=np.float64) for v in (weights, mins, maxs))
        probs = np.zeros((nt, n_classes))
        pred = np.zeros(nt, dtype=np.int32)
        check(lib().wc_wnd_classify(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I), int(n_classes),
                                    w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D), mx.ctypes.data_as(_lib.D),
                                    T.ctypes.data_as(_lib.D), nt, probs.ctypes.data_as(_lib.D),
                                    pred.ctypes.data_as(_lib.I)))
        return probs, pred

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().wc_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def default_engine(precision="fp64"):
    if precision not in _default:
        _default[precision] = Engine(0, precision)
    return _default[precision]


class FeatureComputationPlanExecutor(object):
    """FeatureComputationPlanExecutor::run: features of one ImageMatrix written
    into feature_vec at row `dest_row` (feature_vec sized n_features * rows)."""

    def __init__(self, plan, engine=None):
        self.plan = plan
        self.engine = engine

    def run(self, image, feature_vec, dest_row=0):
        eng = self.engine or default_engine()
        if isinstance(image, ImageMatrix):
            pix, bits = image.pix_plane, image.bits
        else:
            pix, bits = np.asarray(image), 16
        row = eng.extract(self.plan, [pix], bits=bits)[0]
        n = self.plan.n_features
        feature_vec[n * dest_row: n * (dest_row + 1)] = row
        return feature_vec


def extract_batch(plan, images, precision="fp64", bits=16):
    return default_engine(precision).extract(plan, images, bits=bits)


def wnd_fit(train, labels, n_classes, frac=0.15, precision="fp64"):
    return default_engine(precision).wnd_fit(train, labels, n_classes, frac)


def wnd_classify(train, labels, n_classes, weights, mins, maxs, test, precision="fp64"):
    return default_engine(precision).wnd_classify(train, labels, n_classes, weights, mins, maxs, test)


def tiles(pixels, tiles_x, tiles_y):
    """The tiles wndchrm samples from an image (TrainingSet::AddImageFile,
    src/wndchrm_src/TrainingSet.cpp:1465-1476, enumerated x-major as in
    src/wndchrm_src/wndchrm.cpp:95-122): tile (ix, iy) covers columns
    [ix*tw, (ix+1)*tw) and rows [iy*th, (iy+1)*th), tw = W // tiles_x,
    th = H // tiles_y (the remainder at the right and bottom is dropped).
    Returns the list of 2-D views, ix outer, iy inner."""
    a = np.asarray(pixels)
    h, w = a.shape
    tw, th = w // tiles_x, h // tiles_y
    if tw < 1 or th < 1:
        raise WndcharmError("image %dx%d is smaller than %dx%d tiles" % (w, h, tiles_x, tiles_y))
    return [a[iy * th:(iy + 1) * th, ix * tw:(ix + 1) * tw] for ix in range(tiles_x) for iy in range(tiles_y)]


def read_tiff(path):
    """(pixels, bits) of a grayscale 8/16-bit TIFF (uint8 or uint16 array, height x
    width), read as ImageMatrix::LoadTIFF reads it."""
    L = lib()
    w, h, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    p = path.encode()
    check(L.wc_tiff_info(p, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b)))
    out = np.empty((h.value, w.value), dtype=np.uint8 if b.value == 8 else np.uint16)
    check(L.wc_tiff_read(p, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
    return out, b.value
