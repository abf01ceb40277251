"""GB300 (sm_103a) implementation of WND-CHARM's feature-extraction and WND-5
hot path, with the reference's Python/SWIG names for that path.

Reference interface mirrored (paths in the wnd-charm source tree):
  * StdFeatureComputationPlans.getFeatureSet / getFeatureSetLong   src/Tasks.h:355-377
  * FeatureComputationPlan(name).add(group_name), n_features,
    getFeatureNameByIndex(i)                                        src/Tasks.h:272-316
  * FeatureComputationPlanExecutor(plan).run(image, feature_vec, row)
                                                                    src/Tasks.h:318-348
  * ImageMatrix: a pixel plane with bits/width/height, OpenImage, submatrix,
    Downsample, normalize, Rotate                                   src/cmatrix.h:164-339, src/cmatrix.cpp:252-888
  * the samples of one image (rotations x tiles, with OpenImage's
    preprocessing) as TrainingSet::AddImageFile cuts them           src/wndchrm_src/TrainingSet.cpp:1442-1481
  * WND-5 (CLI semantics): normalize, Fisher scores, classify2      src/wndchrm_src/TrainingSet.cpp

Every computation runs in the CUDA library (libwndcharm_gb300.so) through its
C ABI; importing works without a GPU, computing does not.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import WndcharmError, check, lib

__all__ = ["ImageMatrix", "FeatureComputationPlan", "StdFeatureComputationPlans", "FeatureComputationPlanExecutor",
           "Engine", "Sampling", "extract_batch", "extract_samples", "wnd_fit", "wnd_classify", "WndcharmError"]


class Sampling(object):
    """Preprocessing and sampling options of wndchrm (its preproc_opts and
    sampling_opts, src/wndchrm_src/wndchrm.cpp:750-770, 846-900):
    bounding_rect (x, y, w, h) crops; downsample is a percentage (applied when
    0 < downsample < 100, as ImageMatrix::OpenImage does); mean > 0 normalises
    to that mean (and to stddev when > 0); rotations 1 or 4 (the -R switch);
    tiles_x x tiles_y tiles per rotated image (-t).  ratio_x / ratio_y (explicit
    Downsample ratios) and norm_min / norm_max / norm_range (normalize's range
    branch) give the ImageMatrix methods' general forms."""

    def __init__(self, bounding_rect=None, downsample=0, mean=0, stddev=0, rotations=1, tiles_x=1, tiles_y=1,
                 ratio_x=None, ratio_y=None, norm_min=-1, norm_max=-1, norm_range=-1):
        self.bounding_rect = bounding_rect
        self.downsample = downsample
        self.mean, self.stddev = mean, stddev
        self.rotations, self.tiles_x, self.tiles_y = rotations, tiles_x, tiles_y
        self.ratio_x, self.ratio_y = ratio_x, ratio_y
        self.norm_min, self.norm_max, self.norm_range = norm_min, norm_max, norm_range

    def struct(self):
        s = _lib.wc_sampling()
        lib().wc_sampling_default(ctypes.byref(s))
        if self.bounding_rect is not None and self.bounding_rect[0] >= 0:
            s.crop_x, s.crop_y, s.crop_w, s.crop_h = (int(v) for v in self.bounding_rect)
        if self.ratio_x is not None or self.ratio_y is not None:
            s.downsample_x = 1.0 if self.ratio_x is None else float(self.ratio_x)
            s.downsample_y = 1.0 if self.ratio_y is None else float(self.ratio_y)
        elif self.downsample and 0 < self.downsample < 100:
            s.downsample_x = s.downsample_y = float(self.downsample) / 100.0
        if self.mean > 0:
            s.norm_mean, s.norm_std = float(self.mean), float(self.stddev)
        s.norm_min, s.norm_max, s.norm_range = float(self.norm_min), float(self.norm_max), int(self.norm_range)
        s.rotations, s.tiles_x, s.tiles_y = int(self.rotations), int(self.tiles_x), int(self.tiles_y)
        return s

    @property
    def count(self):
        """Samples per image."""
        return check(lib().wc_sampling_count(ctypes.byref(self.struct())))

    def sample_size(self, width, height, sample=0):
        w, h = ctypes.c_int(), ctypes.c_int()
        check(lib().wc_sample_size(ctypes.byref(self.struct()), int(width), int(height), int(sample),
                                   ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value


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

    @staticmethod
    def getFeatureSetColor():
        """2199 features: the short set plus the colour features (RGB images)."""
        return FeatureComputationPlan._standard(_lib.WC_PLAN_SHORT_COLOR, "Color Feature Set")

    @staticmethod
    def getFeatureSetLongColor():
        """4059 features: the long set with the colour features (RGB images)."""
        return FeatureComputationPlan._standard(_lib.WC_PLAN_LONG_COLOR, "Long Color Feature Set")


class ImageMatrix(object):
    """Grayscale pixel plane (row-major, height x width) with its bit depth."""

    def __init__(self, pixels=None, bits=16):
        self.pix_plane = None
        self.bits = bits
        if pixels is not None:
            self.set(pixels, bits)

    def set(self, pixels, bits=None):
        a = np.asarray(pixels)
        if not (a.ndim == 2 or (a.ndim == 3 and a.shape[2] == 3)):
            raise WndcharmError("ImageMatrix needs a 2-D (grayscale) or (height, width, 3) RGB array")
        self.pix_plane = a
        if bits is not None:
            self.bits = bits
        return self

    def OpenImage(self, path, downsample=0, bounding_rect=None, mean=0, stddev=0, engine=None):
        """Read an 8/16-bit grayscale or RGB TIFF as ImageMatrix::OpenImage does
        (src/cmatrix.cpp:252-294): crop to bounding_rect = (x, y, w, h), area
        downsampling to `downsample` percent (0 < downsample < 100), and
        normalisation to `mean` (> 0) and `stddev`, on the GPU (grayscale
        only).  The pixel plane is the file's integers ((height, width, 3)
        for RGB) when nothing is applied, else float64.
        Returns 1 on success, 0 when the file name has no ".tif"/".TIF" (as
        the reference); a rectangle outside the image raises WndcharmError."""
        if ".tif" not in path and ".TIF" not in path:
            return 0
        pix, bits = read_tiff(path)
        opts = Sampling(bounding_rect=bounding_rect, downsample=downsample, mean=mean, stddev=stddev)
        st = opts.struct()
        if st.downsample_x < 1 or st.downsample_y < 1 or st.norm_mean > 0:
            pix = (engine or default_engine()).preprocess(pix, opts, 0, bits)
        elif st.crop_x >= 0:  # a crop alone copies pixels: the file's integers, no GPU needed
            opts.sample_size(pix.shape[1], pix.shape[0])  # refuses a rectangle outside the image
            pix = pix[st.crop_y:st.crop_y + st.crop_h, st.crop_x:st.crop_x + st.crop_w]
        self.set(np.ascontiguousarray(pix), bits)
        return 1

    def _apply(self, matrix_IN, opts, sample=0, engine=None):
        src = matrix_IN if matrix_IN is not None else self
        pix = (engine or default_engine()).preprocess(src.pix_plane, opts, sample, src.bits)
        self.set(pix, src.bits)

    def submatrix(self, matrix_IN, x1, y1, x2, y2, engine=None):
        """ImageMatrix::submatrix (src/cmatrix.cpp:414-470): rows y1..y2 and
        columns x1..x2 of matrix_IN; returns 0 (self unchanged) when x2 or y2 is
        outside it, else 1."""
        if x2 >= matrix_IN.width or y2 >= matrix_IN.height or x2 < x1 or y2 < y1 or x1 < 0 or y1 < 0:
            return 0
        self._apply(matrix_IN, Sampling(bounding_rect=(x1, y1, x2 - x1 + 1, y2 - y1 + 1)), 0, engine)
        return 1

    def Downsample(self, matrix_IN, x_ratio, y_ratio, engine=None):
        """ImageMatrix::Downsample (src/cmatrix.cpp:579-720): area averaging to
        (unsigned)(ratio * size) along each axis; ratios above 1 count as 1."""
        self._apply(matrix_IN, Sampling(ratio_x=x_ratio, ratio_y=y_ratio), 0, engine)

    def normalize(self, n_min, n_max, n_range, n_mean, n_std, engine=None):
        """ImageMatrix::normalize (src/cmatrix.cpp:836-888) in place: to [0,
        n_range] between n_min and n_max (when all three are set), then to
        n_mean / n_std (when n_mean > 0), clamped to [0, 2^bits - 1]."""
        self._apply(None, Sampling(norm_min=n_min, norm_max=n_max, norm_range=n_range, mean=n_mean, stddev=n_std),
                    0, engine)

    def Rotate(self, matrix_IN, angle, engine=None):
        """ImageMatrix::Rotate (src/cmatrix.cpp:727-769): 90 (transpose, rows
        reversed), 180, or 270 (the transpose, as in the reference); other
        angles leave self unchanged."""
        if angle not in (90, 180, 270):
            return
        self._apply(matrix_IN, Sampling(rotations=4), int(angle) // 90, engine)

    @property
    def width(self):
        return self.pix_plane.shape[1]

    @property
    def height(self):
        return self.pix_plane.shape[0]


_DT = {np.dtype(np.uint8): _lib.WC_U8, np.dtype(np.uint16): _lib.WC_U16, np.dtype(np.float32): _lib.WC_F32,
       np.dtype(np.float64): _lib.WC_F64}


_RGB = {np.dtype(np.uint8): _lib.WC_RGB8, np.dtype(np.uint16): _lib.WC_RGB16}


def _as_input(a):
    """A 2-D grayscale array, or an RGB array (height, width, 3) of uint8 / uint16."""
    a = np.asarray(a)
    if a.ndim == 3:
        if a.shape[2] != 3 or a.dtype not in _RGB:
            raise WndcharmError("an RGB image is a (height, width, 3) uint8 or uint16 array")
        return np.ascontiguousarray(a)
    if a.dtype not in _DT:
        a = a.astype(np.float64)
    return np.ascontiguousarray(a)


def _dtype_code(a):
    return _RGB[a.dtype] if a.ndim == 3 else _DT[a.dtype]


def _out_buffer(out, rows, cols):
    """The caller's output array, checked (a writable, C-contiguous float64
    array of shape (rows, cols): the library writes rows * cols doubles
    there), or a new zeroed one."""
    if out is None:
        return np.zeros((rows, cols))
    if (not isinstance(out, np.ndarray) or out.dtype != np.float64 or not out.flags.c_contiguous
            or not out.flags.writeable or out.shape != (rows, cols)):
        raise WndcharmError("out must be a writable C-contiguous float64 array of shape (%d, %d)" % (rows, cols))
    return out


def _wnd_rows(train, labels, test=None):
    """Training rows (N, F) float64, their N labels (int32) and test rows
    (T, F) float64 (a single row may be 1-D), checked against each other: the
    library reads N x F, N and T x F values through these pointers.  Arrays
    that already have the layout are passed on as they are (no copy)."""
    X = np.ascontiguousarray(train, dtype=np.float64)
    y = np.ascontiguousarray(labels, dtype=np.int32)
    if X.ndim != 2 or y.shape != (X.shape[0],):
        raise WndcharmError("training rows must be an (N, F) array with N labels")
    if test is None:
        return X, y
    T = np.ascontiguousarray(np.atleast_2d(test), dtype=np.float64)
    if T.ndim != 2 or T.shape[1] != X.shape[1]:
        raise WndcharmError("test rows must have the training rows' %d features" % X.shape[1])
    return X, y, T


def _wnd_vecs(F, *vecs):
    """Per-feature vectors (weights, mins, maxs, means), F float64 values each."""
    out = []
    for v in vecs:
        a = np.ascontiguousarray(v, dtype=np.float64)
        if a.shape != (F,):
            raise WndcharmError("per-feature vectors must hold %d values" % F)
        out.append(a)
    return out


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

    def profile(self, on=True, serial=False):
        """Per-stage timing on (serial: the lanes run one after another, so each
        stage's time is its own rather than its share of a concurrent step)."""
        check(lib().wc_engine_profile(self._h, (2 if serial else 1) if on else 0))

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

    def tuning(self):
        """The launch-shape tuner's state: {key: (chosen candidate, [ms per candidate])}."""
        buf = ctypes.create_string_buffer(1 << 16)
        check(lib().wc_engine_tuning_report(self._h, buf, 1 << 16))
        out = {}
        for line in buf.value.decode().splitlines():
            f = line.split("\t")
            out[f[0]] = (int(f[1]), [float(x) for x in f[2:]])
        return out

    def graph_stats(self):
        """CUDA-graph use (option 'graph'): {'captures', 'replays', 'failures', 'kept'}."""
        st = (ctypes.c_longlong * 4)()
        check(lib().wc_engine_graph_stats(self._h, st))
        return dict(zip(("captures", "replays", "failures", "kept"), list(st)))

    def set_option(self, name, value):
        """Engine option (wc_engine_set_option): 'f14_exact' (mixed form: f14
        through the FP64 chain, 1 by default), 'qr_iter_per_tone' (real-Schur
        iterations allowed per tone, 40), 'union_find_cap' (labelling
        iterations allowed per link, 0 = the pixel count), 'autotune' (1),
        'graph' (0; 1: repeated batch shapes replay a captured CUDA graph),
        'cf_tensor_cores' (1: the mixed form's Chebyshev-Fourier sums on the
        tensor cores where a batch's planes share one size)."""
        check(lib().wc_engine_set_option(self._h, name.encode(), int(value)))

    def extract(self, plan, images, bits=16, out=None):
        """Features of a list of 2-D arrays (any sizes): (n, n_features) float64."""
        imgs = [_as_input(a) for a in images]
        n = len(imgs)
        descs = (_lib.wc_image_desc * n)()
        for i, a in enumerate(imgs):
            descs[i] = _lib.wc_image_desc(a.ctypes.data, _dtype_code(a), a.shape[1], a.shape[0], bits, 0)
        out = _out_buffer(out, n, plan.n_features)
        check(lib().wc_extract_batch(self._h, plan.handle, descs, n, out.ctypes.data, 0))
        return out

    def preprocess(self, pixels, sampling, sample=0, bits=16):
        """One sample plane (float64) of a 2-D array: sampling's crop,
        downsampling and normalisation, then sample `sample`'s rotation and
        tile (rotation outermost, tile x, tile y innermost)."""
        a = _as_input(pixels)
        st = sampling.struct()
        w, h = ctypes.c_int(), ctypes.c_int()
        check(lib().wc_sample_size(ctypes.byref(st), a.shape[1], a.shape[0], int(sample), ctypes.byref(w),
                                   ctypes.byref(h)))
        out = np.zeros((h.value, w.value))
        d = _lib.wc_image_desc(a.ctypes.data, _dtype_code(a), a.shape[1], a.shape[0], int(bits), 0)
        check(lib().wc_preprocess(self._h, ctypes.byref(d), ctypes.byref(st), int(sample), out.ctypes.data, out.size,
                                  ctypes.byref(w), ctypes.byref(h), 0))
        return out

    def extract_samples(self, plan, images, sampling, bits=16, out=None):
        """Features of every sample of every image ((n * sampling.count,
        n_features), image-major), preprocessing and sampling on the GPU."""
        imgs = [_as_input(a) for a in images]
        n = len(imgs)
        descs = (_lib.wc_image_desc * n)()
        for i, a in enumerate(imgs):
            descs[i] = _lib.wc_image_desc(a.ctypes.data, _dtype_code(a), a.shape[1], a.shape[0], bits, 0)
        st = sampling.struct()
        per = check(lib().wc_sampling_count(ctypes.byref(st)))
        out = _out_buffer(out, n * per, plan.n_features)
        check(lib().wc_extract_samples(self._h, plan.handle, descs, n, ctypes.byref(st), out.ctypes.data, 0))
        return out

    def read_tiffs_device(self, paths):
        """TIFF files decoded into device memory (wc_tiff_read_device): returns
        (buffer, descs) -- a torch uint8 CUDA tensor holding every image's
        samples and a wc_image_desc array (on_device) for extract_device /
        extract_samples_device.  Keep the buffer alive while descs are used."""
        import torch
        arr = (ctypes.c_char_p * len(paths))(*[os.fsencode(p) for p in paths])
        nb = ctypes.c_longlong()
        check(lib().wc_tiff_device_bytes(arr, len(paths), ctypes.byref(nb)))
        buf = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device="cuda")
        descs = (_lib.wc_image_desc * len(paths))()
        check(lib().wc_tiff_read_device(self._h, arr, len(paths), ctypes.c_void_p(buf.data_ptr()), buf.numel(),
                                        descs))
        return buf, descs

    def extract_tiffs(self, plan, paths, sampling=None):
        """Feature rows of TIFF files decoded on the GPU: with a Sampling, every
        sample of every file (wc_extract_samples, image-major), else one row per
        file (wc_extract_batch).  Host rows out."""
        buf, descs = self.read_tiffs_device(paths)
        n = len(paths)
        if sampling is None:
            out = np.zeros((n, plan.n_features))
            check(lib().wc_extract_batch(self._h, plan.handle, descs, n, out.ctypes.data, 0))
        else:
            st = sampling.struct()
            per = check(lib().wc_sampling_count(ctypes.byref(st)))
            out = np.zeros((n * per, plan.n_features))
            check(lib().wc_extract_samples(self._h, plan.handle, descs, n, ctypes.byref(st), out.ctypes.data, 0))
        del buf
        return out

    def extract_device(self, plan, descs, n, out_dev_ptr):
        """Device-resident form: descs is a wc_image_desc array with on_device set;
        features land at out_dev_ptr (device); returns when they are written."""
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
        X, y = _wnd_rows(train, labels)
        N, F = X.shape
        w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
        check(lib().wc_wnd_fit(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I), int(n_classes),
                               float(frac), w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D),
                               mx.ctypes.data_as(_lib.D)))
        return w, mn, mx

    def wnd_classify(self, train, labels, n_classes, weights, mins, maxs, test):
        X, y, T = _wnd_rows(train, labels, test)
        N, F = X.shape
        nt = T.shape[0]
        w, mn, mx = _wnd_vecs(F, weights, mins, maxs)
        probs = np.zeros((nt, n_classes))
        pred = np.zeros(nt, dtype=np.int32)
        check(lib().wc_wnd_classify(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I), int(n_classes),
                                    w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D), mx.ctypes.data_as(_lib.D),
                                    T.ctypes.data_as(_lib.D), nt, probs.ctypes.data_as(_lib.D),
                                    pred.ctypes.data_as(_lib.I)))
        return probs, pred

    def wnd_normalize(self, rows, mins, maxs):
        """signatures::normalize of each row against (mins, maxs): values in [0, 100]."""
        X = np.ascontiguousarray(np.atleast_2d(rows), dtype=np.float64)
        if X.ndim != 2:
            raise WndcharmError("rows must be an (n, F) array")
        n, F = X.shape
        mn, mx = _wnd_vecs(F, mins, maxs)
        out = np.zeros_like(X)
        check(lib().wc_wnd_normalize(self._h, X.ctypes.data_as(_lib.D), n, F, mn.ctypes.data_as(_lib.D),
                                     mx.ctypes.data_as(_lib.D), out.ctypes.data_as(_lib.D)))
        return out

    def wnd_fit_stats(self, stage, train, labels, n_classes, mins=None, maxs=None, means=None):
        """wc_wnd_fit_stats on these training rows (a shard): stage 0 ->
        (mins, maxs, counts (C+1)); stage 1 -> per-label sums ((C+1), F);
        stage 2 -> per-label sums of squared deviations ((C+1), F)."""
        X, y = _wnd_rows(train, labels)
        N, F = X.shape
        C = int(n_classes)
        LL = ctypes.POINTER(ctypes.c_longlong)
        arg = lambda v: None if v is None else _wnd_vecs(F, v)[0]  # noqa: E731
        mn, mx = arg(mins), arg(maxs)
        me = None if means is None else np.ascontiguousarray(means, dtype=np.float64)
        if me is not None and me.shape != (C + 1, F):
            raise WndcharmError("means must be a (%d, %d) array" % (C + 1, F))
        ptr = lambda v: None if v is None else v.ctypes.data_as(_lib.D)  # noqa: E731
        if stage == 0:
            out = np.zeros(2 * F)
            counts = np.zeros(C + 1, dtype=np.int64)
            check(lib().wc_wnd_fit_stats(self._h, 0, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I), C,
                                         None, None, None, out.ctypes.data_as(_lib.D), counts.ctypes.data_as(LL)))
            return out[:F], out[F:], counts
        out = np.zeros((C + 1, F))
        check(lib().wc_wnd_fit_stats(self._h, int(stage), X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I),
                                     C, ptr(mn), ptr(mx), ptr(me), out.ctypes.data_as(_lib.D), None))
        return out

    def wnd_fisher(self, n_classes, frac, sums, counts, sq):
        """Fisher weights (SetFisherScores' selection included) from summed
        wnd_fit_stats statistics."""
        sums = np.ascontiguousarray(sums, dtype=np.float64)
        sq = np.ascontiguousarray(sq, dtype=np.float64)
        counts = np.ascontiguousarray(counts, dtype=np.int64)
        C1 = int(n_classes) + 1
        if sums.ndim != 2 or sums.shape[0] != C1 or sq.shape != sums.shape or counts.shape != (C1,):
            raise WndcharmError("sums and sq must be (%d, F) arrays and counts %d values" % (C1, C1))
        F = sums.shape[1]
        w = np.zeros(F)
        check(lib().wc_wnd_fisher(self._h, F, int(n_classes), float(frac), sums.ctypes.data_as(_lib.D),
                                  counts.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                  sq.ctypes.data_as(_lib.D), w.ctypes.data_as(_lib.D)))
        return w

    def wnd_class_sums(self, train, labels, n_classes, weights, mins, maxs, test):
        """classify2's per-class sums of d^-5 and counts over these training
        rows (a shard): (sums (T, C) float64, counts (T, C) int64)."""
        X, y, T = _wnd_rows(train, labels, test)
        N, F = X.shape
        nt = T.shape[0]
        w, mn, mx = _wnd_vecs(F, weights, mins, maxs)
        sums = np.zeros((nt, n_classes))
        counts = np.zeros((nt, n_classes), dtype=np.int64)
        check(lib().wc_wnd_class_sums(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I),
                                      int(n_classes), w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D),
                                      mx.ctypes.data_as(_lib.D), T.ctypes.data_as(_lib.D), nt,
                                      sums.ctypes.data_as(_lib.D),
                                      counts.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        return sums, counts

    def wnd_fit_classify(self, train, labels, n_classes, test, frac=0.15):
        """wnd_fit on the training rows, then wnd_classify of the test rows,
        each array copied to the GPU once: (probs, pred, weights, mins, maxs)."""
        X, y, T = _wnd_rows(train, labels, test)
        N, F = X.shape
        nt = T.shape[0]
        w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
        probs = np.zeros((nt, n_classes))
        pred = np.zeros(nt, dtype=np.int32)
        check(lib().wc_wnd_fit_classify(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I),
                                        int(n_classes), float(frac), T.ctypes.data_as(_lib.D), nt,
                                        w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D), mx.ctypes.data_as(_lib.D),
                                        probs.ctypes.data_as(_lib.D), pred.ctypes.data_as(_lib.I)))
        return probs, pred, w, mn, mx

    def wnd_classify_device(self, train, labels, n_classes, weights, mins, maxs, test, probs, pred):
        """wc_wnd_classify_device on device tensors (any objects with a
        data_ptr(): float64 train (N, F), int32 labels, float64 weights / mins /
        maxs (F,), float64 test (T, F); outputs float64 probs (T, C), int32 pred)."""
        N, F = train.shape
        T = test.shape[0]
        vp = ctypes.c_void_p
        check(lib().wc_wnd_classify_device(self._h, vp(train.data_ptr()), N, F, vp(labels.data_ptr()),
                                           int(n_classes), vp(weights.data_ptr()), vp(mins.data_ptr()),
                                           vp(maxs.data_ptr()), vp(test.data_ptr()), T, vp(probs.data_ptr()),
                                           vp(pred.data_ptr())))

    def wnd_fit_device(self, train, labels, n_classes, frac, weights, mins, maxs):
        """wc_wnd_fit_device on device tensors (outputs float64 (F,) each)."""
        N, F = train.shape
        vp = ctypes.c_void_p
        check(lib().wc_wnd_fit_device(self._h, vp(train.data_ptr()), N, F, vp(labels.data_ptr()), int(n_classes),
                                      float(frac), vp(weights.data_ptr()), vp(mins.data_ptr()), vp(maxs.data_ptr())))

    @staticmethod
    def wnd_last_stats():
        """What this thread's last WND-5 classification did: (tensor-core path
        ran, test rows recomputed in FP64, weighted features, tensor-core CTAs,
        tensor-core kernel time in ns, tensor FLOPs it issued)."""
        st = (ctypes.c_longlong * 6)()
        check(lib().wc_wnd_last_stats(st))
        return tuple(int(v) for v in st)

    def wnd_classify_images(self, train, labels, n_classes, weights, mins, maxs, test, tiles, max_tile=False):
        """TrainingSet::ClassifyImage with WND-5 for images of `tiles`
        consecutive test rows: (probs (n_images, C), pred (n_images,),
        normalisation factors (n_images,))."""
        X, y, T = _wnd_rows(train, labels, test)
        N, F = X.shape
        if T.shape[0] % tiles:
            raise WndcharmError("%d test rows are not whole images of %d tiles" % (T.shape[0], tiles))
        n_img = T.shape[0] // tiles
        w, mn, mx = _wnd_vecs(F, weights, mins, maxs)
        probs = np.zeros((n_img, n_classes))
        pred = np.zeros(n_img, dtype=np.int32)
        norm = np.zeros(n_img)
        check(lib().wc_wnd_classify_images(self._h, X.ctypes.data_as(_lib.D), N, F, y.ctypes.data_as(_lib.I),
                                           int(n_classes), w.ctypes.data_as(_lib.D), mn.ctypes.data_as(_lib.D),
                                           mx.ctypes.data_as(_lib.D), T.ctypes.data_as(_lib.D), n_img, int(tiles),
                                           1 if max_tile else 0, probs.ctypes.data_as(_lib.D),
                                           pred.ctypes.data_as(_lib.I), norm.ctypes.data_as(_lib.D)))
        return probs, pred, norm

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


def extract_samples(plan, images, sampling, precision="fp64", bits=16):
    return default_engine(precision).extract_samples(plan, images, sampling, bits=bits)


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
    """(pixels, bits) of an 8/16-bit grayscale or RGB TIFF, read as
    ImageMatrix::LoadTIFF reads it: a uint8 / uint16 array of (height, width),
    or (height, width, 3) for RGB."""
    L = lib()
    w, h, b, spp = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    p = path.encode()
    check(L.wc_tiff_layout(p, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b), ctypes.byref(spp)))
    shape = (h.value, w.value) if spp.value == 1 else (h.value, w.value, spp.value)
    out = np.empty(shape, dtype=np.uint8 if b.value == 8 else np.uint16)
    check(L.wc_tiff_read(p, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
    return out, b.value
