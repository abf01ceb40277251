"""ctypes binding of libwndcharm_gb300.so (the C ABI in include/wndcharm_gb300.h).

The library is built in-tree by wnd-charm_gb300/build.py.  Loading fails loudly
when it is missing: there is no CPU fallback behind this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(HERE, "build", "libwndcharm_gb300.so")

WC_OK = 0
WC_PLAN_SHORT, WC_PLAN_LONG, WC_PLAN_SHORT_COLOR, WC_PLAN_LONG_COLOR = 0, 1, 2, 3
WC_U8, WC_U16, WC_F32, WC_F64, WC_RGB8, WC_RGB16 = 0, 1, 2, 3, 4, 5
WC_PREC_FP64, WC_PREC_MIXED = 0, 1

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)


class wc_image_desc(ctypes.Structure):
    _fields_ = [("pixels", ctypes.c_void_p), ("dtype", ctypes.c_int), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("bits", ctypes.c_int), ("on_device", ctypes.c_int)]


class wc_sampling(ctypes.Structure):
    _fields_ = [("crop_x", ctypes.c_int), ("crop_y", ctypes.c_int), ("crop_w", ctypes.c_int), ("crop_h", ctypes.c_int),
                ("downsample_x", ctypes.c_double), ("downsample_y", ctypes.c_double),
                ("norm_min", ctypes.c_double), ("norm_max", ctypes.c_double), ("norm_range", ctypes.c_longlong),
                ("norm_mean", ctypes.c_double), ("norm_std", ctypes.c_double),
                ("rotations", ctypes.c_int), ("tiles_x", ctypes.c_int), ("tiles_y", ctypes.c_int)]


class WndcharmError(RuntimeError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise WndcharmError("CUDA library not built: %s (run wnd-charm_gb300/build.py)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.wc_last_error.restype = ctypes.c_char_p
        L.wc_version.restype = ctypes.c_char_p
        L.wc_plan_get.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.wc_plan_from_names.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.POINTER(vp)]
        L.wc_plan_free.argtypes = [vp]
        L.wc_plan_free.restype = None
        L.wc_plan_n_features.argtypes = [vp]
        L.wc_plan_feature_name.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        L.wc_plan_n_groups.argtypes = [vp]
        L.wc_plan_group.argtypes = [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, I, I]
        L.wc_engine_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.wc_engine_destroy.argtypes = [vp]
        L.wc_engine_destroy.restype = None
        L.wc_engine_set_stream.argtypes = [vp, vp]
        L.wc_engine_set_option.argtypes = [vp, ctypes.c_char_p, ctypes.c_longlong]
        L.wc_engine_tuning_report.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
        L.wc_engine_launch_count.argtypes = [vp]
        L.wc_engine_launch_count.restype = ctypes.c_longlong
        L.wc_engine_profile.argtypes = [vp, ctypes.c_int]
        L.wc_engine_profile_report.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
        L.wc_extract.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, D]
        L.wc_extract_batch.argtypes = [vp, vp, ctypes.POINTER(wc_image_desc), ctypes.c_int, vp, ctypes.c_int]
        L.wc_transform.argtypes = [vp, ctypes.c_char_p, D, ctypes.c_int, ctypes.c_int, D, ctypes.c_longlong, I, I]
        SP = ctypes.POINTER(wc_sampling)
        L.wc_sampling_default.argtypes = [SP]
        L.wc_sampling_default.restype = None
        L.wc_sampling_count.argtypes = [SP]
        L.wc_sample_size.argtypes = [SP, ctypes.c_int, ctypes.c_int, ctypes.c_int, I, I]
        L.wc_preprocess.argtypes = [vp, ctypes.POINTER(wc_image_desc), SP, ctypes.c_int, vp, ctypes.c_longlong, I, I,
                                    ctypes.c_int]
        L.wc_extract_samples.argtypes = [vp, vp, ctypes.POINTER(wc_image_desc), ctypes.c_int, SP, vp, ctypes.c_int]
        L.wc_wavelet_noalloc.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp]
        L.wc_tiff_info.argtypes = [ctypes.c_char_p, I, I, I]
        L.wc_tiff_layout.argtypes = [ctypes.c_char_p, I, I, I, I]
        L.wc_tiff_read.argtypes = [ctypes.c_char_p, vp, ctypes.c_longlong]
        L.wc_engine_graph_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.wc_tiff_device_bytes.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_longlong)]
        L.wc_tiff_read_device.argtypes = [vp, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, vp, ctypes.c_longlong,
                                          ctypes.POINTER(wc_image_desc)]
        L.wc_wnd_fit.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, ctypes.c_double, D, D, D]
        L.wc_wnd_classify.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, D, D, D, D, ctypes.c_int, D, I]
        L.wc_wnd_normalize.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, D, D, D]
        L.wc_wnd_class_sums.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, D, D, D, D, ctypes.c_int, D,
                                        ctypes.POINTER(ctypes.c_longlong)]
        LL = ctypes.POINTER(ctypes.c_longlong)
        L.wc_wnd_fit_stats.argtypes = [vp, ctypes.c_int, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, D, D, D, D, LL]
        L.wc_wnd_fisher.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, D, LL, D, D]
        L.wc_wnd_fit_classify.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, ctypes.c_double, D,
                                          ctypes.c_int, D, D, D, D, I]
        L.wc_wnd_fit_device.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp, vp,
                                         vp]
        L.wc_wnd_classify_device.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp, vp, vp,
                                             ctypes.c_int, vp, vp]
        L.wc_wnd_last_stats.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
        L.wc_wnd_grad.argtypes = [vp, vp, D, ctypes.c_int, I, ctypes.c_int, D, D, D, ctypes.POINTER(wc_image_desc),
                                  ctypes.c_int, D, ctypes.c_int, D, D, D]
        L.wc_wnd_classify_images.argtypes = [vp, D, ctypes.c_int, ctypes.c_int, I, ctypes.c_int, D, D, D, D, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, D, I, D]
        _lib = L
    return _lib


def check(rc):
    if rc < 0:
        raise WndcharmError(lib().wc_last_error().decode(errors="replace"))
    return rc
