"""ctypes declarations of the C ABI in include/qmiv_gb300.h.

This is the binding a Python caller adds on top of libqmiv_gb300.so; the structures
mirror the header field for field. Loading fails loudly (ImportError) when the library
has not been built: there is no CPU fallback behind this module.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqmiv_gb300.so")

QMIV_OK, QMIV_BAD_ARG, QMIV_UNSUPPORTED, QMIV_CUDA_ERROR, QMIV_DEVICE_TIMEOUT, QMIV_OUT_OF_MEMORY, QMIV_TOO_LARGE = range(7)
M_PSNR, M_WSPSNR, M_IVPSNR, M_SSIM, M_MSSSIM, M_IVSSIM = (1 << i for i in range(6))
M_ALL = 0x3F
CF420, CF444 = 420, 444
SSIM_REF10, SSIM_GAUSS11 = 0, 1

c_i32, c_u32, c_u64, c_f32, c_f64 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_double


class Pic(ctypes.Structure):
    _fields_ = [("plane", ctypes.c_void_p * 3), ("stride", c_i32 * 3), ("width", c_i32), ("height", c_i32),
                ("bitdepth", c_i32), ("sample_bytes", c_i32), ("chroma_format", c_i32), ("is_device", c_i32)]


class Options(ctypes.Structure):
    _fields_ = [("search_range", c_i32), ("cmp_w_search", c_i32 * 4), ("cmp_w_avg", c_i32 * 4),
                ("unnoticeable", c_f32 * 4), ("use_ws", c_i32), ("lon_deg", c_i32), ("lat_deg", c_i32),
                ("fake_exact", c_i32), ("legacy_ws8", c_i32), ("ssim_window", c_i32), ("scratch_metrics", c_u32)]


class FrameResult(ctypes.Structure):
    _fields_ = [("metrics", c_u32), ("status", c_i32), ("gcd_r2t", c_i32 * 4), ("exact", c_i32 * 4),
                ("psnr", c_f64 * 4), ("psnr_pic", c_f64), ("wspsnr", c_f64 * 4), ("wspsnr_pic", c_f64),
                ("ivpsnr", c_f64), ("ivpsnr_r2t", c_f64), ("ivpsnr_t2r", c_f64),
                ("sse_r2t", c_u64 * 4), ("sse_t2r", c_u64 * 4),
                ("ssim", c_f64 * 4), ("ssim_pic", c_f64), ("msssim", c_f64 * 4), ("msssim_pic", c_f64),
                ("ivssim", c_f64), ("ivssim_r2t", c_f64), ("ivssim_t2r", c_f64)]

    def to_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class SeqResult(ctypes.Structure):
    _fields_ = [("num_frames", c_i32), ("metrics", c_u32), ("psnr", c_f64 * 4), ("psnr_pic", c_f64),
                ("wspsnr", c_f64 * 4), ("wspsnr_pic", c_f64), ("ivpsnr", c_f64), ("ssim", c_f64 * 4),
                ("ssim_pic", c_f64), ("msssim", c_f64 * 4), ("msssim_pic", c_f64), ("ivssim", c_f64)]


class Mask(ctypes.Structure):
    _fields_ = [("plane", ctypes.c_void_p), ("stride", c_i32), ("bitdepth", c_i32), ("sample_bytes", c_i32),
                ("is_device", c_i32)]


class Job(ctypes.Structure):
    _fields_ = [("pic0", Pic), ("pic1", Pic), ("metrics", c_u32), ("use_ws", c_i32),
                ("scp0", ctypes.c_void_p * 3), ("scp1", ctypes.c_void_p * 3), ("scp_stride", c_i32)]


# every symbol include/qmiv_gb300.h declares: (name, restype, argtypes)
_P = ctypes.POINTER
_vp = ctypes.c_void_p
SIGNATURES = [
    ("qmiv_abi_version", c_i32, []),
    ("qmiv_status_str", ctypes.c_char_p, [c_i32]),
    ("qmiv_last_error", ctypes.c_char_p, []),
    ("qmiv_default_options", None, [_P(Options)]),
    ("qmiv_create", c_i32, [_P(_vp), _P(Options), c_i32, c_i32, c_i32]),
    ("qmiv_destroy", c_i32, [_vp]),
    ("qmiv_set_options", c_i32, [_vp, _P(Options)]),
    ("qmiv_calc_frame", c_i32, [_vp, _P(Pic), _P(Pic), c_u32, _P(FrameResult), _vp]),
    ("qmiv_calc_frame_masked", c_i32, [_vp, _P(Pic), _P(Pic), _P(Mask), c_u32, _P(FrameResult), _vp]),
    ("qmiv_calc_batch", c_i32, [_vp, _P(Job), c_i32, _vp, _vp]),
    ("qmiv_calc_batch_host", c_i32, [_vp, _P(Job), c_i32, _vp, ctypes.c_size_t, _vp]),
    ("qmiv_batch_graph_create", c_i32, [_vp, _P(Job), c_i32, _vp, _vp, _P(_vp)]),
    ("qmiv_batch_graph_launch", c_i32, [_vp, _vp]),
    ("qmiv_batch_graph_destroy", c_i32, [_vp]),
    ("qmiv_gcd", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_i32), _vp]),
    ("qmiv_psnr", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_f64), _P(c_f64), _vp]),
    ("qmiv_psnr_static", c_i32, [_P(Pic), _P(Pic), _P(Options), _P(FrameResult), _vp]),
    ("qmiv_ivpsnr", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_i32), _P(c_f64), _P(c_f64), _P(c_f64), _vp]),
    ("qmiv_scp", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_i32), _P(_vp), _P(_vp), c_i32, c_i32, _vp]),
    ("qmiv_cps_maps", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_i32), _vp, _vp, c_i32, c_i32, _vp, _vp]),
    ("qmiv_ssim", c_i32, [_vp, _P(Pic), _P(Pic), c_i32, _P(c_f64), _vp]),
    ("qmiv_msssim", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_f64), _vp]),
    ("qmiv_ivssim", c_i32, [_vp, _P(Pic), _P(Pic), _P(c_i32), _P(c_f64), _P(c_f64), _P(c_f64), _vp]),
    ("qmiv_loss_workspace_size", c_i32, [c_i32, c_i32, c_i32, _P(Options), _P(ctypes.c_size_t)]),
    ("qmiv_loss_forward", c_i32, [_vp, _vp, c_i32, c_i32, c_i32, _P(Options), _vp, ctypes.c_size_t, _vp, _vp, _vp]),
    ("qmiv_loss_backward", c_i32, [_vp, _vp, c_i32, c_i32, c_i32, _P(Options), _vp, ctypes.c_size_t, _vp, _vp, _vp,
                                   _vp]),
    ("qmiv_check_range", c_i32, [_P(Pic), c_i32, _P(ctypes.c_int64), _vp]),
    ("qmiv_color_convert", c_i32, [_P(Pic), _P(_vp), c_i32, c_i32, c_i32, _vp]),
    ("qmiv_yuv_open", c_i32, [_P(_vp), ctypes.c_char_p, c_i32, c_i32, c_i32, c_i32]),
    ("qmiv_yuv_frames", ctypes.c_int64, [_vp]),
    ("qmiv_yuv_read", c_i32, [_vp, ctypes.c_int64, _P(Pic), _vp]),
    ("qmiv_yuv_close", c_i32, [_vp]),
    ("qmiv_finish_sequence", c_i32, [_vp, _P(SeqResult)]),
    ("qmiv_reset_sequence", c_i32, [_vp]),
    ("qmiv_kernel_launches", ctypes.c_int64, [_vp]),
    ("qmiv_cps_variant_count", c_i32, []),
    ("qmiv_cps_variant_name", ctypes.c_char_p, [c_i32]),
    ("qmiv_set_cps_variant", c_i32, [_vp, c_i32]),
    ("qmiv_autotune_cps", c_i32, [_vp, _P(Job), c_i32, _vp, c_i32, _vp, _P(c_i32), _P(c_f64)]),
    ("qmiv_test_wait_timeout", c_i32, [_vp, c_u32]),
    ("qmiv_set_profiling", c_i32, [_vp, c_i32]),
    ("qmiv_kernel_times", c_i32, [_vp, _P(ctypes.c_char_p), _P(c_f64), c_i32]),
]

_lib = None


def load():
    """Load libqmiv_gb300.so and declare every entry point. Raises ImportError if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libqmiv_gb300.so is not built (run __graft_entry__.build() or "
                          "python ivpsnr_gb300/build.py); the metric path has no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class QmivError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.qmiv_last_error().decode(errors="replace")
        super().__init__("%s failed: %s (%s)" % (where, lib.qmiv_status_str(status).decode(), msg))
        self.status = status


def check(status, where):
    if status != QMIV_OK:
        raise QmivError(status, where)
