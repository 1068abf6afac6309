"""ivpsnr_gb300 — GB300 implementation of the QMIV metric path (IV-PSNR, PSNR, WS-PSNR,
SSIM, MS-SSIM, IV-SSIM) behind the C ABI in include/qmiv_gb300.h.

The Python layer is a thin ctypes client of libqmiv_gb300.so (see _abi.py): it builds the
picture descriptors from numpy arrays (host memory) or torch CUDA tensors (device memory)
and calls the C ABI; every metric is computed by the CUDA kernels.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import (CF420, CF444, M_ALL, M_IVPSNR, M_IVSSIM, M_MSSSIM, M_PSNR, M_SSIM, M_WSPSNR, QmivError,
                   SSIM_GAUSS11, SSIM_REF10)

__all__ = ["Processor", "make_pic", "cps_variants", "default_options", "QmivError", "CF420", "CF444", "M_ALL", "M_PSNR",
           "M_WSPSNR", "M_IVPSNR", "M_SSIM", "M_MSSSIM", "M_IVSSIM", "SSIM_REF10", "SSIM_GAUSS11"]


def default_options(**kw):
    o = _abi.Options()
    _abi.load().qmiv_default_options(ctypes.byref(o))
    for k, v in kw.items():
        if k in ("cmp_w_search", "cmp_w_avg", "unnoticeable"):
            getattr(o, k)[:] = list(v) + [0] * (4 - len(v))
        else:
            setattr(o, k, int(v))
    return o


def _ptr_and_stride(a):
    """(address, row stride in samples, is_device, itemsize) of a 2-D numpy array or torch tensor."""
    if hasattr(a, "data_ptr"):  # torch tensor
        assert a.dim() == 2
        return a.data_ptr(), a.stride(0), int(a.is_cuda), a.element_size()
    assert a.ndim == 2 and a.strides[1] == a.itemsize
    return a.ctypes.data, a.strides[0] // a.itemsize, 0, a.itemsize


def cps_variants():
    lib = _abi.load()
    return [lib.qmiv_cps_variant_name(i).decode() for i in range(lib.qmiv_cps_variant_count())]


def make_pic(planes, bitdepth, chroma_format=CF420):
    """qmiv_pic for three 2-D planes (Y, Cb, Cr) of uint8/uint16 numpy arrays or torch tensors."""
    p = _abi.Pic()
    keep = []
    dev = None
    for c in range(3):
        addr, stride, is_dev, isz = _ptr_and_stride(planes[c])
        p.plane[c] = addr
        p.stride[c] = stride
        dev = is_dev if dev is None else dev
        keep.append(planes[c])
        p.sample_bytes = isz
    y = planes[0]
    shape = tuple(y.shape)
    p.height, p.width = int(shape[0]), int(shape[1])
    p.bitdepth = bitdepth
    p.chroma_format = chroma_format
    p.is_device = dev
    p._keep = keep
    return p


class BatchGraph:
    """A captured batch (qmiv_batch_graph_*): launch() replays it on a stream."""

    def __init__(self, lib, g):
        self.lib, self.g = lib, g

    def launch(self, stream):
        _abi.check(self.lib.qmiv_batch_graph_launch(self.g, stream), "qmiv_batch_graph_launch")

    def close(self):
        if self.g:
            self.lib.qmiv_batch_graph_destroy(self.g)
            self.g = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Processor:
    """One qmiv handle: the GPU counterpart of the reference's processor objects
    (xIVPSNR / xSSIM / xIVSSIM / xGlobClrDiffProc / xShftCompPicProc)."""

    def __init__(self, max_width, max_height, max_jobs=1, **opts):
        self.lib = _abi.load()
        self.opts = default_options(**opts)
        h = ctypes.c_void_p()
        _abi.check(self.lib.qmiv_create(ctypes.byref(h), ctypes.byref(self.opts), max_width, max_height, max_jobs),
                   "qmiv_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.qmiv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def calc_frame(self, pic0, pic1, metrics=M_ALL, stream=0):
        r = _abi.FrameResult()
        _abi.check(self.lib.qmiv_calc_frame(self.h, ctypes.byref(pic0), ctypes.byref(pic1), metrics,
                                            ctypes.byref(r), stream), "qmiv_calc_frame")
        return r.to_dict()

    def calc_frame_masked(self, pic0, pic1, mask, mask_bitdepth=8, metrics=M_PSNR | M_WSPSNR | M_IVPSNR, stream=0):
        """qmiv_calc_frame_masked; mask: a 2-D uint8/uint16 numpy array or torch tensor (luma size)."""
        addr, stride, is_dev, isz = _ptr_and_stride(mask)
        m = _abi.Mask(addr, stride, mask_bitdepth, isz, is_dev)
        r = _abi.FrameResult()
        _abi.check(self.lib.qmiv_calc_frame_masked(self.h, ctypes.byref(pic0), ctypes.byref(pic1), ctypes.byref(m),
                                                   metrics, ctypes.byref(r), stream), "qmiv_calc_frame_masked")
        return r.to_dict()

    def gcd(self, pic0, pic1, stream=0):
        g = (ctypes.c_int32 * 4)()
        _abi.check(self.lib.qmiv_gcd(self.h, ctypes.byref(pic0), ctypes.byref(pic1), g, stream), "qmiv_gcd")
        return list(g)

    def ivpsnr(self, pic0, pic1, gcd=None, stream=0):
        iv, r2t, t2r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        g = (ctypes.c_int32 * 4)(*(list(gcd) + [0] * (4 - len(gcd)))) if gcd is not None else None
        _abi.check(self.lib.qmiv_ivpsnr(self.h, ctypes.byref(pic0), ctypes.byref(pic1), g, ctypes.byref(iv),
                                        ctypes.byref(r2t), ctypes.byref(t2r), stream), "qmiv_ivpsnr")
        return iv.value, r2t.value, t2r.value

    def scp(self, pic0, pic1, scp0, scp1, gcd=None, is_device=False, stream=0):
        """scp0/scp1: three 2-D uint16 planes each (numpy or torch); written in place."""
        g = (ctypes.c_int32 * 4)(*(list(gcd) + [0] * (4 - len(gcd)))) if gcd is not None else None
        a0 = (ctypes.c_void_p * 3)(*[_ptr_and_stride(x)[0] for x in scp0])
        a1 = (ctypes.c_void_p * 3)(*[_ptr_and_stride(x)[0] for x in scp1])
        stride = _ptr_and_stride(scp0[0])[1]
        _abi.check(self.lib.qmiv_scp(self.h, ctypes.byref(pic0), ctypes.byref(pic1), g, a0, a1, stride,
                                     int(is_device), stream), "qmiv_scp")

    def cps_maps(self, pic0, pic1, gcd=None, stream=0):
        """qmiv_cps_maps with host outputs: (map_r2t, map_t2r) int16 (H, W) window indices
        (dy + B)(2B + 1) + (dx + B) of each pixel's argmin, and the per-row squared errors at the
        argmin, uint64 (2, H, 3)."""
        w, h = pic0.width, pic0.height
        m0 = np.zeros((h, w), np.int16)
        m1 = np.zeros((h, w), np.int16)
        rows = np.zeros((2, h, 3), np.uint64)
        g = (ctypes.c_int32 * 4)(*(list(gcd) + [0] * (4 - len(gcd)))) if gcd is not None else None
        _abi.check(self.lib.qmiv_cps_maps(self.h, ctypes.byref(pic0), ctypes.byref(pic1), g, m0.ctypes.data,
                                          m1.ctypes.data, w, 0, rows.ctypes.data, stream), "qmiv_cps_maps")
        return m0, m1, rows

    def calc_batch(self, jobs, results_ptr, stream=0):
        arr = (_abi.Job * len(jobs))(*jobs)
        _abi.check(self.lib.qmiv_calc_batch(self.h, arr, len(jobs), results_ptr, stream), "qmiv_calc_batch")

    def calc_batch_host(self, jobs, results_ptr, group_bytes=0, stream=0):
        """qmiv_calc_batch_host: jobs with host (pinned) pictures, uploaded in groups overlapped with
        the measurement; results_ptr is device memory; asynchronous on stream."""
        arr = (_abi.Job * len(jobs))(*jobs)
        _abi.check(self.lib.qmiv_calc_batch_host(self.h, arr, len(jobs), results_ptr, group_bytes, stream),
                   "qmiv_calc_batch_host")

    def capture_batch(self, jobs, results_ptr, stream):
        """qmiv_batch_graph_create: the batch recorded once as a CUDA graph; returns a BatchGraph."""
        arr = (_abi.Job * len(jobs))(*jobs)
        g = ctypes.c_void_p()
        _abi.check(self.lib.qmiv_batch_graph_create(self.h, arr, len(jobs), results_ptr, stream, ctypes.byref(g)),
                   "qmiv_batch_graph_create")
        return BatchGraph(self.lib, g)

    def finish_sequence(self):
        r = _abi.SeqResult()
        _abi.check(self.lib.qmiv_finish_sequence(self.h, ctypes.byref(r)), "qmiv_finish_sequence")
        return {n: (list(getattr(r, n)) if hasattr(getattr(r, n), "__len__") else getattr(r, n)) for n, _ in r._fields_}

    def test_wait_timeout(self, polls):
        """qmiv_test_wait_timeout: polls > 0 makes the first bulk-copy wait of every block give up."""
        _abi.check(self.lib.qmiv_test_wait_timeout(self.h, polls), "qmiv_test_wait_timeout")

    def set_cps_variant(self, v):
        _abi.check(self.lib.qmiv_set_cps_variant(self.h, v), "qmiv_set_cps_variant")

    def autotune_cps(self, jobs, results_ptr, reps=3, stream=0):
        """qmiv_autotune_cps: (variant index, variant name, CPS ms) of the fastest fitting variant,
        which the handle keeps using."""
        arr = (_abi.Job * len(jobs))(*jobs)
        best, ms = ctypes.c_int32(), ctypes.c_double()
        _abi.check(self.lib.qmiv_autotune_cps(self.h, arr, len(jobs), results_ptr, reps, stream, ctypes.byref(best),
                                              ctypes.byref(ms)), "qmiv_autotune_cps")
        return best.value, self.lib.qmiv_cps_variant_name(best.value).decode(), ms.value

    def set_profiling(self, on=True):
        _abi.check(self.lib.qmiv_set_profiling(self.h, int(on)), "qmiv_set_profiling")

    def kernel_times(self, max_n=64):
        """[(kernel name, ms)] of the last calc call's launches (needs set_profiling(True))."""
        names = (ctypes.c_char_p * max_n)()
        ms = (ctypes.c_double * max_n)()
        n = self.lib.qmiv_kernel_times(self.h, names, ms, max_n)
        if n < 0:
            raise RuntimeError("qmiv_kernel_times failed")
        return [(names[i].decode(), ms[i]) for i in range(n)]

    def kernel_launches(self):
        return int(self.lib.qmiv_kernel_launches(self.h))
