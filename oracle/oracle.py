"""ctypes wrapper of the CPU oracle (oracle/qmiv_oracle.c) — TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and bench.py's CPU-baseline leg import this module, and
only as the checker. It restates the reference's metric path (libs/pmbb-ivqm) on the
CPU; see qmiv_oracle.h for the file:line map and how it is pinned to the reference.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class OqPic(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("bitdepth", ctypes.c_int32),
                ("plane", ctypes.POINTER(ctypes.c_uint16) * 3)]


class OqOpts(ctypes.Structure):
    _fields_ = [("search_range", ctypes.c_int32), ("w_search", ctypes.c_int32 * 3), ("w_avg", ctypes.c_int32 * 3),
                ("unnoticeable", ctypes.c_float * 3), ("use_ws", ctypes.c_int32), ("lat_range_deg", ctypes.c_int32),
                ("ssim_window", ctypes.c_int32), ("nthreads", ctypes.c_int32)]


class OqFrameResult(ctypes.Structure):
    _fields_ = [("gcd", ctypes.c_int32 * 3), ("exact", ctypes.c_int32 * 3),
                ("psnr", ctypes.c_double * 3), ("wspsnr", ctypes.c_double * 3),
                ("ivpsnr", ctypes.c_double), ("ivpsnr_r2t", ctypes.c_double), ("ivpsnr_t2r", ctypes.c_double),
                ("sse_r2t", ctypes.c_uint64 * 3), ("sse_t2r", ctypes.c_uint64 * 3),
                ("ssim", ctypes.c_double * 3), ("msssim", ctypes.c_double * 3),
                ("ivssim", ctypes.c_double), ("ivssim_r2t", ctypes.c_double), ("ivssim_t2r", ctypes.c_double)]


def build():
    """Compile liboq.so with the committed Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboq.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.oq_frame.argtypes = [P(OqPic), P(OqPic), P(OqOpts), ctypes.c_int32, P(OqFrameResult)]
        L.oq_cps_dir.argtypes = [P(OqPic), P(OqPic), P(ctypes.c_int32), ctypes.c_int32, P(ctypes.c_int32),
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
        L.oq_gcd.argtypes = [P(OqPic), P(OqPic), P(ctypes.c_float), P(ctypes.c_int32)]
        L.oq_ssim_plane.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        L.oq_ssim_plane.restype = ctypes.c_double
        L.oq_msssim.argtypes = [P(OqPic), P(OqPic), ctypes.c_int32, ctypes.c_int32, P(ctypes.c_double)]
        L.oq_ssim_table.argtypes = [ctypes.c_int32, ctypes.c_void_p]
        L.oq_kbns.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.oq_kbns.restype = ctypes.c_double
        L.oq_ws_weights.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, P(ctypes.c_double)]
        L.oq_unpack_frame.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_void_p]
        L.oq_unpack_frame.restype = ctypes.c_int
        L.oq_downsample.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
        L.oq_count_nonzero.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]
        L.oq_count_nonzero.restype = ctypes.c_int32
        L.oq_gcd_masked.argtypes = [P(OqPic), P(OqPic), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                    P(ctypes.c_float), P(ctypes.c_int32)]
        L.oq_psnr_masked.argtypes = [P(OqPic), P(OqPic), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_void_p, ctypes.c_double, P(ctypes.c_double)]
        L.oq_ivpsnr_masked.argtypes = [P(OqPic), P(OqPic), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                       P(ctypes.c_int32), P(OqOpts), ctypes.c_void_p,
                                       P(ctypes.c_double), P(ctypes.c_double)]
        L.oq_ivpsnr_masked.restype = ctypes.c_double
        L.oq_color_matrix.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
        L.oq_color_convert.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_int32]
        L.oq_range_clip.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        L.oq_range_clip.restype = ctypes.c_int64
        _LIB = L
    return _LIB


def _pic(planes444, bd):
    """planes444: uint16 array (3, H, W), C-contiguous."""
    a = np.ascontiguousarray(planes444, dtype=np.uint16)
    p = OqPic()
    p.height, p.width = int(a.shape[1]), int(a.shape[2])
    p.bitdepth = bd
    for c in range(3):
        p.plane[c] = a[c].ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
    return p, a


def opts(search_range=2, w_search=(4, 1, 1), w_avg=(4, 1, 1), unnoticeable=(0.01, 0.01, 0.01),
         use_ws=False, lat_range_deg=180, ssim_window=0, nthreads=1):
    o = OqOpts()
    o.search_range = search_range
    o.w_search[:] = list(w_search)
    o.w_avg[:] = list(w_avg)
    o.unnoticeable[:] = list(unnoticeable)
    o.use_ws = int(use_ws)
    o.lat_range_deg = lat_range_deg
    o.ssim_window = ssim_window
    o.nthreads = nthreads
    return o


def upsample420(planes420, w, h):
    """Planar 4:2:0 (Y, Cb, Cr) -> (3, H, W) 4:4:4 by nearest-neighbour (xPixelOpsSTD.cpp:30)."""
    y, cb, cr = planes420
    out = np.empty((3, h, w), np.uint16)
    out[0] = y.reshape(h, w)
    out[1] = np.repeat(np.repeat(cb.reshape(h // 2, w // 2), 2, 0), 2, 1)
    out[2] = np.repeat(np.repeat(cr.reshape(h // 2, w // 2), 2, 0), 2, 1)
    return out


def frame(p0, p1, bd, do_ssim=True, **kw):
    """Every metric of one frame pair, in the application's order (xAppQMIV.cpp:661-751).
    p0, p1: uint16 (3, H, W) 4:4:4 planes. Returns a dict."""
    L = lib()
    a, a_keep = _pic(p0, bd)
    b, b_keep = _pic(p1, bd)
    o = opts(**kw)
    r = OqFrameResult()
    L.oq_frame(ctypes.byref(a), ctypes.byref(b), ctypes.byref(o), int(do_ssim), ctypes.byref(r))
    out = {
        "gcd": list(r.gcd), "exact": list(r.exact), "psnr": list(r.psnr), "wspsnr": list(r.wspsnr),
        "ivpsnr": r.ivpsnr, "ivpsnr_r2t": r.ivpsnr_r2t, "ivpsnr_t2r": r.ivpsnr_t2r,
        "sse_r2t": list(r.sse_r2t), "sse_t2r": list(r.sse_t2r),
    }
    if do_ssim:
        out.update({"ssim": list(r.ssim), "msssim": list(r.msssim), "ivssim": r.ivssim,
                    "ivssim_r2t": r.ivssim_r2t, "ivssim_t2r": r.ivssim_t2r})
    return out


def cps_dir(tst, ref, bd, gcd, search_range=2, w=(4, 1, 1), nthreads=1):
    """One CPS direction: returns (row_sse (H,3) uint64, argmin (H,W) int8, minerr (H,W) int32, scp (3,H,W))."""
    L = lib()
    a, ak = _pic(tst, bd)
    b, bk = _pic(ref, bd)
    H, W = tst.shape[1], tst.shape[2]
    rows = np.zeros((H, 3), np.uint64)
    am = np.zeros((H, W), np.int8)
    me = np.zeros((H, W), np.int32)
    scp = np.zeros((3, H, W), np.uint16)
    g = (ctypes.c_int32 * 3)(*gcd)
    ww = (ctypes.c_int32 * 3)(*w)
    L.oq_cps_dir(ctypes.byref(a), ctypes.byref(b), g, search_range, ww, rows.ctypes.data, am.ctypes.data,
                 me.ctypes.data, scp.ctypes.data, nthreads)
    return rows, am, me, scp


def gcd(p0, p1, bd, unnoticeable=(0.01, 0.01, 0.01)):
    L = lib()
    a, ak = _pic(p0, bd)
    b, bk = _pic(p1, bd)
    out = (ctypes.c_int32 * 3)()
    L.oq_gcd(ctypes.byref(a), ctypes.byref(b), (ctypes.c_float * 3)(*unnoticeable), out)
    return list(out)


def ssim_plane(t, r, bd, calc_l=True, window=0, nthreads=1):
    t = np.ascontiguousarray(t, np.uint16)
    r = np.ascontiguousarray(r, np.uint16)
    return lib().oq_ssim_plane(t.ctypes.data, r.ctypes.data, t.shape[1], t.shape[0], bd, int(calc_l), window, nthreads)


def msssim(p0, p1, bd, window=0, nthreads=1):
    L = lib()
    a, ak = _pic(p0, bd)
    b, bk = _pic(p1, bd)
    out = (ctypes.c_double * 3)()
    L.oq_msssim(ctypes.byref(a), ctypes.byref(b), window, nthreads, out)
    return list(out)


def ssim_table(window=0):
    t = np.zeros((11, 11), np.float32)
    lib().oq_ssim_table(window, t.ctypes.data)
    return t


def kbns(x):
    x = np.ascontiguousarray(x, np.float64)
    return lib().oq_kbns(x.ctypes.data, x.size)


def ws_weights(h, lat_deg=180):
    w = np.zeros(h, np.float64)
    corr = ctypes.c_double()
    lib().oq_ws_weights(h, lat_deg, w.ctypes.data, ctypes.byref(corr))
    return w, corr.value


def downsample(plane):
    plane = np.ascontiguousarray(plane, np.uint16)
    h, w = plane.shape
    out = np.zeros((h // 2, w // 2), np.uint16)
    lib().oq_downsample(plane.ctypes.data, w, h, out.ctypes.data)
    return out


def masked(p0, p1, mask, bd, mask_bd=8, use_ws=False, lat_range_deg=180, **kw):
    """Masked GCD / PSNR / WS-PSNR / IV-PSNR (xAppQMIV.cpp:693-695, 831-893 with a mask)."""
    L = lib()
    a, ak = _pic(p0, bd)
    b, bk = _pic(p1, bd)
    m = np.ascontiguousarray(mask, np.uint16)
    H, W = m.shape
    nnm = L.oq_count_nonzero(m.ctypes.data, W, H)
    o = opts(use_ws=use_ws, lat_range_deg=lat_range_deg, **kw)
    g = (ctypes.c_int32 * 3)()
    L.oq_gcd_masked(ctypes.byref(a), ctypes.byref(b), m.ctypes.data, nnm, mask_bd, o.unnoticeable, g)
    ws, corr = (ws_weights(H, lat_range_deg) if use_ws else (None, 1.0))
    psnr = (ctypes.c_double * 3)()
    L.oq_psnr_masked(ctypes.byref(a), ctypes.byref(b), m.ctypes.data, nnm, mask_bd, None, 1.0, psnr)
    wsp = (ctypes.c_double * 3)()
    L.oq_psnr_masked(ctypes.byref(a), ctypes.byref(b), m.ctypes.data, nnm, mask_bd,
                     ws.ctypes.data if ws is not None else None, corr, wsp)
    r2t = ctypes.c_double()
    t2r = ctypes.c_double()
    iv = L.oq_ivpsnr_masked(ctypes.byref(a), ctypes.byref(b), m.ctypes.data, nnm, mask_bd, g, ctypes.byref(o),
                            ws.ctypes.data if ws is not None else None, ctypes.byref(r2t), ctypes.byref(t2r))
    exact = [int(np.array_equal(p0[c], p1[c])) for c in range(3)]
    area = W * H
    fake = 10.0 * np.log10(float(area * ((1 << bd) - 1) ** 2))
    psnr = [fake if exact[c] else psnr[c] for c in range(3)]
    wsp = [fake if exact[c] else wsp[c] for c in range(3)]
    return {"nnm": nnm, "gcd": list(g), "psnr": psnr, "wspsnr": wsp, "ivpsnr": iv,
            "ivpsnr_r2t": r2t.value, "ivpsnr_t2r": t2r.value, "exact": exact}


def color_convert(planes, bd, space, to_ycbcr):
    """xColorSpaceSTD::ConvertRGB2YCbCr_I32 / ConvertYCbCr2RGB_I32 of three uint16 planes."""
    src = np.ascontiguousarray(np.stack(planes), np.uint16)
    _, h, w = src.shape
    out = np.zeros_like(src)
    lib().oq_color_convert(src.ctypes.data, out.ctypes.data, w, h, bd, space, int(to_ycbcr))
    return out


def color_matrix(space, to_ycbcr):
    m = (ctypes.c_int32 * 9)()
    lib().oq_color_matrix(space, int(to_ycbcr), m)
    return [list(m[0:3]), list(m[3:6]), list(m[6:9])]


def range_clip(plane, bd):
    """(number of samples above 2^bd - 1, the clipped plane)."""
    p = np.ascontiguousarray(plane, np.uint16).copy()
    h, w = p.shape
    n = lib().oq_range_clip(p.ctypes.data, w, h, bd)
    return int(n), p


def unpack_frame(raw, w, h, bps, cf):
    """xSeqBase::xUnpackFrame of one raw planar frame (bytes): (3, H, W) uint16, 4:4:4."""
    buf = np.frombuffer(raw, np.uint8)
    out = np.zeros((3, h, w), np.uint16)
    if lib().oq_unpack_frame(buf.ctypes.data, w, h, bps, cf, out.ctypes.data) != 0:
        raise ValueError("unsupported frame layout")
    return out
