"""Python access to the deterministic synthetic-picture generator (csrc/qmiv_synth.c).

The generator writes the same bytes on x86-64 and aarch64, so inputs regenerated on any
machine match the golden fixtures made elsewhere.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


class SynthParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("bitdepth", ctypes.c_int32),
                ("seed", ctypes.c_uint32), ("shift_seed", ctypes.c_uint32), ("frame", ctypes.c_int32),
                ("drift", ctypes.c_int32), ("holes", ctypes.c_int32), ("noise_sigma", ctypes.c_double),
                ("offset", ctypes.c_double * 3), ("nthreads", ctypes.c_int32)]


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.SYNTH):
            _build.build()
        lib = ctypes.CDLL(_build.SYNTH)
        lib.qs_generate_pair.argtypes = [ctypes.POINTER(SynthParams), ctypes.c_void_p, ctypes.c_void_p]
        lib.qs_generate_pair.restype = ctypes.c_int
        lib.qs_generate_float444.argtypes = [ctypes.POINTER(SynthParams), ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_double, ctypes.c_double]
        lib.qs_generate_float444.restype = ctypes.c_int
        _lib = lib
    return _lib


def seed_for(config, view, frame):
    """Seed of one picture of a workload: 0xC0FFEE + config*1000 + view*100 + frame."""
    return (0xC0FFEE + config * 1000 + view * 100 + frame) & 0xFFFFFFFF


def pair420(width, height, bitdepth=8, seed=1, noise_sigma=2.0, offset=(3.0, -2.0, 1.0), holes=False,
            drift=False, shift_seed=0, frame=0, nthreads=None, out=None):
    """Reference and tested 4:2:0 pictures as two flat uint16 arrays (Y, then Cb, then Cr).

    noise_sigma and offset are in 8-bit units and scale with 2**(bitdepth-8)."""
    n = width * height + 2 * (width // 2) * (height // 2)
    if out is None:
        ref = np.empty(n, np.uint16)
        tst = np.empty(n, np.uint16)
    else:
        ref, tst = out
    p = SynthParams(width, height, bitdepth, seed, shift_seed, frame, int(drift), int(holes), noise_sigma,
                    (ctypes.c_double * 3)(*offset), nthreads or min(16, os.cpu_count() or 1))
    if _load().qs_generate_pair(ctypes.byref(p), ref.ctypes.data, tst.ctypes.data) != 0:
        raise ValueError("unsupported synthetic picture %dx%d@%d" % (width, height, bitdepth))
    return ref, tst


def split420(flat, width, height):
    """Views (Y, Cb, Cr) of a flat 4:2:0 array."""
    a = width * height
    ca = (width // 2) * (height // 2)
    return (flat[:a].reshape(height, width), flat[a:a + ca].reshape(height // 2, width // 2),
            flat[a + ca:a + 2 * ca].reshape(height // 2, width // 2))


def float444(width, height, seed=1, sigma=0.02, off_range=0.02):
    """Reference and tested 4:4:4 float32 pictures in [0,1] (3, H, W) each."""
    ref = np.empty((3, height, width), np.float32)
    tst = np.empty((3, height, width), np.float32)
    p = SynthParams(width, height, 8, seed, 0, 0, 0, 0, 0.0, (ctypes.c_double * 3)(0, 0, 0), 1)
    if _load().qs_generate_float444(ctypes.byref(p), ref.ctypes.data, tst.ctypes.data, sigma, off_range) != 0:
        raise ValueError("unsupported synthetic picture")
    return ref, tst
