"""qmiv_psnr_static (no handle, no allocation, static device scratch) against the handle-based
PSNR path, through the C ABI. Collected last so that it also runs after every other GPU test.

Bar: bit-exact GCD, exact flags and PSNR values (the same per-row integer sums and the same
FP64 finalisation); the doubles are compared with a 1e-12 tolerance."""
import ctypes

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _host_planes(flat, w, h, dtype, cf444=False):
    if cf444:
        from oracle.oracle import upsample420
        planes = upsample420(synth.split420(flat, w, h), w, h)
    else:
        planes = synth.split420(flat, w, h)
    return [np.ascontiguousarray(p.astype(dtype)) for p in planes]


def _device_planes(flat, w, h, dtype, cf444=False):
    return _to_device(_host_planes(flat, w, h, dtype, cf444))


def _to_device(planes):
    import torch
    return [torch.from_numpy(p).cuda() for p in planes]


def _static(lib, a, b, opts=None):
    from ivpsnr_gb300 import _abi
    r = _abi.FrameResult()
    _abi.check(lib.qmiv_psnr_static(ctypes.byref(a), ctypes.byref(b), ctypes.byref(opts) if opts else None,
                                    ctypes.byref(r), None), "qmiv_psnr_static")
    return r.to_dict()


CASES = [
    (1920, 1080, 8, 11, False, False),
    (640, 360, 10, 12, True, False),
    (130, 66, 12, 13, False, True),
    (2, 2, 10, 14, False, False),
]


@pytest.mark.parametrize("w,h,bd,seed,holes,cf444", CASES)
def test_static_psnr_matches_handle_path(gpu_lib, w, h, bd, seed, holes, cf444):
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=holes)
    dtype = np.uint8 if bd == 8 else np.uint16
    d0 = _device_planes(ref, w, h, dtype, cf444)
    d1 = _device_planes(tst, w, h, dtype, cf444)
    cf = gpu_lib.CF444 if cf444 else gpu_lib.CF420
    a, b = gpu_lib.make_pic(d0, bd, cf), gpu_lib.make_pic(d1, bd, cf)
    with gpu_lib.Processor(w, h) as P:
        want = P.calc_frame(a, b, gpu_lib.M_PSNR)
    for _ in range(2):  # two calls in a row: the counter and the result are reset each call
        got = _static(gpu_lib._abi.load(), a, b)
        assert got["gcd_r2t"] == want["gcd_r2t"]
        assert got["exact"] == want["exact"]
        np.testing.assert_allclose(got["psnr"], want["psnr"], rtol=0, atol=TOL)
        assert abs(got["psnr_pic"] - want["psnr_pic"]) <= TOL
        assert got["ivpsnr"] == 0.0 and got["ssim"] == [0.0] * 4


def test_static_psnr_options_and_exact_components(gpu_lib):
    w, h, bd = 256, 128, 10
    ref, _ = synth.pair420(w, h, bd, seed=21)
    h0 = _host_planes(ref, w, h, np.uint16)
    h1 = [p.copy() for p in h0]
    h1[1][0, 0] = (h1[1][0, 0] + 1) % 1024  # only Cb differs: Y and Cr are exact
    d0, d1 = _to_device(h0), _to_device(h1)
    a, b = gpu_lib.make_pic(d0, bd), gpu_lib.make_pic(d1, bd)
    lib = gpu_lib._abi.load()
    for fake in (1, 0):
        opts = gpu_lib.default_options(fake_exact=fake, unnoticeable=(0.0, 0.0, 0.0))
        with gpu_lib.Processor(w, h, fake_exact=fake, unnoticeable=(0.0, 0.0, 0.0)) as P:
            want = P.calc_frame(a, b, gpu_lib.M_PSNR)
        for _ in range(2):
            got = _static(lib, a, b, opts)
            assert got["exact"][:3] == [1, 0, 1] == want["exact"][:3]
            assert got["gcd_r2t"] == want["gcd_r2t"]
            for c in range(3):
                assert got["psnr"][c] == want["psnr"][c] or abs(got["psnr"][c] - want["psnr"][c]) <= TOL


def test_static_psnr_rejects_what_it_cannot_hold(gpu_lib):
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    w, h = 64, 8194
    d = _to_device([np.zeros((h >> s, w >> s), np.uint16) for s in (0, 1, 1)])
    a = gpu_lib.make_pic(d, 10)
    r = _abi.FrameResult()
    assert lib.qmiv_psnr_static(ctypes.byref(a), ctypes.byref(a), None, ctypes.byref(r), None) == _abi.QMIV_TOO_LARGE
    assert b"8192" in lib.qmiv_last_error()
    # a row wider than 65536 samples would overflow the kernel's 32-bit per-row difference sums
    w, h = 65538, 2
    d = _to_device([np.zeros((h >> s, w >> s), np.uint16) for s in (0, 1, 1)])
    a = gpu_lib.make_pic(d, 14)
    assert lib.qmiv_psnr_static(ctypes.byref(a), ctypes.byref(a), None, ctypes.byref(r), None) == _abi.QMIV_TOO_LARGE
    assert b"65536" in lib.qmiv_last_error()
    ref, tst = synth.pair420(64, 32, 10, seed=5)
    host = gpu_lib.make_pic([np.ascontiguousarray(p) for p in synth.split420(ref, 64, 32)], 10)
    assert lib.qmiv_psnr_static(ctypes.byref(host), ctypes.byref(host), None, ctypes.byref(r), None) == _abi.QMIV_BAD_ARG
    assert lib.qmiv_psnr_static(None, ctypes.byref(host), None, ctypes.byref(r), None) == _abi.QMIV_BAD_ARG
