"""The corresponding-pixel search per pixel (qmiv_cps_maps through the C ABI): both directions'
argmin window indices against the reference's own maps (cps_md5 of tests/golden/cases.json, made by
oracle/ref_harness.cpp -dump through xCorrespPixelShift::xFindBestPixelWithinBlock) and against the
oracle's maps, and the per-row squared errors at the argmin against the oracle's rows
(xCorrespPixelShift::xCalcDistAsymmetricRow).

Bar: bit-exact (index and integer work)."""
import hashlib
import json
import os

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "cases.json")))


def _planes(flat, w, h, dtype=np.uint16):
    return [np.ascontiguousarray(p.astype(dtype)) for p in synth.split420(flat, w, h)]


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_cps_maps_match_reference_golden(gpu_lib, case):
    w, h, bd = case["w"], case["h"], case["bd"]
    gen = dict(case["gen"])
    if "offset" in gen:
        gen["offset"] = tuple(gen["offset"])
    ref, tst = synth.pair420(w, h, bd, seed=case["seed"], **gen)
    o = case["opts"]
    dtype = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, search_range=o.get("sr", 2), use_ws=o.get("erp", False), lat_deg=o.get("lat", 180)) as P:
        m0, m1, rows = P.cps_maps(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd))
    hh = hashlib.md5()
    hh.update(m0.astype(np.int8).tobytes())  # the harness writes int8 indices, R2T then T2R
    hh.update(m1.astype(np.int8).tobytes())
    assert hh.hexdigest() == case["cps_md5"]
    e = case["expected"]
    assert [int(v) for v in rows[0].sum(axis=0)] == e["sse_r2t"]
    assert [int(v) for v in rows[1].sum(axis=0)] == e["sse_t2r"]


def _oracle_dirs(oq, ref, tst, w, h, bd, sr, gcd=None):
    from oracle.oracle import upsample420
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    g = gcd if gcd is not None else oq.gcd(p0, p1, bd)
    r0, a0, _, _ = oq.cps_dir(p0, p1, bd, g, sr, nthreads=8)
    r1, a1, _, _ = oq.cps_dir(p1, p0, bd, [-x for x in g], sr, nthreads=8)
    return (a0, a1), (r0, r1), g


# (w, h, bd, seed, sr): the TMA kernels (ranges 1-4, 8 and 10 bits), ragged sizes, 14-bit samples
# (64-bit keys), and the generic kernel (0, 5, 8; indices above 127 compare as the oracle's int8)
MAP_CASES = [(1920, 1080, 10, synth.seed_for(1, 3, 0), 2), (352, 98, 8, 71, 2), (200, 100, 10, 72, 1),
             (256, 128, 10, 73, 3), (130, 66, 10, 74, 4), (96, 64, 14, 75, 2), (96, 64, 10, 76, 0),
             (120, 72, 10, 77, 5), (128, 80, 8, 78, 8), (2, 2, 8, 79, 2), (6, 4, 10, 80, 2)]


@pytest.mark.parametrize("w,h,bd,seed,sr", MAP_CASES)
def test_cps_maps_and_rows_match_oracle(gpu_lib, oq, w, h, bd, seed, sr):
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=True)
    (a0, a1), (r0, r1), g = _oracle_dirs(oq, ref, tst, w, h, bd, sr)
    dtype = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, search_range=sr) as P:
        m0, m1, rows = P.cps_maps(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd))
    np.testing.assert_array_equal(m0.astype(np.int8), a0)
    np.testing.assert_array_equal(m1.astype(np.int8), a1)
    np.testing.assert_array_equal(rows[0], r0)
    np.testing.assert_array_equal(rows[1], r1)
    if (2 * sr + 1) ** 2 <= 128:
        assert m0.min() >= 0 and m0.max() < (2 * sr + 1) ** 2


def test_cps_maps_device_outputs_and_given_gcd(gpu_lib, oq):
    """Device map outputs with a row pitch wider than the picture, and a caller-supplied GCD."""
    import ctypes
    import torch
    from ivpsnr_gb300 import _abi
    w, h, bd = 320, 180, 10
    ref, tst = synth.pair420(w, h, bd, seed=81, holes=True)
    gcd = [5, -3, 2]
    (a0, a1), (r0, r1), _ = _oracle_dirs(oq, ref, tst, w, h, bd, 2, gcd=gcd)
    d0 = torch.full((h, w + 40), -7, dtype=torch.int16, device="cuda")
    d1 = torch.full((h, w + 40), -7, dtype=torch.int16, device="cuda")
    rows = np.zeros((2, h, 3), np.uint64)
    with gpu_lib.Processor(w, h) as P:
        g = (ctypes.c_int32 * 4)(*gcd, 0)
        pa = gpu_lib.make_pic(_planes(ref, w, h), bd)
        pb = gpu_lib.make_pic(_planes(tst, w, h), bd)
        _abi.check(P.lib.qmiv_cps_maps(P.h, ctypes.byref(pa), ctypes.byref(pb), g, d0.data_ptr(), d1.data_ptr(),
                                       w + 40, 1, rows.ctypes.data, None), "qmiv_cps_maps")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d0[:, :w].cpu().numpy().astype(np.int8), a0)
    np.testing.assert_array_equal(d1[:, :w].cpu().numpy().astype(np.int8), a1)
    assert bool((d0[:, w:] == -7).all()) and bool((d1[:, w:] == -7).all())  # nothing written past the width
    np.testing.assert_array_equal(rows[0], r0)
    np.testing.assert_array_equal(rows[1], r1)
