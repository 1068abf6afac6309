"""Masked GCD / PSNR / WS-PSNR / IV-PSNR on the GPU (qmiv_calc_frame_masked) against the masked
golden cases of the reference (tests/golden/masked.json) and against the oracle's masked
restatement on further cases. Bar: bit-exact GCD and non-masked count, PSNR family within
1e-10 dB."""
import json
import os

import numpy as np
import pytest

from ivpsnr_gb300 import synth

from .golden.make_golden import make_mask

pytestmark = pytest.mark.gpu
DB_TOL = 1e-10
MASKED = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "masked.json")))


def _planes(flat, w, h, dtype):
    return [np.ascontiguousarray(p.astype(dtype)) for p in synth.split420(flat, w, h)]


def _check(g, e):
    assert g["gcd_r2t"][:3] == e["gcd"]
    np.testing.assert_allclose(g["psnr"][:3], e["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(g["wspsnr"][:3], e["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(g[k] - e[k]) <= DB_TOL, (k, g[k], e[k])


@pytest.mark.parametrize("case", MASKED["cases"], ids=[c["name"] for c in MASKED["cases"]])
def test_masked_matches_reference_golden(gpu_lib, case):
    w, h, bd = case["w"], case["h"], case["bd"]
    ref, tst = synth.pair420(w, h, bd, seed=case["seed"], **dict(case["gen"]))
    mask = make_mask(w, h, case["seed"], case["mask"]).astype(np.uint8)
    o = case["opts"]
    dt = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, search_range=o.get("sr", 2), use_ws=o.get("erp", False),
                           lat_deg=o.get("lat", 180)) as P:
        g = P.calc_frame_masked(gpu_lib.make_pic(_planes(ref, w, h, dt), bd), gpu_lib.make_pic(_planes(tst, w, h, dt), bd),
                                mask, case["mask_bd"])
    _check(g, case["expected"])


CASES = [  # w, h, bd, seed, holes, mask kind, mask dtype / bit depth, device inputs, 4:4:4, erp
    (200, 120, 10, 401, True, "ellipses", np.uint8, 8, False, False, False),
    (96, 80, 12, 402, False, "graded", np.uint16, 10, True, False, False),
    (128, 64, 8, 403, False, "graded", np.uint8, 8, True, True, False),
    (256, 128, 10, 404, True, "ellipses", np.uint16, 16, False, False, True),
]


@pytest.mark.parametrize("w,h,bd,seed,holes,kind,mdt,mbd,dev,cf444,erp", CASES)
def test_masked_matches_oracle(gpu_lib, oq, w, h, bd, seed, holes, kind, mdt, mbd, dev, cf444, erp):
    import torch
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=holes)
    mask = make_mask(w, h, seed, kind).astype(np.int64)
    if mbd > 8:  # spread the 8-bit pattern over the wider range
        mask = mask * ((1 << mbd) - 1) // 255
    mask = mask.astype(mdt)
    p0 = oq.upsample420(synth.split420(ref, w, h), w, h)
    p1 = oq.upsample420(synth.split420(tst, w, h), w, h)
    want = oq.masked(p0, p1, mask, bd, mask_bd=mbd, use_ws=erp, nthreads=8)
    dt = np.uint8 if bd == 8 else np.uint16
    if cf444:
        a, b, cf = [np.ascontiguousarray(p.astype(dt)) for p in p0], [np.ascontiguousarray(p.astype(dt)) for p in p1], gpu_lib.CF444
    else:
        a, b, cf = _planes(ref, w, h, dt), _planes(tst, w, h, dt), gpu_lib.CF420
    m = mask
    if dev:
        a = [torch.from_numpy(x).cuda() for x in a]
        b = [torch.from_numpy(x).cuda() for x in b]
        m = torch.from_numpy(mask.view(np.int16) if mdt == np.uint16 else mask).cuda()
    with gpu_lib.Processor(w, h, use_ws=erp) as P:
        g = P.calc_frame_masked(gpu_lib.make_pic(a, bd, cf), gpu_lib.make_pic(b, bd, cf), m, mbd)
    _check(g, want)
    assert g["exact"][:3] == want["exact"]


def test_masked_exact_components_and_rejections(gpu_lib, oq):
    w, h, bd = 64, 48, 10
    ref, _ = synth.pair420(w, h, bd, seed=7)
    p = _planes(ref, w, h, np.uint16)
    q = [x.copy() for x in p]
    q[2][3, 4] += 5  # only Cr differs
    mask = make_mask(w, h, 7, "ellipses").astype(np.uint8)
    want = oq.masked(oq.upsample420(p, w, h), oq.upsample420(q, w, h), mask, bd, mask_bd=8)
    with gpu_lib.Processor(w, h) as P:
        g = P.calc_frame_masked(gpu_lib.make_pic(p, bd), gpu_lib.make_pic(q, bd), mask, 8)
        _check(g, want)
        assert g["exact"][:3] == [1, 1, 0]
        with pytest.raises(gpu_lib.QmivError):
            P.calc_frame_masked(gpu_lib.make_pic(p, bd), gpu_lib.make_pic(q, bd), mask, 8, gpu_lib.M_SSIM)
        with pytest.raises(gpu_lib.QmivError):
            P.calc_frame_masked(gpu_lib.make_pic(p, bd), gpu_lib.make_pic(q, bd), np.ascontiguousarray(mask[:, :10]), 8)


@pytest.mark.parametrize("sr,bd,w_search", [(0, 10, (4, 1, 1)), (1, 10, (4, 1, 1)), (3, 8, (4, 1, 1)),
                                            (4, 10, (4, 1, 1)), (6, 10, (4, 1, 1)), (16, 10, (2, 1, 3)),
                                            (2, 14, (8, 1, 1)), (5, 14, (8, 1, 1))])
def test_masked_search_ranges_and_wide_costs(gpu_lib, oq, sr, bd, w_search):
    """Every search-range specialisation of the tiled masked search (1-4 compiled, others at run
    time, 16 the largest halo) and the 64-bit cost form, taken when the largest possible cost
    (14-bit samples, luma weight 8) does not fit 31 bits; the synthetic pairs' actual costs stay
    small, so the oracle's 32-bit costs are exact there."""
    w, h = 112, 72
    ref, tst = synth.pair420(w, h, bd, seed=500 + sr + bd, holes=True)
    mask = make_mask(w, h, 500 + sr, "ellipses").astype(np.uint8)
    p0 = oq.upsample420(synth.split420(ref, w, h), w, h)
    p1 = oq.upsample420(synth.split420(tst, w, h), w, h)
    want = oq.masked(p0, p1, mask, bd, mask_bd=8, search_range=sr, w_search=w_search, nthreads=8)
    dt = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, search_range=sr, cmp_w_search=w_search) as P:
        g = P.calc_frame_masked(gpu_lib.make_pic(_planes(ref, w, h, dt), bd), gpu_lib.make_pic(_planes(tst, w, h, dt), bd),
                                mask, 8)
    _check(g, want)
