"""GPU results against the golden vectors produced by the reference itself (tests/golden/cases.json):
GCD, exact-component flags and CPS squared-error sums bit-exact, the shift-compensated pictures
bit-exact (md5 of both pictures), PSNR-family dB within 1e-10."""
import hashlib
import json
import os

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "cases.json")))
DB_TOL = 1e-10


def _planes(flat, w, h, dtype):
    return [np.ascontiguousarray(p.astype(dtype)) for p in synth.split420(flat, w, h)]


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_gpu_matches_reference_golden(gpu_lib, case):
    w, h, bd = case["w"], case["h"], case["bd"]
    gen = dict(case["gen"])
    if "offset" in gen:
        gen["offset"] = tuple(gen["offset"])
    ref, tst = synth.pair420(w, h, bd, seed=case["seed"], **gen)
    hh = hashlib.md5()
    hh.update(ref.tobytes())
    hh.update(tst.tobytes())
    assert hh.hexdigest() == case["input_md5"]
    o = case["opts"]
    dtype = np.uint8 if bd == 8 else np.uint16
    pic0 = gpu_lib.make_pic(_planes(ref, w, h, dtype), bd)
    pic1 = gpu_lib.make_pic(_planes(tst, w, h, dtype), bd)
    with gpu_lib.Processor(w, h, search_range=o.get("sr", 2), use_ws=o.get("erp", False),
                           lat_deg=o.get("lat", 180)) as P:
        r = P.calc_frame(pic0, pic1, gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
        s0 = [np.zeros((h, w), np.uint16) for _ in range(3)]
        s1 = [np.zeros((h, w), np.uint16) for _ in range(3)]
        P.scp(pic0, pic1, s0, s1)
    e = case["expected"]
    assert r["status"] == 0
    assert r["gcd_r2t"][:3] == e["gcd"]
    assert r["exact"][:3] == e["exact"]
    assert r["sse_r2t"][:3] == e["sse_r2t"] and r["sse_t2r"][:3] == e["sse_t2r"]
    np.testing.assert_allclose(r["psnr"][:3], e["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(r["wspsnr"][:3], e["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL, (k, r[k], e[k])
    hh = hashlib.md5()
    for p in s0 + s1:
        hh.update(p.tobytes())
    assert hh.hexdigest() == case["scp_md5"]
