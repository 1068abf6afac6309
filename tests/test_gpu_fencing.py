"""The reference's example pictures (the first frame of view 8 of the Fencing sequence, 1920x1080
8-bit 4:2:0, committed under tests/golden/fencing/) through the C ABI: the values the reference
publishes for them (example/README.md:44-47,67-69, rounded to 4 decimals), and every value its own
build gives at full precision (tests/golden/fencing.json): GCD, CPS squared-error sums, argmin maps
and shift-compensated pictures bit-exact, PSNR-family dB within 1e-10, SSIM family within 1e-6."""
import hashlib

import numpy as np
import pytest

from ivpsnr_gb300 import synth

from .golden import fencing_io

pytestmark = pytest.mark.gpu
DB_TOL, SSIM_TOL = 1e-10, 1e-6
W, H = fencing_io.W, fencing_io.H

# example/README.md:46-47 (PSNR-Y, IV-PSNR) and :69 (masked, objects only)
PUBLISHED = {"origJpgCompressed": (34.3362, 39.1335), "synthesized": (34.0128, 44.3555)}
PUBLISHED_MASKED = (39.5414, 50.7716)


def _pic(gpu_lib, key):
    return gpu_lib.make_pic([np.ascontiguousarray(p.astype(np.uint8)) for p in synth.split420(fencing_io.flat(key), W, H)], 8)


CASES = [c for c in fencing_io.FIXTURE["cases"] if "mask" not in c]


@pytest.mark.parametrize("case", CASES, ids=[c["pic1"] for c in CASES])
def test_fencing_matches_published_and_reference_build(gpu_lib, case):
    e = case["expected"]
    p0, p1 = _pic(gpu_lib, case["pic0"]), _pic(gpu_lib, case["pic1"])
    with gpu_lib.Processor(W, H) as P:
        r = P.calc_frame(p0, p1, gpu_lib.M_ALL)
        m0, m1, _ = P.cps_maps(p0, p1)
        s0 = [np.zeros((H, W), np.uint16) for _ in range(3)]
        s1 = [np.zeros((H, W), np.uint16) for _ in range(3)]
        P.scp(p0, p1, s0, s1)
    psnr_y, ivpsnr = PUBLISHED[case["pic1"]]
    assert round(r["psnr"][0], 4) == psnr_y
    assert round(r["ivpsnr"], 4) == ivpsnr
    assert r["status"] == 0
    assert r["gcd_r2t"][:3] == e["gcd"] and r["exact"][:3] == e["exact"]
    assert r["sse_r2t"][:3] == e["sse_r2t"] and r["sse_t2r"][:3] == e["sse_t2r"]
    np.testing.assert_allclose(r["psnr"][:3], e["psnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL, k
    np.testing.assert_allclose(r["ssim"][:3], e["ssim"], rtol=0, atol=SSIM_TOL)
    np.testing.assert_allclose(r["msssim"][:3], e["msssim"], rtol=0, atol=SSIM_TOL)
    for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
        assert abs(r[k] - e[k]) <= SSIM_TOL, k
    hh = hashlib.md5()
    hh.update(m0.astype(np.int8).tobytes())
    hh.update(m1.astype(np.int8).tobytes())
    assert hh.hexdigest() == case["cps_md5"]
    hh = hashlib.md5()
    for p in s0 + s1:
        hh.update(p.tobytes())
    assert hh.hexdigest() == case["scp_md5"]


def test_fencing_masked_matches_published_and_reference_build(gpu_lib):
    case = [c for c in fencing_io.FIXTURE["cases"] if "mask" in c][0]
    e = case["expected"]
    mask = np.ascontiguousarray(fencing_io.flat(case["mask"])[:W * H].reshape(H, W).astype(np.uint8))
    with gpu_lib.Processor(W, H) as P:
        r = P.calc_frame_masked(_pic(gpu_lib, case["pic0"]), _pic(gpu_lib, case["pic1"]), mask, 8,
                                gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
    assert round(r["psnr"][0], 4) == PUBLISHED_MASKED[0]
    assert round(r["ivpsnr"], 4) == PUBLISHED_MASKED[1]
    assert r["gcd_r2t"][:3] == e["gcd"]
    np.testing.assert_allclose(r["psnr"][:3], e["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(r["wspsnr"][:3], e["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL, k
