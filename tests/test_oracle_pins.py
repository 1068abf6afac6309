"""CPU tests: the oracle against the reference's published values, its golden vectors and
the closed-form expectations of the reference's own core unit tests.

These run without a GPU. Tests that need the reference sources (or the reference build in
oracle/_ref) skip when those are absent.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from ivpsnr_gb300 import synth

from .conftest import ROOT
from .golden import fencing_io

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "cases.json")))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "qmiv_ref_harness")
DB_TOL = 1e-10
SSIM_TOL = 1e-12  # oracle vs reference are both FP64 (the x86-64-v4 build contracts some FMAs)


def _pics(case):
    gen = dict(case["gen"])
    if "offset" in gen:
        gen["offset"] = tuple(gen["offset"])
    ref, tst = synth.pair420(case["w"], case["h"], case["bd"], seed=case["seed"], **gen)
    return ref, tst


def _444(flat, w, h):
    from oracle.oracle import upsample420
    return upsample420(synth.split420(flat, w, h), w, h)


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_oracle_matches_golden(oq, case):
    import hashlib
    w, h, bd = case["w"], case["h"], case["bd"]
    ref, tst = _pics(case)
    hh = hashlib.md5()
    hh.update(ref.tobytes())
    hh.update(tst.tobytes())
    assert hh.hexdigest() == case["input_md5"], "synthetic generator is not reproducing the fixture's bytes"
    p0, p1 = _444(ref, w, h), _444(tst, w, h)
    o = case["opts"]
    do_ssim = "ssim" in case["expected"]
    r = oq.frame(p0, p1, bd, do_ssim, search_range=o.get("sr", 2), use_ws=o.get("erp", False),
                 lat_range_deg=o.get("lat", 180), nthreads=8)
    e = case["expected"]
    assert r["gcd"] == e["gcd"]
    assert r["exact"] == e["exact"]
    assert r["sse_r2t"] == e["sse_r2t"] and r["sse_t2r"] == e["sse_t2r"]
    np.testing.assert_allclose(r["psnr"], e["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(r["wspsnr"], e["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL
    assert abs(e["ivpsnr"] - e["ivpsnr_planar"]) <= DB_TOL  # interleaved SSE path == planar path
    if do_ssim:
        np.testing.assert_allclose(r["ssim"], e["ssim"], rtol=0, atol=SSIM_TOL)
        np.testing.assert_allclose(r["msssim"], e["msssim"], rtol=0, atol=SSIM_TOL)
        for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
            assert abs(r[k] - e[k]) <= SSIM_TOL
    # CPS argmin maps and shift-compensated pictures, bit-exact
    g = e["gcd"]
    sr = o.get("sr", 2)
    _, am0, _, scp1 = oq.cps_dir(p0, p1, bd, g, sr)
    _, am1, _, scp0 = oq.cps_dir(p1, p0, bd, [-x for x in g], sr)
    hh = hashlib.md5()
    hh.update(am0.tobytes())
    hh.update(am1.tobytes())
    assert hh.hexdigest() == case["cps_md5"]
    hh = hashlib.md5()
    hh.update(scp0.tobytes())
    hh.update(scp1.tobytes())
    assert hh.hexdigest() == case["scp_md5"]


# ---- the reference's published example values (example/README.md:44-47,67-69) --------------
PUBLISHED = [
    ("Fencing_v8_origJpgCompressed_1920x1080_yuv420p.yuv", 34.3362, 39.1335),
    ("Fencing_v8_synthesized_1920x1080_yuv420p.yuv", 34.0128, 44.3555),
]


def _load_example(name, w=1920, h=1080):
    """One of the reference's example pictures (committed compressed under tests/golden/fencing/)."""
    key = name.split("_")[2]
    return _444(fencing_io.flat(key), w, h)


@pytest.fixture(scope="module")
def example_dir(tmp_path_factory):
    """The example pictures as the reference's files, for the reference build's harness."""
    d = tmp_path_factory.mktemp("example")
    for key in ("original", "origJpgCompressed", "synthesized", "objectsMask"):
        fencing_io.write(key, str(d / ("Fencing_v8_%s_1920x1080_yuv420p.yuv" % key)))
    return str(d)


@pytest.mark.parametrize("name,psnr_y,ivpsnr", PUBLISHED)
def test_oracle_reproduces_published_example(oq, name, psnr_y, ivpsnr):
    p0 = _load_example("Fencing_v8_original_1920x1080_yuv420p.yuv")
    p1 = _load_example(name)
    r = oq.frame(p0, p1, 8, False, nthreads=8)
    assert round(r["psnr"][0], 4) == psnr_y
    assert round(r["ivpsnr"], 4) == ivpsnr


def test_oracle_reproduces_published_masked_example(oq):
    p0 = _load_example("Fencing_v8_original_1920x1080_yuv420p.yuv")
    p1 = _load_example("Fencing_v8_synthesized_1920x1080_yuv420p.yuv")
    m = _load_example("Fencing_v8_objectsMask_1920x1080_yuv420p.yuv")[0]
    r = oq.masked(p0, p1, m, 8, mask_bd=8, nthreads=8)
    assert round(r["psnr"][0], 4) == 39.5414
    assert round(r["ivpsnr"], 4) == 50.7716


@pytest.mark.skipif(not os.path.exists(HARNESS), reason="reference build not present")
def test_oracle_matches_reference_on_example_full_precision(oq, example_dir):
    a = os.path.join(example_dir, "Fencing_v8_original_1920x1080_yuv420p.yuv")
    b = os.path.join(example_dir, "Fencing_v8_origJpgCompressed_1920x1080_yuv420p.yuv")
    e = json.loads(subprocess.check_output([HARNESS, "-w", "1920", "-h", "1080", "-bd", "8", "-cf", "420",
                                            "-i0", a, "-i1", b, "-nth", "8"]).decode().splitlines()[0])
    r = oq.frame(_load_example(os.path.basename(a)), _load_example(os.path.basename(b)), 8, True, nthreads=8)
    assert r["gcd"] == e["gcd"] and r["sse_r2t"] == e["sse_r2t"] and r["sse_t2r"] == e["sse_t2r"]
    assert abs(r["ivpsnr"] - e["ivpsnr"]) <= DB_TOL
    np.testing.assert_allclose(r["ssim"], e["ssim"], atol=SSIM_TOL)
    assert abs(r["ivssim"] - e["ivssim"]) <= SSIM_TOL


@pytest.mark.skipif(not os.path.exists(HARNESS), reason="reference build not present")
def test_oracle_matches_reference_masked(oq, example_dir):
    a = os.path.join(example_dir, "Fencing_v8_original_1920x1080_yuv420p.yuv")
    b = os.path.join(example_dir, "Fencing_v8_synthesized_1920x1080_yuv420p.yuv")
    mk = os.path.join(example_dir, "Fencing_v8_objectsMask_1920x1080_yuv420p.yuv")
    e = json.loads(subprocess.check_output([HARNESS, "-w", "1920", "-h", "1080", "-bd", "8", "-cf", "420",
                                            "-i0", a, "-i1", b, "-im", mk, "-nth", "8"]).decode().splitlines()[0])
    r = oq.masked(_load_example(os.path.basename(a)), _load_example(os.path.basename(b)),
                  _load_example(os.path.basename(mk))[0], 8, mask_bd=8, nthreads=8)
    assert r["nnm"] == e["nnm"] and r["gcd"] == e["gcd"]
    np.testing.assert_allclose(r["psnr"], e["psnr"], atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL


# ---- the window table ------------------------------------------------------------------------
def test_ssim_table_equals_reference_constants(oq):
    # the reference's c_FilterF (xStructSimConsts.h:31-44), recorded by tests/golden/make_golden.py
    doc = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ssim_window.json")))
    vals = np.array(doc["values"], np.float32).reshape(11, 11)
    np.testing.assert_array_equal(oq.ssim_table(0), vals)


def test_oracle_matches_reference_build_on_example_fixture(oq):
    """Every value the reference build gave on the example pictures (tests/golden/fencing.json)."""
    for case in fencing_io.FIXTURE["cases"]:
        if "mask" in case:
            continue
        e = case["expected"]
        p0 = _444(fencing_io.flat(case["pic0"]), 1920, 1080)
        p1 = _444(fencing_io.flat(case["pic1"]), 1920, 1080)
        r = oq.frame(p0, p1, 8, True, nthreads=8)
        assert r["gcd"] == e["gcd"] and r["sse_r2t"] == e["sse_r2t"] and r["sse_t2r"] == e["sse_t2r"]
        np.testing.assert_allclose(r["psnr"], e["psnr"], atol=DB_TOL)
        for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
            assert abs(r[k] - e[k]) <= DB_TOL
        np.testing.assert_allclose(r["ssim"], e["ssim"], atol=SSIM_TOL)
        np.testing.assert_allclose(r["msssim"], e["msssim"], atol=SSIM_TOL)
        for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
            assert abs(r[k] - e[k]) <= SSIM_TOL


# ---- closed-form expectations restated from the reference's core unit tests -------------------
@pytest.mark.parametrize("v", [0.0, 0.01, 0.1, 0.9, 0.99, 1.0])
def test_kbns_known_sums(oq, v):
    # libs/pmbb-core/test/test-core-xMathUtils.cpp:50-100: N copies of V sum to exactly N*V
    for i in range(0, 16):
        n = 1 << i
        assert oq.kbns(np.full(n, v)) == n * v


@pytest.mark.parametrize("size,bd", [(127, 8), (128, 10), (255, 14), (513, 12)])
def test_distortion_constant_planes(oq, size, bd):
    # libs/pmbb-core/test/test-core-xDistortion.cpp:27-140: planes c-1, c, c+1 give SD and SSD of
    # +-Area and Area; extremes give Max^2 * Area
    c = (1 << bd) // 2
    w = h = size if size % 2 == 0 else size + 1
    area = w * h
    mid = np.full((3, h, w), c, np.uint16)
    up = np.full((3, h, w), c + 1, np.uint16)
    lo = np.full((3, h, w), 0, np.uint16)
    hi = np.full((3, h, w), (1 << bd) - 1, np.uint16)
    r = oq.frame(mid, up, bd, False)
    fake = 10 * np.log10(area * ((1 << bd) - 1) ** 2)
    np.testing.assert_allclose(r["psnr"], [10 * np.log10(area * ((1 << bd) - 1) ** 2 / area)] * 3, atol=1e-12)
    r = oq.frame(lo, hi, bd, False)
    np.testing.assert_allclose(r["psnr"], [0.0] * 3, atol=1e-12)
    r = oq.frame(mid, mid, bd, False)
    assert r["exact"] == [1, 1, 1]
    np.testing.assert_allclose(r["psnr"], [fake] * 3, atol=1e-9)


def test_downsample_rounding(oq):
    # DownsampleHV (xPixelOpsSTD.cpp:50-67): (a+b+c+d+2)>>2, odd trailing row/column dropped
    rng = np.random.default_rng(666)
    a = rng.integers(0, 1024, (9, 13), dtype=np.uint16)
    d = oq.downsample(a)
    exp = ((a[0:8:2, 0:12:2].astype(int) + a[0:8:2, 1:13:2] + a[1:9:2, 0:12:2] + a[1:9:2, 1:13:2] + 2) >> 2)
    np.testing.assert_array_equal(d, exp)


def test_ws_weights_match_closed_form(oq):
    # xWeightedSpherically.cpp:13-29 for a full-latitude ERP picture: w_h = cos((h + 0.5 - H/2) pi / H)
    h = 64
    w, corr = oq.ws_weights(h, 180)
    np.testing.assert_allclose(w, np.cos((np.arange(h) + 0.5 - h / 2) * np.pi / h), atol=1e-15)
    assert abs(corr - h / w.sum()) < 1e-12


# ---- masked golden cases (reference harness with -im) ---------------------------------------
MASKED = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "masked.json")))


@pytest.mark.parametrize("case", MASKED["cases"], ids=[c["name"] for c in MASKED["cases"]])
def test_oracle_matches_masked_golden(oq, case):
    from tests.golden.make_golden import make_mask
    w, h, bd = case["w"], case["h"], case["bd"]
    gen = dict(case["gen"])
    ref, tst = synth.pair420(w, h, bd, seed=case["seed"], **gen)
    mask = make_mask(w, h, case["seed"], case["mask"])
    p0 = oq.upsample420(synth.split420(ref, w, h), w, h)
    p1 = oq.upsample420(synth.split420(tst, w, h), w, h)
    o = case["opts"]
    r = oq.masked(p0, p1, mask, bd, mask_bd=case["mask_bd"], use_ws=o.get("erp", False),
                  lat_range_deg=o.get("lat", 180), search_range=o.get("sr", 2), nthreads=8)
    e = case["expected"]
    assert r["nnm"] == e["nnm"] and r["gcd"] == e["gcd"]
    np.testing.assert_allclose(r["psnr"], e["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(r["wspsnr"], e["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(r[k] - e[k]) <= DB_TOL, k
