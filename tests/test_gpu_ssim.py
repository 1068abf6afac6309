"""GPU parity of SSIM, MS-SSIM and IV-SSIM against the FP64 CPU oracle, through the C ABI.

Bar: every SSIM-family value within 1e-6 of the FP64 oracle (the GPU computes window
statistics in FP32 on tile-centred samples; picture sums in FP64)."""
import ctypes
import json
import os

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
TOL = 1e-6
SSIM_METRICS = None


def _planes(flat, w, h, dtype=np.uint16):
    return [np.ascontiguousarray(p.astype(dtype)) for p in synth.split420(flat, w, h)]


def _oracle(oq, ref, tst, w, h, bd, window=0, search_range=2):
    from oracle.oracle import upsample420
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    return oq.frame(p0, p1, bd, True, ssim_window=window, search_range=search_range, nthreads=8), p0, p1


def _cmp_ssim(g, o):
    np.testing.assert_allclose(g["ssim"][:3], o["ssim"], rtol=0, atol=TOL)
    np.testing.assert_allclose(g["msssim"][:3], o["msssim"], rtol=0, atol=TOL)
    for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
        assert abs(g[k] - o[k]) <= TOL, (k, g[k], o[k])
    w = np.array([4, 1, 1]) / 6.0
    assert abs(g["ssim_pic"] - float(np.dot(w, o["ssim"]))) <= TOL


CASES = [
    (1920, 1080, 8, synth.seed_for(0, 0, 0), False, 0),
    (1920, 1080, 10, synth.seed_for(2, 0, 0), True, 0),
    (640, 360, 10, 101, True, 1),
    (1920, 1080, 12, 106, True, 1),    # 12-bit at full HD, Gaussian window
    (1920, 1080, 14, 107, True, 0),    # 14-bit: the 64-bit-key search variants
    (130, 66, 8, 102, False, 0),
    (96, 64, 12, 103, False, 0),
    (64, 48, 14, 104, False, 1),
    (16, 16, 8, 105, False, 0),
]


@pytest.mark.parametrize("w,h,bd,seed,holes,window", CASES)
def test_frame_ssim_family(gpu_lib, oq, w, h, bd, seed, holes, window):
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=holes)
    o, _, _ = _oracle(oq, ref, tst, w, h, bd, window)
    dtype = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, ssim_window=window) as P:
        g = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd),
                         gpu_lib.M_ALL)
    _cmp_ssim(g, o)
    assert g["gcd_r2t"][:3] == o["gcd"]
    assert abs(g["ivpsnr"] - o["ivpsnr"]) <= 1e-10


@pytest.mark.parametrize("sr", [0, 6])
def test_ivssim_with_generic_search(gpu_lib, oq, sr):
    """IV-SSIM from shift-compensated pictures of the generic search kernel (search ranges the
    specialised kernels do not take)."""
    w, h, bd = 144, 96, 10
    ref, tst = synth.pair420(w, h, bd, seed=140 + sr, holes=True)
    o, _, _ = _oracle(oq, ref, tst, w, h, bd, search_range=sr)
    with gpu_lib.Processor(w, h, search_range=sr) as P:
        g = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h), bd), gpu_lib.make_pic(_planes(tst, w, h), bd), gpu_lib.M_ALL)
    _cmp_ssim(g, o)
    assert g["gcd_r2t"][:3] == o["gcd"]
    assert abs(g["ivpsnr"] - o["ivpsnr"]) <= 1e-10


def test_ssim_444_and_tiny(gpu_lib, oq):
    from oracle.oracle import upsample420
    w, h, bd = 100, 60, 10
    ref, tst = synth.pair420(w, h, bd, seed=7)
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    o = oq.frame(p0, p1, bd, True)
    with gpu_lib.Processor(w, h) as P:
        g = P.calc_frame(gpu_lib.make_pic(list(p0), bd, gpu_lib.CF444), gpu_lib.make_pic(list(p1), bd, gpu_lib.CF444), gpu_lib.M_ALL)
    _cmp_ssim(g, o)
    # smaller than the window: SSIM is 0 (no valid pixel); MS-SSIM is refused below 16x16
    w, h = 10, 8
    ref, tst = synth.pair420(w, h, 8, seed=8)
    with gpu_lib.Processor(w, h) as P:
        g = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h, np.uint8), 8), gpu_lib.make_pic(_planes(tst, w, h, np.uint8), 8),
                         gpu_lib.M_SSIM | gpu_lib.M_IVSSIM)
        assert g["ssim"][:3] == [0.0, 0.0, 0.0] and g["ivssim"] == 0.0
        with pytest.raises(gpu_lib.QmivError):
            P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h, np.uint8), 8), gpu_lib.make_pic(_planes(tst, w, h, np.uint8), 8),
                         gpu_lib.M_MSSSIM)


def test_msssim_level_without_window_columns(gpu_lib, oq):
    """96x320: MS-SSIM level 4 is 6x20, rows but no window columns; those rows add nothing (the
    oracle's MS-SSIM is 0), also after a larger call has left other values in the handle's
    per-tile sums."""
    w, h, bd = 96, 320, 10
    ref, tst = synth.pair420(w, h, bd, seed=11, holes=True)
    o, _, _ = _oracle(oq, ref, tst, w, h, bd)
    assert o["msssim"] == [0.0, 0.0, 0.0]
    big_ref, big_tst = synth.pair420(256, 320, bd, seed=12, holes=True)
    with gpu_lib.Processor(256, 320) as P:
        P.calc_frame(gpu_lib.make_pic(_planes(big_ref, 256, 320), bd), gpu_lib.make_pic(_planes(big_tst, 256, 320), bd),
                     gpu_lib.M_ALL)
        g = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h), bd), gpu_lib.make_pic(_planes(tst, w, h), bd), gpu_lib.M_ALL)
    _cmp_ssim(g, o)


def test_standalone_ssim_call(gpu_lib, oq):
    from ivpsnr_gb300 import _abi
    w, h, bd = 256, 144, 10
    ref, tst = synth.pair420(w, h, bd, seed=9, holes=True)
    o, p0, p1 = _oracle(oq, ref, tst, w, h, bd)
    with gpu_lib.Processor(w, h) as P:
        out = (ctypes.c_double * 4)()
        a = gpu_lib.make_pic(_planes(ref, w, h), bd)
        b = gpu_lib.make_pic(_planes(tst, w, h), bd)
        _abi.check(P.lib.qmiv_ssim(P.h, ctypes.byref(a), ctypes.byref(b), 0, out, None), "qmiv_ssim")
    cs = [oq.ssim_plane(p0[c], p1[c], bd, False, 0) for c in range(3)]
    np.testing.assert_allclose(list(out)[:3], cs, atol=TOL)


def test_batch_with_ssim_metrics(gpu_lib, oq):
    import torch
    from ivpsnr_gb300 import _abi
    sizes = [(320, 180, 10, True), (256, 128, 8, False), (192, 96, 10, False)]
    jobs, keep, oras = [], [], []
    for i, (w, h, bd, holes) in enumerate(sizes):
        ref, tst = synth.pair420(w, h, bd, seed=200 + i, holes=holes)
        o, _, _ = _oracle(oq, ref, tst, w, h, bd)
        oras.append(o)
        dtype = np.uint8 if bd == 8 else np.uint16
        d0 = [torch.from_numpy(p).cuda() for p in _planes(ref, w, h, dtype)]
        d1 = [torch.from_numpy(p).cuda() for p in _planes(tst, w, h, dtype)]
        keep += [d0, d1]
        j = _abi.Job()
        j.pic0 = gpu_lib.make_pic(d0, bd)
        j.pic1 = gpu_lib.make_pic(d1, bd)
        j.metrics = gpu_lib.M_ALL
        jobs.append(j)
    rs = ctypes.sizeof(_abi.FrameResult)
    res = torch.zeros(len(jobs) * rs, dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(320, 180, max_jobs=len(jobs)) as P:
        for _ in range(2):
            res.zero_()
            P.calc_batch(jobs, res.data_ptr())
            torch.cuda.synchronize()
            host = res.cpu().numpy().tobytes()
            for i, o in enumerate(oras):
                r = _abi.FrameResult.from_buffer_copy(host[i * rs:(i + 1) * rs]).to_dict()
                _cmp_ssim(r, o)
                assert abs(r["ivpsnr"] - o["ivpsnr"]) <= 1e-10


def test_sequence_average(gpu_lib, oq):
    w, h, bd = 128, 96, 10
    vals = []
    with gpu_lib.Processor(w, h) as P:
        for f in range(3):
            ref, tst = synth.pair420(w, h, bd, seed=300 + f)
            r = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h), bd), gpu_lib.make_pic(_planes(tst, w, h), bd), gpu_lib.M_ALL)
            vals.append(r)
        s = P.finish_sequence()
    assert s["num_frames"] == 3
    assert abs(s["ivssim"] - np.mean([v["ivssim"] for v in vals])) < 1e-12
    assert abs(s["ivpsnr"] - np.mean([v["ivpsnr"] for v in vals])) < 1e-12
    np.testing.assert_allclose(s["msssim"][:3], np.mean([v["msssim"][:3] for v in vals], axis=0), atol=1e-12)


GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "cases.json")))


@pytest.mark.parametrize("case", [c for c in GOLDEN["cases"] if "ssim" in c["expected"]],
                         ids=[c["name"] for c in GOLDEN["cases"] if "ssim" in c["expected"]])
def test_ssim_family_matches_reference_golden(gpu_lib, case):
    w, h, bd = case["w"], case["h"], case["bd"]
    gen = dict(case["gen"])
    if "offset" in gen:
        gen["offset"] = tuple(gen["offset"])
    ref, tst = synth.pair420(w, h, bd, seed=case["seed"], **gen)
    o = case["opts"]
    dtype = np.uint8 if bd == 8 else np.uint16
    with gpu_lib.Processor(w, h, search_range=o.get("sr", 2), use_ws=o.get("erp", False), lat_deg=o.get("lat", 180)) as P:
        g = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd),
                         gpu_lib.M_ALL)
    e = case["expected"]
    np.testing.assert_allclose(g["ssim"][:3], e["ssim"], atol=TOL)
    np.testing.assert_allclose(g["msssim"][:3], e["msssim"], atol=TOL)
    for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
        assert abs(g[k] - e[k]) <= TOL


@pytest.mark.parametrize("w,h,bd,cf444,window", [(320, 180, 10, False, 0), (256, 144, 8, False, 0),
                                                 (192, 128, 10, True, 0), (200, 120, 10, False, 1)])
def test_fused_staging_paths_agree(gpu_lib, oq, w, h, bd, cf444, window):
    """The fused SSIM kernel stages 16-byte aligned planes with bulk-tensor loads and other planes
    with plain loads; both must give identical values (they differ only in samples that feed no
    valid output). The unaligned copies sit 3 samples into rows 3 samples wider."""
    import torch
    from oracle.oracle import upsample420
    ref, tst = synth.pair420(w, h, bd, seed=300 + w, holes=True)
    dtype = np.uint8 if bd == 8 else np.uint16
    if cf444:
        p0 = [np.ascontiguousarray(p.astype(dtype)) for p in upsample420(synth.split420(ref, w, h), w, h)]
        p1 = [np.ascontiguousarray(p.astype(dtype)) for p in upsample420(synth.split420(tst, w, h), w, h)]
    else:
        p0, p1 = _planes(ref, w, h, dtype), _planes(tst, w, h, dtype)
    tview = lambda a: torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a)
    aligned = [[tview(p).cuda() for p in ps] for ps in (p0, p1)]
    def padded(p):
        buf = torch.zeros((p.shape[0], p.shape[1] + 3), dtype=tview(p).dtype, device="cuda")
        buf[:, 3:] = tview(p).cuda()
        return buf[:, 3:]
    unaligned = [[padded(p) for p in ps] for ps in (p0, p1)]
    cf = gpu_lib.CF444 if cf444 else gpu_lib.CF420
    with gpu_lib.Processor(w, h, ssim_window=window) as P:
        a = P.calc_frame(gpu_lib.make_pic(aligned[0], bd, cf), gpu_lib.make_pic(aligned[1], bd, cf), gpu_lib.M_ALL)
        b = P.calc_frame(gpu_lib.make_pic(unaligned[0], bd, cf), gpu_lib.make_pic(unaligned[1], bd, cf), gpu_lib.M_ALL)
    for k in ("ssim", "msssim", "ssim_pic", "msssim_pic", "ivssim", "ivssim_r2t", "ivssim_t2r", "ivpsnr", "psnr"):
        assert a[k] == b[k], (k, a[k], b[k])
    o = oq.frame(upsample420(synth.split420(ref, w, h), w, h), upsample420(synth.split420(tst, w, h), w, h), bd, True,
                 ssim_window=window, nthreads=8)
    _cmp_ssim(a, o)


# ---- the sizes the benchmarks time ---------------------------------------------------------------
@pytest.mark.parametrize("w,h,sr,ws,window,cfg", [(4096, 2048, 2, True, 0, 1), (7680, 3840, 4, True, 0, 4),
                                                  (4096, 2048, 2, False, 1, 1)])
def test_ssim_family_large_planes(gpu_lib, oq, w, h, sr, ws, window, cfg):
    """SSIM, MS-SSIM (five levels from the full picture) and IV-SSIM on device pictures of the ERP
    view size of the multiview workload and of the 8K sequence (search range 4), against the oracle
    (xSSIM.cpp:67-87,192-210): the persistent SSIM kernels' tile walks over large planes."""
    import torch
    from oracle.oracle import upsample420
    ref, tst = synth.pair420(w, h, 10, seed=synth.seed_for(cfg, 0, 0), holes=True)
    d0 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(ref, w, h)]
    d1 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(tst, w, h)]
    with gpu_lib.Processor(w, h, search_range=sr, use_ws=ws, ssim_window=window) as P:
        g = P.calc_frame(gpu_lib.make_pic(d0, 10), gpu_lib.make_pic(d1, 10), gpu_lib.M_ALL)
    o = oq.frame(upsample420(synth.split420(ref, w, h), w, h), upsample420(synth.split420(tst, w, h), w, h), 10, True,
                 use_ws=ws, search_range=sr, ssim_window=window, nthreads=16)
    _cmp_ssim(g, o)
    assert g["gcd_r2t"][:3] == o["gcd"]
    assert g["sse_r2t"][:3] == o["sse_r2t"] and g["sse_t2r"][:3] == o["sse_t2r"]
    assert abs(g["ivpsnr"] - o["ivpsnr"]) <= 1e-10


@pytest.mark.parametrize("window", [0, 1])
def test_ssim_sequence_of_17_drifting_frames(gpu_lib, oq, window):
    """The 17-frame SSIM workload (1920x1080 10-bit 4:2:0, block shifts drifting over time) in one
    batched call, each frame against the oracle, and the per-sequence means of the same frames
    measured one call per frame (xMetricStat::calcAvgMetric, xAppQMIV.h:256-260) against the
    compensated mean of the oracle's per-frame values."""
    import ctypes
    import torch
    from ivpsnr_gb300 import _abi
    from oracle.oracle import upsample420
    w, h, nf, bd = 1920, 1080, 17, 10
    jobs, keep, oras, pics = [], [], [], []
    for f in range(nf):
        ref, tst = synth.pair420(w, h, bd, seed=synth.seed_for(2, 0, f), drift=True, shift_seed=synth.seed_for(2, 0, 0),
                                 frame=f)
        oras.append(oq.frame(upsample420(synth.split420(ref, w, h), w, h), upsample420(synth.split420(tst, w, h), w, h),
                             bd, True, ssim_window=window, nthreads=16))
        d0 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(ref, w, h)]
        d1 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(tst, w, h)]
        keep += [d0, d1]
        j = _abi.Job()
        j.pic0 = gpu_lib.make_pic(d0, bd)
        j.pic1 = gpu_lib.make_pic(d1, bd)
        j.metrics = gpu_lib.M_ALL
        jobs.append(j)
        pics.append((j.pic0, j.pic1))
    rs = ctypes.sizeof(_abi.FrameResult)
    res = torch.zeros(nf * rs, dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(w, h, max_jobs=nf, ssim_window=window) as P:
        P.calc_batch(jobs, res.data_ptr())
        torch.cuda.synchronize()
        host = res.cpu().numpy().tobytes()
        for f, o in enumerate(oras):
            r = _abi.FrameResult.from_buffer_copy(host[f * rs:(f + 1) * rs]).to_dict()
            assert r["status"] == 0
            _cmp_ssim(r, o)
            assert r["gcd_r2t"][:3] == o["gcd"] and abs(r["ivpsnr"] - o["ivpsnr"]) <= 1e-10
        for p0, p1 in pics:
            P.calc_frame(p0, p1, gpu_lib.M_ALL)
        s = P.finish_sequence()
    assert s["num_frames"] == nf
    wv = np.array([4, 1, 1]) / 6.0
    assert abs(s["ivssim"] - oq.kbns([o["ivssim"] for o in oras]) / nf) <= TOL
    assert abs(s["ivpsnr"] - oq.kbns([o["ivpsnr"] for o in oras]) / nf) <= 1e-10
    for c in range(3):
        assert abs(s["ssim"][c] - oq.kbns([o["ssim"][c] for o in oras]) / nf) <= TOL
        assert abs(s["msssim"][c] - oq.kbns([o["msssim"][c] for o in oras]) / nf) <= TOL
    assert abs(s["ssim_pic"] - oq.kbns([float(np.dot(wv, o["ssim"])) for o in oras]) / nf) <= TOL
