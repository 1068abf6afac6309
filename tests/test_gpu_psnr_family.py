"""GPU parity of GCD, PSNR, WS-PSNR, the CPS search (per-component SSE sums, IV-PSNR) and the
shift-compensated pictures against the CPU oracle, through the C ABI.

Bars: integers (GCD, SSE sums, SCP samples) bit-exact; dB values within 1e-10.
"""
import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
DB_TOL = 1e-10


def _planes(flat, w, h, dtype=np.uint16):
    y, cb, cr = synth.split420(flat, w, h)
    return [np.ascontiguousarray(p.astype(dtype)) for p in (y, cb, cr)]


def _case(w, h, bd, seed, holes=False, **kw):
    sigma = kw.pop("sigma", 2.0)
    off = kw.pop("offset", (3.0, -2.0, 1.0))
    ref, tst = synth.pair420(w, h, bd, seed=seed, noise_sigma=sigma, offset=off, holes=holes)
    return ref, tst


def _oracle(oq, ref, tst, w, h, bd, **opts):
    from oracle.oracle import upsample420
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    o = dict(opts)
    if "cmp_w_search" in o:
        o["w_search"] = o.pop("cmp_w_search")
    if "cmp_w_avg" in o:
        o["w_avg"] = o.pop("cmp_w_avg")
    return oq.frame(p0, p1, bd, False, nthreads=8, **o), p0, p1


def _cmp(gpu, ora, ws=False):
    assert gpu["gcd_r2t"][:3] == ora["gcd"]
    assert gpu["exact"][:3] == ora["exact"]
    assert gpu["sse_r2t"][:3] == ora["sse_r2t"]
    assert gpu["sse_t2r"][:3] == ora["sse_t2r"]
    np.testing.assert_allclose(gpu["psnr"][:3], ora["psnr"], rtol=0, atol=DB_TOL)
    np.testing.assert_allclose(gpu["wspsnr"][:3], ora["wspsnr"], rtol=0, atol=DB_TOL)
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(gpu[k] - ora[k]) <= DB_TOL, (k, gpu[k], ora[k])


CASES = [
    # (w, h, bd, seed, holes, opts)
    (1920, 1080, 8, synth.seed_for(0, 0, 0), False, {}),
    (2048, 1088, 10, synth.seed_for(1, 9, 0), True, {}),
    (640, 360, 10, 77, True, {"use_ws": True}),
    (130, 66, 8, 5, False, {}),
    (66, 34, 10, 6, False, {"search_range": 1}),
    (200, 100, 10, 7, False, {"search_range": 3}),
    (256, 128, 10, 8, False, {"search_range": 4}),
    (96, 64, 12, 9, False, {}),
    (64, 48, 14, 10, False, {}),
    (2, 2, 8, 11, False, {}),
    (6, 4, 8, 12, False, {}),
    (64, 64, 10, 13, False, {"cmp_w_search": (1, 1, 1), "cmp_w_avg": (1, 1, 1)}),
    (64, 64, 10, 14, False, {"cmp_w_search": (3, 2, 1)}),
    # search ranges the specialised kernels do not take (generic kernel): none, and 5 to 16
    (96, 64, 10, 15, True, {"search_range": 0}),
    (120, 72, 10, 16, True, {"search_range": 5}),
    (128, 80, 8, 17, True, {"search_range": 8}),
    (160, 96, 10, 18, True, {"search_range": 16}),
]


@pytest.mark.parametrize("w,h,bd,seed,holes,opts", CASES)
def test_frame_host_input(gpu_lib, oq, w, h, bd, seed, holes, opts):
    ref, tst = _case(w, h, bd, seed, holes)
    ora, _, _ = _oracle(oq, ref, tst, w, h, bd, **opts)
    dtype = np.uint8 if bd == 8 else np.uint16
    pic0 = gpu_lib.make_pic(_planes(ref, w, h, dtype), bd)
    pic1 = gpu_lib.make_pic(_planes(tst, w, h, dtype), bd)
    with gpu_lib.Processor(w, h, **opts) as P:
        gpu = P.calc_frame(pic0, pic1, gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
    _cmp(gpu, ora)


def test_frame_device_input_erp_4k(gpu_lib, oq):
    import torch
    w, h, bd = 4096, 2048, 10
    ref, tst = _case(w, h, bd, synth.seed_for(1, 0, 0), True, sigma=2.0, offset=(3.0, -2.0, 1.0))
    ora, _, _ = _oracle(oq, ref, tst, w, h, bd, use_ws=True)
    d0 = [torch.from_numpy(p).cuda() for p in _planes(ref, w, h)]
    d1 = [torch.from_numpy(p).cuda() for p in _planes(tst, w, h)]
    with gpu_lib.Processor(w, h, use_ws=True) as P:
        gpu = P.calc_frame(gpu_lib.make_pic(d0, bd), gpu_lib.make_pic(d1, bd), gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
    _cmp(gpu, ora)


def test_444_input_generic_kernel(gpu_lib, oq):
    from oracle.oracle import upsample420
    w, h, bd = 200, 120, 10
    ref, tst = _case(w, h, bd, 21)
    ora, p0, p1 = _oracle(oq, ref, tst, w, h, bd)
    pic0 = gpu_lib.make_pic([p0[c] for c in range(3)], bd, gpu_lib.CF444)
    pic1 = gpu_lib.make_pic([p1[c] for c in range(3)], bd, gpu_lib.CF444)
    with gpu_lib.Processor(w, h) as P:
        gpu = P.calc_frame(pic0, pic1, gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
    _cmp(gpu, ora)


N_CPS_VARIANTS = 30  # compiled CPS variants (qmiv_cps_variant_count); checked below


def test_cps_variant_count(gpu_lib):
    assert len(gpu_lib.cps_variants()) == N_CPS_VARIANTS


@pytest.mark.parametrize("variant", range(N_CPS_VARIANTS))
def test_every_cps_variant(gpu_lib, oq, variant):
    names = gpu_lib.cps_variants()
    name = names[variant]
    sr = 2 if variant == 0 else int(name.split("_sr")[1].split("_")[0])
    # 14-bit samples need 64-bit keys at every search range; 8-bit variants read uint8 planes
    bd = 14 if "k64" in name else (8 if name.endswith("_u8") else 10)
    dtype = np.uint8 if bd == 8 else np.uint16
    # 352 x 98: not multiples of the chunk or strip; rows of 16-byte multiples in 8 and 16 bits
    w, h = 352, 98
    ref, tst = _case(w, h, bd, 31 + variant)
    ora, _, _ = _oracle(oq, ref, tst, w, h, bd, search_range=sr)
    with gpu_lib.Processor(w, h, search_range=sr) as P:
        P.set_cps_variant(variant)
        P.set_profiling(True)
        gpu = P.calc_frame(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd),
                           gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
        ran = [n for n, _ in P.kernel_times()]
        m0, m1, rows = P.cps_maps(gpu_lib.make_pic(_planes(ref, w, h, dtype), bd), gpu_lib.make_pic(_planes(tst, w, h, dtype), bd))
        ran_maps = [n for n, _ in P.kernel_times()]
    assert name in ran, (name, ran)  # the requested variant is the one that ran
    assert name in ran_maps, (name, ran_maps)
    _cmp(gpu, ora)
    assert gpu["status"] == 0
    # per-pixel argmin and per-row sums of both directions, bit-exact
    from oracle.oracle import upsample420
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    r0, a0, _, _ = oq.cps_dir(p0, p1, bd, ora["gcd"], sr, nthreads=8)
    r1, a1, _, _ = oq.cps_dir(p1, p0, bd, [-x for x in ora["gcd"]], sr, nthreads=8)
    np.testing.assert_array_equal(m0.astype(np.int8), a0)
    np.testing.assert_array_equal(m1.astype(np.int8), a1)
    np.testing.assert_array_equal(rows[0], r0)
    np.testing.assert_array_equal(rows[1], r1)


def test_scp_bit_exact(gpu_lib, oq):
    w, h, bd = 512, 256, 10
    ref, tst = _case(w, h, bd, 41, True)
    ora, p0, p1 = _oracle(oq, ref, tst, w, h, bd)
    g = ora["gcd"]
    _, _, _, scp1 = oq.cps_dir(p0, p1, bd, g, 2)
    _, _, _, scp0 = oq.cps_dir(p1, p0, bd, [-x for x in g], 2)
    s0 = [np.zeros((h, w), np.uint16) for _ in range(3)]
    s1 = [np.zeros((h, w), np.uint16) for _ in range(3)]
    with gpu_lib.Processor(w, h) as P:
        P.scp(gpu_lib.make_pic(_planes(ref, w, h), bd), gpu_lib.make_pic(_planes(tst, w, h), bd), s0, s1)
    for c in range(3):
        np.testing.assert_array_equal(s0[c], scp0[c])
        np.testing.assert_array_equal(s1[c], scp1[c])


def test_given_gcd_and_identical_pictures(gpu_lib, oq):
    w, h, bd = 128, 64, 10
    ref, tst = _case(w, h, bd, 51)
    pic0 = gpu_lib.make_pic(_planes(ref, w, h), bd)
    with gpu_lib.Processor(w, h) as P:
        r = P.calc_frame(pic0, gpu_lib.make_pic(_planes(ref, w, h), bd), gpu_lib.M_ALL & 0x7)
        assert r["exact"][:3] == [1, 1, 1]
        fake = 10 * np.log10(w * h * 1023.0 ** 2)
        np.testing.assert_allclose(r["psnr"][:3], [fake] * 3, atol=1e-10)
        # IV-PSNR of identical pictures: every SSE is 0 and counts as 1 (xIVPSNR.cpp:126)
        assert r["sse_r2t"][:3] == [0, 0, 0]
        iv, r2t, t2r = P.ivpsnr(pic0, gpu_lib.make_pic(_planes(tst, w, h), bd), gcd=[1, -1, 2])
    from oracle.oracle import upsample420
    p0 = upsample420(synth.split420(ref, w, h), w, h)
    p1 = upsample420(synth.split420(tst, w, h), w, h)
    rows0, _, _, _ = oq.cps_dir(p0, p1, bd, [1, -1, 2], 2)
    rows1, _, _, _ = oq.cps_dir(p1, p0, bd, [-1, 1, -2], 2)
    lib = oq.lib()
    import ctypes
    wavg = (ctypes.c_int32 * 3)(4, 1, 1)
    lib.oq_quality_from_rows.restype = ctypes.c_double
    lib.oq_quality_from_rows.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_void_p, ctypes.c_void_p]
    q0 = lib.oq_quality_from_rows(rows0.ctypes.data, h, w * h, bd, None, wavg)
    q1 = lib.oq_quality_from_rows(rows1.ctypes.data, h, w * h, bd, None, wavg)
    assert abs(r2t - q0) <= DB_TOL and abs(t2r - q1) <= DB_TOL and abs(iv - min(q0, q1)) <= DB_TOL


def test_batch_mixed_sizes(gpu_lib, oq):
    import torch
    sizes = [(640, 360, 10, True), (320, 180, 10, False), (256, 256, 8, False), (128, 66, 10, True)]
    jobs, keep, oras = [], [], []
    from ivpsnr_gb300 import _abi
    import ctypes
    for i, (w, h, bd, ws) in enumerate(sizes):
        ref, tst = _case(w, h, bd, 60 + i, holes=True)
        ora, _, _ = _oracle(oq, ref, tst, w, h, bd, use_ws=ws)
        oras.append((ora, ws))
        d0 = [torch.from_numpy(p).cuda() for p in _planes(ref, w, h)]
        d1 = [torch.from_numpy(p).cuda() for p in _planes(tst, w, h)]
        keep += [d0, d1]
        j = _abi.Job()
        j.pic0 = gpu_lib.make_pic(d0, bd)
        j.pic1 = gpu_lib.make_pic(d1, bd)
        j.metrics = gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR
        j.use_ws = int(ws)
        jobs.append(j)
    res = torch.zeros(len(jobs) * ctypes.sizeof(_abi.FrameResult), dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(640, 360, max_jobs=len(jobs)) as P:
        for _ in range(2):  # twice: the per-job counters must reset themselves
            res.zero_()
            P.calc_batch(jobs, res.data_ptr())
            torch.cuda.synchronize()
            host = res.cpu().numpy().tobytes()
            for i, (ora, ws) in enumerate(oras):
                r = _abi.FrameResult.from_buffer_copy(host[i * ctypes.sizeof(_abi.FrameResult):(i + 1) * ctypes.sizeof(_abi.FrameResult)])
                _cmp(r.to_dict(), ora)


def test_8k_erp_sr4_matches_oracle(gpu_lib, oq):
    """The streamed-sequence picture size: 7680x3840 ERP 10-bit, search range 4, device input."""
    import torch
    w, h, bd = 7680, 3840, 10
    ref, tst = synth.pair420(w, h, bd, seed=synth.seed_for(4, 0, 0), holes=True)
    d0 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(ref, w, h)]
    d1 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(tst, w, h)]
    with gpu_lib.Processor(w, h, search_range=4, use_ws=True, scratch_metrics=gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR) as P:
        g = P.calc_frame(gpu_lib.make_pic(d0, bd), gpu_lib.make_pic(d1, bd), gpu_lib.M_PSNR | gpu_lib.M_WSPSNR | gpu_lib.M_IVPSNR)
    from oracle.oracle import upsample420
    o = oq.frame(upsample420(synth.split420(ref, w, h), w, h), upsample420(synth.split420(tst, w, h), w, h), bd, False,
                 use_ws=True, search_range=4, nthreads=16)
    assert g["gcd_r2t"][:3] == o["gcd"]
    assert g["sse_r2t"][:3] == o["sse_r2t"] and g["sse_t2r"][:3] == o["sse_t2r"]
    for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
        assert abs(g[k] - o[k]) <= 1e-10
    assert max(abs(a - b) for a, b in zip(g["wspsnr"][:3], o["wspsnr"])) <= 1e-10
