"""The all-metrics multiview batch at its own sizes: one frame of each of its 12 views (three
4096x2048 ERP with WS-PSNR, six 1920x1080, three 2048x1088; 10-bit 4:2:0 with holes) in one
qmiv_calc_batch with every metric (GCD, PSNR, WS-PSNR, IV-PSNR, SSIM, MS-SSIM, IV-SSIM), each pair
against the FP64 oracle: GCD, exact flags and CPS squared-error sums bit-exact, PSNR-family dB
within 1e-10, SSIM family within 1e-6."""
import ctypes

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
DB_TOL, SSIM_TOL = 1e-10, 1e-6
VIEWS = [(4096, 2048, True)] * 3 + [(1920, 1080, False)] * 6 + [(2048, 1088, False)] * 3


def test_multiview_all_metrics_batch(gpu_lib, oq):
    import torch
    from ivpsnr_gb300 import _abi
    from oracle.oracle import upsample420
    q = gpu_lib
    dev = lambda flat, w, h: [torch.from_numpy(np.ascontiguousarray(p.astype(np.uint16))).cuda() for p in synth.split420(flat, w, h)]
    jobs, keep, want = [], [], []
    for v, (w, h, erp) in enumerate(VIEWS):
        ref, tst = synth.pair420(w, h, 10, seed=synth.seed_for(1, v, 0), holes=True)
        d0, d1 = dev(ref, w, h), dev(tst, w, h)
        keep.append((d0, d1))
        j = _abi.Job()
        j.pic0 = q.make_pic(d0, 10)
        j.pic1 = q.make_pic(d1, 10)
        j.metrics = q.M_ALL
        j.use_ws = int(erp)
        jobs.append(j)
        p0 = upsample420(synth.split420(ref, w, h), w, h)
        p1 = upsample420(synth.split420(tst, w, h), w, h)
        want.append(oq.frame(p0, p1, 10, True, use_ws=erp, nthreads=16))
    rs = ctypes.sizeof(_abi.FrameResult)
    res = torch.zeros(len(jobs) * rs, dtype=torch.uint8, device="cuda")
    with q.Processor(4096, 2048, max_jobs=len(jobs)) as P:
        P.calc_batch(jobs, res.data_ptr(), 0)
        torch.cuda.synchronize()
    host = res.cpu().numpy().tobytes()
    for i, o in enumerate(want):
        g = _abi.FrameResult.from_buffer_copy(host[i * rs:(i + 1) * rs]).to_dict()
        assert g["status"] == 0, i
        assert g["gcd_r2t"][:3] == o["gcd"] and g["exact"][:3] == o["exact"], i
        assert g["sse_r2t"][:3] == o["sse_r2t"] and g["sse_t2r"][:3] == o["sse_t2r"], i
        np.testing.assert_allclose(g["psnr"][:3], o["psnr"], rtol=0, atol=DB_TOL)
        np.testing.assert_allclose(g["wspsnr"][:3], o["wspsnr"], rtol=0, atol=DB_TOL)
        for k in ("ivpsnr", "ivpsnr_r2t", "ivpsnr_t2r"):
            assert abs(g[k] - o[k]) <= DB_TOL, (i, k)
        np.testing.assert_allclose(g["ssim"][:3], o["ssim"], rtol=0, atol=SSIM_TOL)
        np.testing.assert_allclose(g["msssim"][:3], o["msssim"], rtol=0, atol=SSIM_TOL)
        for k in ("ivssim", "ivssim_r2t", "ivssim_t2r"):
            assert abs(g[k] - o[k]) <= SSIM_TOL, (i, k)
