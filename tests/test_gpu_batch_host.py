"""qmiv_calc_batch_host: a batch of host pictures uploaded in groups on the handle's own upload
stream while the previous group is measured. Its results must equal qmiv_calc_batch on device
copies of the same pictures, whatever the grouping (one job per group, the default eighth of the
batch, one group), for padded host rows, 8- and 10-bit, 4:2:0 and 4:4:4, back-to-back calls
without a synchronisation between them, and with fewer job slots than jobs."""
import ctypes

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu

SIZES = [  # w, h, bd, 4:4:4, holes, metrics, use_ws, padded host rows
    (320, 180, 10, False, True, "all", 0, False),
    (256, 128, 8, False, False, "ivpsnr", 1, True),
    (192, 96, 10, True, False, "ivssim", 0, False),
    (640, 360, 10, False, True, "psnr", 1, True),
    (128, 64, 8, True, True, "all", 0, True),
    (96, 64, 12, False, False, "ivpsnr", 0, False),
    (512, 256, 10, False, False, "all", 1, False),
]


def _metrics(q, name):
    return {"all": q.M_ALL, "ivpsnr": q.M_PSNR | q.M_WSPSNR | q.M_IVPSNR, "ivssim": q.M_IVSSIM | q.M_IVPSNR,
            "psnr": q.M_PSNR | q.M_WSPSNR}[name]


def _host_planes(flat, w, h, bd, cf444, padded):
    from oracle.oracle import upsample420
    dt = np.uint8 if bd == 8 else np.uint16
    planes = list(upsample420(synth.split420(flat, w, h), w, h)) if cf444 else list(synth.split420(flat, w, h))
    out = []
    for p in planes:
        p = p.astype(dt)
        if padded:  # rows inside a wider buffer: the host stride is not the width
            buf = np.zeros((p.shape[0], p.shape[1] + 13), dt)
            buf[:, 5:5 + p.shape[1]] = p
            p = buf[:, 5:5 + p.shape[1]]
        out.append(p)
    return out


def _jobs(q, device):
    import torch
    from ivpsnr_gb300 import _abi
    jobs, keep = [], []
    for i, (w, h, bd, cf444, holes, m, ws, padded) in enumerate(SIZES):
        ref, tst = synth.pair420(w, h, bd, seed=900 + i, holes=holes)
        cf = q.CF444 if cf444 else q.CF420
        p0 = _host_planes(ref, w, h, bd, cf444, padded and not device)
        p1 = _host_planes(tst, w, h, bd, cf444, padded and not device)
        if device:
            conv = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16 if a.dtype == np.uint16 else np.uint8)).cuda()
            p0, p1 = [conv(a) for a in p0], [conv(a) for a in p1]
        keep.append((p0, p1))
        j = _abi.Job()
        j.pic0 = q.make_pic(p0, bd, cf)
        j.pic1 = q.make_pic(p1, bd, cf)
        j.metrics = _metrics(q, m)
        j.use_ws = ws
        jobs.append(j)
    return jobs, keep


def _results(res, n):
    from ivpsnr_gb300 import _abi
    rs = ctypes.sizeof(_abi.FrameResult)
    host = res.cpu().numpy().tobytes()
    return [_abi.FrameResult.from_buffer_copy(host[i * rs:(i + 1) * rs]).to_dict() for i in range(n)]


def _same(a, b):
    if isinstance(a, (list, tuple)):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    if isinstance(a, float) and a != a:
        return b != b
    return a == b


def _diff(got, want):
    """(job, field, got, want) of every field that differs; NaN equals NaN."""
    return [(i, k, g[k], w[k]) for i, (g, w) in enumerate(zip(got, want)) for k in w if not _same(g[k], w[k])]


def test_host_batch_matches_device_batch(gpu_lib):
    import torch
    from ivpsnr_gb300 import _abi
    q = gpu_lib
    n = len(SIZES)
    rs = ctypes.sizeof(_abi.FrameResult)
    djobs, dkeep = _jobs(q, device=True)
    hjobs, hkeep = _jobs(q, device=False)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    with q.Processor(640, 360, max_jobs=n) as P, torch.cuda.stream(stream):
        ref = torch.zeros(n * rs, dtype=torch.uint8, device="cuda")
        P.calc_batch(djobs, ref.data_ptr(), sp)
        stream.synchronize()
        want = _results(ref, n)
        assert all(w["status"] == 0 for w in want)
        for group_bytes in (1, 0, 1 << 40):
            got = torch.full((n * rs,), 0xAB, dtype=torch.uint8, device="cuda")
            P.calc_batch_host(hjobs, got.data_ptr(), group_bytes, sp)
            stream.synchronize()
            assert not _diff(_results(got, n), want), group_bytes
        # back to back, no synchronisation in between, into two result buffers
        a = torch.zeros(n * rs, dtype=torch.uint8, device="cuda")
        b = torch.zeros_like(a)
        P.calc_batch_host(hjobs, a.data_ptr(), 1, sp)
        P.calc_batch_host(hjobs[::-1], b.data_ptr(), 0, sp)
        stream.synchronize()
        assert not _diff(_results(a, n), want)
        assert not _diff(_results(b, n), want[::-1])


def test_host_batch_with_fewer_slots_pinned_and_default_stream(gpu_lib):
    import torch
    from ivpsnr_gb300 import _abi
    q = gpu_lib
    n = len(SIZES)
    rs = ctypes.sizeof(_abi.FrameResult)
    djobs, dkeep = _jobs(q, device=True)
    with q.Processor(640, 360, max_jobs=n) as P:
        ref = torch.zeros(n * rs, dtype=torch.uint8, device="cuda")
        P.calc_batch(djobs, ref.data_ptr(), 0)
        torch.cuda.synchronize()
        want = _results(ref, n)
    # page-locked host copies of the same pictures
    pinned = []
    hjobs = []
    for j, (p0, p1) in zip(djobs, dkeep):
        h0 = [t.cpu().pin_memory() for t in p0]
        h1 = [t.cpu().pin_memory() for t in p1]
        pinned.append((h0, h1))
        k = _abi.Job()
        k.pic0 = q.make_pic(h0, j.pic0.bitdepth, j.pic0.chroma_format)
        k.pic1 = q.make_pic(h1, j.pic1.bitdepth, j.pic1.chroma_format)
        k.metrics, k.use_ws = j.metrics, j.use_ws
        hjobs.append(k)
    with q.Processor(640, 360, max_jobs=3) as P:  # groups hold at most three jobs
        got = torch.zeros(n * rs, dtype=torch.uint8, device="cuda")
        P.calc_batch_host(hjobs, got.data_ptr(), 0, 0)
        torch.cuda.synchronize()
        assert not _diff(_results(got, n), want)
        with pytest.raises(q.QmivError):
            P.calc_batch_host(djobs, got.data_ptr(), 0, 0)
