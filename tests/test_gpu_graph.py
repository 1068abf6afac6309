"""A batch captured as a CUDA graph (qmiv_batch_graph_*) gives the same results as the direct
batched call, replays correctly after the device pictures are rewritten in place, and keeps
working after the handle is used for other calls in between."""
import ctypes

import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu


def _device_pair(w, h, bd, seed, holes):
    import torch
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=holes)
    dt = np.uint8 if bd == 8 else np.uint16
    up = lambda flat: [torch.from_numpy(np.ascontiguousarray(p.astype(dt))).cuda() for p in synth.split420(flat, w, h)]
    return up(ref), up(tst)


def _results(res, n):
    from ivpsnr_gb300 import _abi
    rs = ctypes.sizeof(_abi.FrameResult)
    host = res.cpu().numpy().tobytes()
    return [_abi.FrameResult.from_buffer_copy(host[i * rs:(i + 1) * rs]).to_dict() for i in range(n)]


def test_graph_replay_matches_direct_batch(gpu_lib):
    import torch
    from ivpsnr_gb300 import _abi
    sizes = [(320, 180, 10, True, gpu_lib.M_ALL), (256, 128, 8, False, gpu_lib.M_PSNR | gpu_lib.M_IVPSNR),
             (192, 96, 10, False, gpu_lib.M_IVSSIM | gpu_lib.M_IVPSNR)]
    pics, jobs = [], []
    for i, (w, h, bd, holes, m) in enumerate(sizes):
        d0, d1 = _device_pair(w, h, bd, 500 + i, holes)
        pics.append((d0, d1))
        j = _abi.Job()
        j.pic0 = gpu_lib.make_pic(d0, bd)
        j.pic1 = gpu_lib.make_pic(d1, bd)
        j.metrics = m
        jobs.append(j)
    rs = ctypes.sizeof(_abi.FrameResult)
    res_direct = torch.zeros(len(jobs) * rs, dtype=torch.uint8, device="cuda")
    res_graph = torch.zeros_like(res_direct)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    with gpu_lib.Processor(320, 180, max_jobs=len(jobs)) as P, torch.cuda.stream(stream):
        P.calc_batch(jobs, res_direct.data_ptr(), sp)
        stream.synchronize()
        want = _results(res_direct, len(jobs))
        with P.capture_batch(jobs, res_graph.data_ptr(), sp) as G:
            for rep in range(3):
                res_graph.zero_()
                G.launch(sp)
                stream.synchronize()
                got = _results(res_graph, len(jobs))
                for g, wnt in zip(got, want):
                    assert g == wnt, rep
                # another call on the handle between replays
                P.calc_frame(gpu_lib.make_pic(pics[1][0], 8), gpu_lib.make_pic(pics[1][1], 8), gpu_lib.M_ALL, sp)
            # new frame contents in the same buffers: the replay measures them
            d0n, d1n = _device_pair(320, 180, 10, 777, True)
            for c in range(3):
                pics[0][0][c].copy_(d0n[c])
                pics[0][1][c].copy_(d1n[c])
            G.launch(sp)
            P.calc_batch(jobs, res_direct.data_ptr(), sp)
            stream.synchronize()
            res_graph.zero_()
            G.launch(sp)
            stream.synchronize()
            assert _results(res_graph, len(jobs)) == _results(res_direct, len(jobs))
            assert _results(res_graph, 1)[0]["ivpsnr"] != want[0]["ivpsnr"]


def test_graph_rejects_default_stream(gpu_lib):
    import torch
    from ivpsnr_gb300 import _abi
    d0, d1 = _device_pair(64, 32, 8, 9, False)
    j = _abi.Job()
    j.pic0 = gpu_lib.make_pic(d0, 8)
    j.pic1 = gpu_lib.make_pic(d1, 8)
    j.metrics = gpu_lib.M_PSNR
    res = torch.zeros(ctypes.sizeof(_abi.FrameResult), dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(64, 32) as P:
        with pytest.raises(gpu_lib.QmivError):
            P.capture_batch([j], res.data_ptr(), 0)


def test_autotuner_picks_a_fitting_variant_and_keeps_results(gpu_lib):
    import torch
    from ivpsnr_gb300 import _abi
    jobs, keep = [], []
    for i, (w, h) in enumerate([(1920, 1080), (1280, 720)]):
        d0, d1 = _device_pair(w, h, 10, 600 + i, True)
        keep.append((d0, d1))
        j = _abi.Job()
        j.pic0 = gpu_lib.make_pic(d0, 10)
        j.pic1 = gpu_lib.make_pic(d1, 10)
        j.metrics = gpu_lib.M_PSNR | gpu_lib.M_IVPSNR
        jobs.append(j)
    rs = ctypes.sizeof(_abi.FrameResult)
    res = torch.zeros(len(jobs) * rs, dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(1920, 1080, max_jobs=2) as P:
        P.calc_batch(jobs, res.data_ptr())
        torch.cuda.synchronize()
        want = _results(res, 2)
        v, name, ms = P.autotune_cps(jobs, res.data_ptr(), reps=2)
        assert v > 0 and name.startswith(("tma420_sr2", "cps420_sr2")) and ms > 0
        res.zero_()
        P.calc_batch(jobs, res.data_ptr())
        torch.cuda.synchronize()
        assert _results(res, 2) == want
