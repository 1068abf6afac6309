"""The failure path of the bounded device-side waits, made to run without any fault: with
qmiv_test_wait_timeout the first bulk-copy wait of every block polls a barrier that no copy
arrives on, gives up, records QMIV_DEVICE_TIMEOUT, waits (with the full limit) for its own copies
in flight and stops. The call must report the timeout, and the same handle must then give the
normal results again (every kernel's counters and statuses reset themselves)."""
import numpy as np
import pytest

from ivpsnr_gb300 import synth

pytestmark = pytest.mark.gpu
POLLS = 64


def _device_pics(gpu_lib, w, h, bd, seed):
    import torch
    ref, tst = synth.pair420(w, h, bd, seed=seed, holes=True)
    d0 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(ref, w, h)]
    d1 = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in synth.split420(tst, w, h)]
    return (d0, d1), gpu_lib.make_pic(d0, bd), gpu_lib.make_pic(d1, bd)


def _same(a, b, keys):
    for k in keys:
        assert a[k] == b[k], (k, a[k], b[k])


@pytest.mark.parametrize("metrics_name", ["ivpsnr", "ivssim"])
def test_timeout_is_reported_and_the_handle_recovers(gpu_lib, metrics_name):
    """ivpsnr: the TMA search kernel (search range 2) is the only kernel with bulk-copy waits.
    ivssim: search range 5 runs the generic search kernel (plain loads), so the fused SSIM kernel
    is the one whose wait gives up."""
    from ivpsnr_gb300 import _abi
    w, h, bd = 640, 360, 10
    keep, p0, p1 = _device_pics(gpu_lib, w, h, bd, 901)
    if metrics_name == "ivpsnr":
        metrics, sr, keys = gpu_lib.M_PSNR | gpu_lib.M_IVPSNR, 2, ("ivpsnr", "sse_r2t", "sse_t2r", "psnr", "gcd_r2t")
    else:
        metrics, sr, keys = gpu_lib.M_ALL, 5, ("ivssim", "ssim", "msssim", "ivpsnr", "sse_r2t")
    with gpu_lib.Processor(w, h, search_range=sr) as P:
        good = P.calc_frame(p0, p1, metrics)
        assert good["status"] == 0
        P.set_profiling(True)
        P.test_wait_timeout(POLLS)
        with pytest.raises(gpu_lib.QmivError) as e:
            P.calc_frame(p0, p1, metrics)
        assert e.value.status == _abi.QMIV_DEVICE_TIMEOUT
        ran = [n for n, _ in P.kernel_times()]
        if metrics_name == "ivpsnr":
            assert any(n.startswith("tma420_") for n in ran), ran
        else:
            assert "cps_generic" in ran and any(n.startswith("k_ssim_quad") for n in ran), ran
        P.test_wait_timeout(0)
        for _ in range(2):
            again = P.calc_frame(p0, p1, metrics)
            assert again["status"] == 0
            _same(good, again, keys)


def test_timeout_in_a_batch_marks_every_frame(gpu_lib):
    import ctypes
    import torch
    from ivpsnr_gb300 import _abi
    w, h, bd = 320, 180, 10
    pics = [_device_pics(gpu_lib, w, h, bd, 910 + i) for i in range(3)]
    jobs = []
    for _, a, b in pics:
        j = _abi.Job()
        j.pic0, j.pic1, j.metrics = a, b, gpu_lib.M_PSNR | gpu_lib.M_IVPSNR
        jobs.append(j)
    rs = ctypes.sizeof(_abi.FrameResult)
    res = torch.zeros(len(jobs) * rs, dtype=torch.uint8, device="cuda")
    with gpu_lib.Processor(w, h, max_jobs=len(jobs)) as P:
        out = []
        for polls in (0, POLLS, 0):
            P.test_wait_timeout(polls)
            P.calc_batch(jobs, res.data_ptr())
            torch.cuda.synchronize()
            host = res.cpu().numpy().tobytes()
            out.append([_abi.FrameResult.from_buffer_copy(host[i * rs:(i + 1) * rs]).to_dict() for i in range(len(jobs))])
    assert all(r["status"] == 0 for r in out[0] + out[2])
    assert all(r["status"] == _abi.QMIV_DEVICE_TIMEOUT for r in out[1])
    for a, b in zip(out[0], out[2]):
        _same(a, b, ("ivpsnr", "sse_r2t", "sse_t2r", "psnr"))
