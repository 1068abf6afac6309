"""Input-side operations on the GPU against the reference golden outputs (tests/golden/io.json)
and the oracle: colour conversion, range check / concealment, and the raw YUV reader feeding
the metric path (4:2:0, 4:2:2 and 4:4:4 files, 8 and 10 bit)."""
import ctypes
import json
import os

import numpy as np
import pytest

from ivpsnr_gb300 import synth

from .golden.make_golden import io_inputs, md5

pytestmark = pytest.mark.gpu
IO = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "io.json")))


def _dev_pic(gpu_lib, planes, bd, cf):
    import torch
    d = [torch.from_numpy(np.ascontiguousarray(p).view(np.int16)).cuda() for p in planes]
    return gpu_lib.make_pic(d, bd, cf), d


@pytest.mark.parametrize("case", [c for c in IO["cases"] if c["kind"] == "color"],
                         ids=["s%d_to%d_bd%d" % (c["space"], c["to_ycbcr"], c["bd"]) for c in IO["cases"] if c["kind"] == "color"])
def test_color_matches_reference(gpu_lib, case):
    import torch
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    w, h, bd = case["w"], case["h"], case["bd"]
    x = io_inputs("color", w, h, bd, case["seed"])
    pic, keep = _dev_pic(gpu_lib, list(x), bd, gpu_lib.CF444)
    out = torch.zeros((3, h, w), dtype=torch.int16, device="cuda")
    dst = (ctypes.c_void_p * 3)(*[out[c].data_ptr() for c in range(3)])
    _abi.check(lib.qmiv_color_convert(ctypes.byref(pic), dst, w, case["to_ycbcr"], case["space"], None), "qmiv_color_convert")
    torch.cuda.synchronize()
    y = out.cpu().numpy().view(np.uint16)
    assert md5(y) == case["output_md5"]
    # in place, as xAppQMIV::preprocessFrames converts its input pictures
    dst = (ctypes.c_void_p * 3)(*[k.data_ptr() for k in keep])
    _abi.check(lib.qmiv_color_convert(ctypes.byref(pic), dst, w, case["to_ycbcr"], case["space"], None), "qmiv_color_convert")
    torch.cuda.synchronize()
    assert md5(np.stack([k.cpu().numpy() for k in keep])) == case["output_md5"]


@pytest.mark.parametrize("case", [c for c in IO["cases"] if c["kind"] == "range"], ids=lambda c: "bd%d" % c["bd"])
def test_range_check_matches_reference(gpu_lib, oq, case):
    import torch
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    w, h, bd = case["w"], case["h"], case["bd"]
    x = io_inputs("range", w, h, bd, case["seed"])
    planes = [x, x[: h // 2, : w // 2].copy(), x[h // 2:, w // 2:].copy()]
    pic, keep = _dev_pic(gpu_lib, planes, bd, gpu_lib.CF420)
    cnt = (ctypes.c_int64 * 3)()
    _abi.check(lib.qmiv_check_range(ctypes.byref(pic), 0, cnt, None), "qmiv_check_range")
    want = [oq.range_clip(p, bd)[0] for p in planes]
    assert list(cnt) == want and (want[0] == 0) == bool(case["in_range"])
    _abi.check(lib.qmiv_check_range(ctypes.byref(pic), 1, cnt, None), "qmiv_check_range")
    torch.cuda.synchronize()
    assert md5(keep[0].cpu().numpy()) == case["output_md5"]
    _abi.check(lib.qmiv_check_range(ctypes.byref(pic), 0, cnt, None), "qmiv_check_range")
    assert list(cnt) == [0, 0, 0]


# the last case's frames (1.6 MiB) take the reader's parallel slice reads (frames of 1 MiB and
# more), the others a single read
@pytest.mark.parametrize("cf,bd,w,h", [(420, 8, 96, 64), (422, 10, 96, 64), (444, 10, 96, 64), (420, 10, 1024, 544)])
def test_yuv_reader_feeds_the_metrics(gpu_lib, oq, tmp_path, cf, bd, w, h):
    import torch
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    nf = 3
    frames = []
    for f in range(nf):
        r, t = synth.pair420(w, h, bd, seed=70 + f, holes=True)
        ry, rcb, rcr = synth.split420(r, w, h)
        ty, tcb, tcr = synth.split420(t, w, h)
        if cf == 420:
            frames.append(([ry, rcb, rcr], [ty, tcb, tcr]))
        elif cf == 422:  # chroma planes (w/2) x h: repeat the 4:2:0 rows
            frames.append(([ry, np.repeat(rcb, 2, 0), np.repeat(rcr, 2, 0)], [ty, np.repeat(tcb, 2, 0), np.repeat(tcr, 2, 0)]))
        else:
            frames.append(([ry, np.repeat(np.repeat(rcb, 2, 0), 2, 1), np.repeat(np.repeat(rcr, 2, 0), 2, 1)],
                           [ty, np.repeat(np.repeat(tcb, 2, 0), 2, 1), np.repeat(np.repeat(tcr, 2, 0), 2, 1)]))
    dt = np.uint8 if bd == 8 else np.dtype("<u2")
    paths = []
    for i in range(2):
        p = tmp_path / ("in%d.yuv" % i)
        with open(p, "wb") as fh:
            for fr in frames:
                fh.write(b"".join(np.ascontiguousarray(x.astype(dt)).tobytes() for x in fr[i]))
        paths.append(str(p).encode())
    readers = []
    for p in paths:
        r = ctypes.c_void_p()
        _abi.check(lib.qmiv_yuv_open(ctypes.byref(r), p, w, h, bd, cf), "qmiv_yuv_open")
        readers.append(r)
    try:
        assert lib.qmiv_yuv_frames(readers[0]) == nf
        with gpu_lib.Processor(w, h) as P:
            for f in (2, 0, 1):
                a, b = _abi.Pic(), _abi.Pic()
                _abi.check(lib.qmiv_yuv_read(readers[0], f, ctypes.byref(a), None), "qmiv_yuv_read")
                _abi.check(lib.qmiv_yuv_read(readers[1], f, ctypes.byref(b), None), "qmiv_yuv_read")
                g = P.calc_frame(a, b, gpu_lib.M_PSNR | gpu_lib.M_IVPSNR | gpu_lib.M_SSIM)
                raw0 = open(paths[0], "rb").read()
                raw1 = open(paths[1], "rb").read()
                fb = len(raw0) // nf
                bps = 1 if bd == 8 else 2
                p0 = oq.unpack_frame(raw0[f * fb:(f + 1) * fb], w, h, bps, cf)
                p1 = oq.unpack_frame(raw1[f * fb:(f + 1) * fb], w, h, bps, cf)
                o = oq.frame(p0, p1, bd, True)
                assert g["gcd_r2t"][:3] == o["gcd"]
                assert abs(g["ivpsnr"] - o["ivpsnr"]) <= 1e-10
                np.testing.assert_allclose(g["psnr"][:3], o["psnr"], atol=1e-10)
                np.testing.assert_allclose(g["ssim"][:3], o["ssim"], atol=1e-6)
    finally:
        for r in readers:
            lib.qmiv_yuv_close(r)
        torch.cuda.synchronize()


def test_input_side_rejections(gpu_lib, tmp_path):
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    x = np.zeros((3, 8, 8), np.uint16)
    host = gpu_lib.make_pic(list(x), 10, gpu_lib.CF444)
    cnt = (ctypes.c_int64 * 3)()
    assert lib.qmiv_check_range(ctypes.byref(host), 0, cnt, None) != 0
    dev, keep = _dev_pic(gpu_lib, list(x), 16, gpu_lib.CF444)
    dst = (ctypes.c_void_p * 3)(*[k.data_ptr() for k in keep])
    assert lib.qmiv_color_convert(ctypes.byref(dev), dst, 8, 1, 0, None) != 0  # 16-bit input
    p = tmp_path / "odd.yuv"
    p.write_bytes(b"\0" * 1000)
    r = ctypes.c_void_p()
    assert lib.qmiv_yuv_open(ctypes.byref(r), str(p).encode(), 7, 4, 8, 420) != 0
    assert lib.qmiv_yuv_open(ctypes.byref(r), str(p).encode(), 8, 4, 8, 411) != 0
    _abi.check(lib.qmiv_yuv_open(ctypes.byref(r), str(p).encode(), 8, 4, 8, 420), "qmiv_yuv_open")
    try:
        assert lib.qmiv_yuv_frames(r) == 1000 // 48
        out = _abi.Pic()
        assert lib.qmiv_yuv_read(r, 1000 // 48, ctypes.byref(out), None) != 0
    finally:
        lib.qmiv_yuv_close(r)


def test_range_check_from_several_threads(gpu_lib):
    """qmiv_check_range keeps its counters per calling thread and device: four host threads
    checking different pictures at once (ctypes releases the GIL) each get their own counts,
    also on their first call, when the counters are made."""
    import threading

    import torch
    from ivpsnr_gb300 import _abi
    lib = _abi.load()
    w, h, bd = 256, 64, 10
    rng = np.random.default_rng(11)
    pics, want = [], []
    for k in range(4):
        planes = [rng.integers(0, 1 << bd, (h, w)).astype(np.uint16) for _ in range(3)]
        for c in range(3):  # k + c + 1 samples above 1023 in component c of picture k
            idx = rng.choice(w * h, size=k + c + 1, replace=False)
            planes[c].reshape(-1)[idx] = 1023 + 1 + rng.integers(0, 100, size=idx.size)
        pic, keep = _dev_pic(gpu_lib, planes, bd, gpu_lib.CF444)
        pics.append((pic, keep))
        want.append([k + 1, k + 2, k + 3])
    torch.cuda.synchronize()
    got = [None] * 4
    errors = []

    def work(k):
        try:
            torch.cuda.set_device(0)
            for _ in range(20):
                cnt = (ctypes.c_int64 * 3)()
                _abi.check(lib.qmiv_check_range(ctypes.byref(pics[k][0]), 0, cnt, None), "qmiv_check_range")
                if list(cnt) != want[k]:
                    errors.append((k, list(cnt)))
            got[k] = list(cnt)
        except Exception as ex:  # reported below, not swallowed
            errors.append((k, repr(ex)))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert got == want
