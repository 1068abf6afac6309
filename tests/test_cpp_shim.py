"""The header-only C++ processors (include/qmiv_gb300.hpp) that mirror the reference's metric
classes: they compile against the C ABI, fail cleanly without a GPU, and on a GPU give the
same numbers as the C ABI called directly."""
import json
import os
import subprocess

import numpy as np
import pytest

from .conftest import ROOT


def _build(tmp_path):
    exe = str(tmp_path / "shim_demo")
    lib_dir = os.path.join(ROOT, "ivpsnr_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_demo.cpp"), "-o", exe, "-L", lib_dir, "-lqmiv_gb300",
                    "-Wl,-rpath," + lib_dir], check=True)
    return exe


def test_cpp_processors_compile_and_fail_cleanly_without_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ivpsnr_gb300 import _abi
    _abi.load()  # the library is built
    out = subprocess.run([_build(tmp_path), "probe"], check=True, capture_output=True, text=True).stdout
    assert json.loads(out)["status"] == _abi.QMIV_CUDA_ERROR


@pytest.mark.gpu
@pytest.mark.parametrize("w,h,erp", [(320, 180, False), (512, 256, True)])
def test_cpp_processors_match_the_c_abi(gpu_lib, tmp_path, w, h, erp):
    from ivpsnr_gb300 import synth
    bd = 10
    ref, tst = synth.pair420(w, h, bd, seed=77 + w, holes=True)
    ref.tofile(tmp_path / "ref.raw")
    tst.tofile(tmp_path / "tst.raw")
    args = [_build(tmp_path), str(w), str(h), str(bd), str(tmp_path / "ref.raw"), str(tmp_path / "tst.raw")]
    got = json.loads(subprocess.run(args + (["erp"] if erp else []), check=True, capture_output=True, text=True).stdout)
    planes = lambda flat: [np.ascontiguousarray(p) for p in synth.split420(flat, w, h)]
    with gpu_lib.Processor(w, h, use_ws=erp) as P:
        want = P.calc_frame(gpu_lib.make_pic(planes(tst), bd), gpu_lib.make_pic(planes(ref), bd), gpu_lib.M_ALL)
    assert got["gcd"] == want["gcd_r2t"][:3]
    assert got["psnr"] == want["psnr"][:3] and got["wspsnr"] == want["wspsnr"][:3]
    assert got["ivpsnr"] == want["ivpsnr"]
    # calc_frame evaluates the IV-SSIM frame family in one fused pass, the shim in separate calls:
    # both FP32 forms are within 1e-6 of the FP64 oracle, and within 1e-7 of each other
    np.testing.assert_allclose(got["ssim"], want["ssim"][:3], rtol=0, atol=1e-7)
    np.testing.assert_allclose(got["msssim"], want["msssim"][:3], rtol=0, atol=1e-7)
    assert abs(got["ivssim"] - want["ivssim"]) <= 1e-7
