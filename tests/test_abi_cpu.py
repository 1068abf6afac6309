"""CPU tests of the C-ABI library: it loads, exports every entry point include/*.h declares,
reports defaults and rejects bad arguments without touching a GPU."""
import ctypes
import glob
import os
import re

import pytest

from .conftest import ROOT


def _declared_symbols():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(hdr).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(qmiv_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from ivpsnr_gb300 import _abi
    return _abi.load()


def test_library_exports_every_declared_symbol(lib):
    names = _declared_symbols()
    assert len(names) >= 20
    raw = ctypes.CDLL(os.path.join(ROOT, "ivpsnr_gb300", "libqmiv_gb300.so"))
    missing = [n for n in sorted(names) if not hasattr(raw, n)]
    assert not missing, missing


def test_library_exports_nothing_but_the_c_abi(lib):
    """The version script keeps launchers, kernel stubs and the static CUDA runtime local."""
    import shutil
    import subprocess
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "ivpsnr_gb300", "libqmiv_gb300.so")],
                         stdout=subprocess.PIPE, text=True, check=True).stdout
    funcs = {ln.split()[-1] for ln in out.splitlines() if len(ln.split()) == 3 and ln.split()[1] in "TW"}
    assert funcs == _declared_symbols(), sorted(funcs ^ _declared_symbols())


def test_python_binding_declares_every_symbol():
    from ivpsnr_gb300 import _abi
    declared = {n for n, _, _ in _abi.SIGNATURES}
    assert _declared_symbols() <= declared


def test_defaults_match_reference(lib):
    from ivpsnr_gb300 import _abi
    o = _abi.Options()
    lib.qmiv_default_options(ctypes.byref(o))
    assert o.search_range == 2                       # xCorrespPixelShift.h:32
    assert list(o.cmp_w_search) == [4, 1, 1, 0]      # xCorrespPixelShift.h:33
    assert list(o.cmp_w_avg) == [4, 1, 1, 0]
    assert [round(x, 6) for x in o.unnoticeable] == [0.01, 0.01, 0.01, 0.0]  # xGlobClrDiff.h:20
    assert (o.lon_deg, o.lat_deg, o.fake_exact, o.legacy_ws8, o.use_ws, o.scratch_metrics) == (360, 180, 1, 0, 0, 63)


def test_status_strings_and_version(lib):
    assert lib.qmiv_abi_version() == 1
    for s in range(7):
        assert lib.qmiv_status_str(s)


def test_null_arguments_are_rejected(lib):
    from ivpsnr_gb300 import _abi
    assert lib.qmiv_create(None, None, 64, 64, 1) == _abi.QMIV_BAD_ARG
    assert lib.qmiv_destroy(None) == _abi.QMIV_OK
    r = _abi.FrameResult()
    assert lib.qmiv_calc_frame(None, None, None, 0, ctypes.byref(r), None) == _abi.QMIV_BAD_ARG
    assert lib.qmiv_finish_sequence(None, None) == _abi.QMIV_BAD_ARG
    assert lib.qmiv_set_cps_variant(None, 0) == _abi.QMIV_BAD_ARG


def test_bad_options_are_rejected_before_any_device_call(lib):
    from ivpsnr_gb300 import _abi
    o = _abi.Options()
    lib.qmiv_default_options(ctypes.byref(o))
    h = ctypes.c_void_p()
    o.search_range = 99
    assert lib.qmiv_create(ctypes.byref(h), ctypes.byref(o), 64, 64, 1) == _abi.QMIV_BAD_ARG
    lib.qmiv_default_options(ctypes.byref(o))
    o.cmp_w_avg[0] = o.cmp_w_avg[1] = o.cmp_w_avg[2] = 0
    assert lib.qmiv_create(ctypes.byref(h), ctypes.byref(o), 64, 64, 1) == _abi.QMIV_BAD_ARG
    lib.qmiv_default_options(ctypes.byref(o))
    assert lib.qmiv_create(ctypes.byref(h), ctypes.byref(o), 1, 64, 1) == _abi.QMIV_BAD_ARG
    assert lib.qmiv_create(ctypes.byref(h), ctypes.byref(o), 64, 64, 0) == _abi.QMIV_BAD_ARG


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ivpsnr_gb300 import _abi
    h = ctypes.c_void_p()
    assert lib.qmiv_create(ctypes.byref(h), None, 64, 64, 1) == _abi.QMIV_CUDA_ERROR
    assert not h.value
    assert lib.qmiv_last_error()


def test_cps_variant_table(lib):
    import ivpsnr_gb300 as q
    names = q.cps_variants()
    assert names[0] == "cps_generic"
    assert any(n.startswith("tma420_sr2") for n in names)
    assert len(set(names)) == len(names)
