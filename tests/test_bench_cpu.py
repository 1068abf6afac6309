"""CPU checks of the measurement entry points that need no GPU: the reference arm of bench.py
prints one JSON line with the contract's keys (the reference's own library where it is built on
this machine, the oracle port otherwise), and the build recognises libraries and objects made
for another machine architecture (they are rebuilt, not loaded)."""
import json
import os
import struct
import subprocess
import sys

from .conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                         timeout=600, check=True).stdout
    line = json.loads(out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["unit"] == "Gpixel/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["pairs"] == 96 and line["config"]["luma_pixels_per_step"] == 354336768


def _elf(path, machine):
    # a minimal 64-bit little-endian ELF header with the given e_machine
    hdr = b"\x7fELF" + bytes([2, 1, 1]) + bytes(9) + struct.pack("<HH", 3, machine) + bytes(44)
    with open(path, "wb") as f:
        f.write(hdr)


def test_build_recognises_foreign_architectures(tmp_path):
    from ivpsnr_gb300 import build
    import platform
    x86, arm = tmp_path / "x86.so", tmp_path / "arm.so"
    _elf(x86, 62)
    _elf(arm, 183)
    here = platform.machine()
    if here in ("x86_64", "AMD64"):
        assert not build._foreign(str(x86)) and build._foreign(str(arm))
    elif here in ("aarch64", "arm64"):
        assert build._foreign(str(x86)) and not build._foreign(str(arm))
    assert build.BUILD.endswith(here)
