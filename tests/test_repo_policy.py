"""Repository rules that can be checked without a GPU: every ncu command recorded under profiles/
leaves the GPU clocks alone (--clock-control none), and the product package neither imports nor
loads the CPU oracle (the oracle is test infrastructure; the library has no CPU fallback)."""
import glob
import os
import re

from .conftest import ROOT


def _ncu_commands(text):
    """ncu command lines of a profile summary, continuation lines joined."""
    joined = re.sub(r"\\\n\s*", " ", text)
    return [ln.strip() for ln in joined.splitlines() if re.match(r"\s*ncu\s", ln)]


def test_profiles_record_ncu_commands_that_leave_clocks_alone():
    seen = 0
    for path in glob.glob(os.path.join(ROOT, "profiles", "*.md")):
        for cmd in _ncu_commands(open(path).read()):
            seen += 1
            assert "--clock-control none" in cmd, (os.path.basename(path), cmd)
    assert seen >= 8


def test_product_package_does_not_use_the_oracle():
    pkg = os.path.join(ROOT, "ivpsnr_gb300")
    files = glob.glob(os.path.join(pkg, "*.py")) + glob.glob(os.path.join(pkg, "csrc", "*"))
    assert files
    for path in files:
        if os.path.isdir(path):
            continue
        text = open(path, errors="replace").read()
        assert not re.search(r"^\s*(from|import)\s+oracle\b", text, re.M), path
        assert "liboq" not in text and "qmiv_oracle" not in text, path
