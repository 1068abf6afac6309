"""In-tree build of the native libraries (no CMake, no setuptools).

* libqmiv_gb300.so : the CUDA kernels for sm_103a plus the C-ABI host code (nvcc).
* libqmiv_synth.so : the deterministic synthetic-picture generator (host C).

Translation units compile in parallel; objects go to ivpsnr_gb300/_build/<machine>/ and are
reused while newer than their sources and headers. A library or object built for another
architecture (a working tree copied between an x86-64 and an aarch64 host) is never reused: the
object folder is per machine, and a library whose ELF machine differs from the host's is rebuilt.
"""
import concurrent.futures as cf
import glob
import os
import platform
import shutil
import struct
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine() or "host")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libqmiv_gb300.so")
SYNTH = os.path.join(HERE, "libqmiv_synth.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqmiv_gb300.so")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


_ELF_MACHINE = {"x86_64": 62, "AMD64": 62, "aarch64": 183, "arm64": 183}


def _foreign(path):
    """True when path is an ELF file built for another machine than this host."""
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if want is None or len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    endian = "<" if head[5] == 1 else ">"
    return struct.unpack(endian + "H", head[18:20])[0] != want


def _stale(out, deps):
    if not os.path.exists(out) or _foreign(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "qmiv_*.cpp")))
    steps = []
    objs = []
    for src in cu + cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                   "-I", INCLUDE, "-diag-suppress", "177", "-c", src, "-o", obj]
            steps.append(cmd)
    synth_src = os.path.join(CSRC, "qmiv_synth.c")
    synth_cmd = None
    if _stale(SYNTH, [synth_src, os.path.join(CSRC, "qmiv_synth.h")]):
        synth_cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                     synth_src, "-o", SYNTH, "-lm"]
    with cf.ThreadPoolExecutor(max_workers=jobs or max(4, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, c) for c in steps]
        if synth_cmd:
            futs.append(ex.submit(_run, synth_cmd))
        for f in futs:
            out = f.result()
            if verbose and out.strip():
                print(out)
    exports = os.path.join(CSRC, "exports.map")
    if steps or not os.path.exists(LIB) or _foreign(LIB) or _stale(LIB, [exports]):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xlinker", "--version-script=" + exports,
                                                              "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(verbose=True), "%.1fs" % (time.time() - t))
