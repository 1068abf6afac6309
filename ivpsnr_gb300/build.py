"""In-tree build of the native libraries (no CMake, no setuptools).

* libqmiv_gb300.so : the CUDA kernels for sm_103a plus the C-ABI host code (nvcc).
* libqmiv_synth.so : the deterministic synthetic-picture generator (host C).

Translation units compile in parallel; objects go to ivpsnr_gb300/_build/ and are reused
while newer than their sources and headers.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
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


def _stale(out, deps):
    if not os.path.exists(out):
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
    if steps or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(verbose=True), "%.1fs" % (time.time() - t))
