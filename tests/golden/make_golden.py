"""Regenerates tests/golden/cases.json from the reference itself.

Inputs are the deterministic synthetic pictures of ivpsnr_gb300.synth (their bytes are
pinned by an md5 per case, so any machine can regenerate them); the expected values come
from the reference's metric library built from its own sources by oracle/build_ref.sh and
driven by oracle/ref_harness.cpp. Run on a machine that has the reference sources:

    oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from ivpsnr_gb300 import synth  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "qmiv_ref_harness")
IO_CHECKER = os.path.join(ROOT, "oracle", "_ref", "qmiv_ref_io")

# name, w, h, bd, seed, generator kwargs, harness options
CASES = [
    # 8-bit widths avoid 64 (mod 128): there the reference's AVX-512 8-bit chroma upsample stores
    # nothing (libs/pmbb-core/src/xPixelOpsAVX512.cpp:293, a shift by 64 in its tail mask)
    ("cfg0_like_8bit_96x48", 96, 48, 8, synth.seed_for(0, 0, 0), {}, {}),
    ("8bit_130x66", 130, 66, 8, 5, {}, {}),
    ("10bit_holes_128x96", 128, 96, 10, 123, {"holes": True}, {}),
    ("10bit_erp_256x128", 256, 128, 10, 77, {"holes": True}, {"erp": True}),
    ("10bit_erp_lat90_128x64", 128, 64, 10, 78, {}, {"erp": True, "lat": 90}),
    ("10bit_sr1_66x34", 66, 34, 10, 6, {}, {"sr": 1}),
    ("10bit_sr3_100x50", 100, 50, 10, 7, {}, {"sr": 3}),
    ("10bit_sr4_96x64", 96, 64, 10, 8, {}, {"sr": 4}),
    ("12bit_96x64", 96, 64, 12, 9, {}, {}),
    ("14bit_64x48", 64, 48, 14, 10, {}, {}),
    ("8bit_tiny_6x4", 6, 4, 8, 12, {}, {}),
    ("8bit_2x2", 2, 2, 8, 11, {}, {}),
    ("10bit_noiseless_64x64", 64, 64, 10, 13, {"noise_sigma": 0.0, "offset": (0.0, 0.0, 0.0)}, {}),
    ("10bit_bigoffset_80x40", 80, 40, 10, 14, {"offset": (9.0, -9.0, 6.0)}, {}),
    ("cfg0_1920x1080_8bit", 1920, 1080, 8, synth.seed_for(0, 0, 0), {}, {}),
    ("cfg1_view3_1920x1080_10bit", 1920, 1080, 10, synth.seed_for(1, 3, 0), {"holes": True}, {}),
]


# masked cases (-im): name, w, h, bd, seed, generator kwargs, harness options, mask kind
MASKED_CASES = [
    ("masked_8bit_ellipses_160x96", 160, 96, 8, 301, {}, {}, "ellipses"),
    ("masked_10bit_graded_128x64", 128, 64, 10, 302, {"holes": True}, {}, "graded"),
    ("masked_10bit_erp_ellipses_256x128", 256, 128, 10, 303, {}, {"erp": True}, "ellipses"),
    ("masked_10bit_sr3_graded_96x64", 96, 64, 10, 304, {}, {"sr": 3}, "graded"),
    ("masked_8bit_cfg0_1920x1080", 1920, 1080, 8, synth.seed_for(0, 0, 0), {}, {}, "ellipses"),
]


def make_mask(w, h, seed, kind):
    """Deterministic 8-bit mask: 'ellipses' (0 inside a few ellipses, 255 elsewhere) or 'graded'
    (values 0..255 from a smooth ramp with a zero band)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    if kind == "ellipses":
        m = np.full((h, w), 255, np.uint16)
        for _ in range(4):
            cx, cy = rng.uniform(0, w), rng.uniform(0, h)
            ax, ay = rng.uniform(0.05, 0.25) * w, rng.uniform(0.05, 0.25) * h
            m[((x - cx) / ax) ** 2 + ((y - cy) / ay) ** 2 <= 1.0] = 0
        return m
    m = np.clip(np.round(255.0 * (0.5 + 0.5 * np.sin(x / (w / 3.0) + y / (h / 2.0)))), 0, 255).astype(np.uint16)
    m[:, w // 3:w // 3 + max(1, w // 10)] = 0
    return m


def run_masked_case(name, w, h, bd, seed, gkw, hopt, kind, tmp):
    ref, tst = synth.pair420(w, h, bd, seed=seed, **gkw)
    a, b, mk = os.path.join(tmp, "a.yuv"), os.path.join(tmp, "b.yuv"), os.path.join(tmp, "m.yuv")
    if bd == 8:
        ref.astype(np.uint8).tofile(a)
        tst.astype(np.uint8).tofile(b)
    else:
        ref.tofile(a)
        tst.tofile(b)
    mask = make_mask(w, h, seed, kind)
    np.concatenate([mask.astype(np.uint8).ravel(), np.zeros(2 * (w // 2) * (h // 2), np.uint8)]).tofile(mk)
    cmd = [HARNESS, "-w", str(w), "-h", str(h), "-bd", str(bd), "-cf", "420", "-i0", a, "-i1", b, "-nth", "2",
           "-im", mk, "-bdm", "8"]
    if hopt.get("erp"):
        cmd += ["-erp", "-lat", str(hopt.get("lat", 180))]
    if "sr" in hopt:
        cmd += ["-sr", str(hopt["sr"])]
    out = json.loads(subprocess.check_output(cmd).decode().splitlines()[0])
    out.pop("frame", None)
    return {
        "name": name, "w": w, "h": h, "bd": bd, "seed": seed, "gen": {k: list(v) if isinstance(v, tuple) else v for k, v in gkw.items()},
        "opts": hopt, "mask": kind, "mask_bd": 8, "input_md5": md5(ref, tst), "mask_md5": md5(mask), "expected": out,
    }


def io_inputs(kind, w, h, bd, seed):
    """Deterministic inputs of the input-side cases: three uint16 planes (colour) or one plane
    with some samples above the bit depth's peak (range)."""
    rng = np.random.default_rng(seed)
    if kind == "color":
        return rng.integers(0, 1 << bd, (3, h, w)).astype(np.uint16)
    return rng.integers(0, (1 << bd) + (1 << bd) // 8, (h, w)).astype(np.uint16)


def run_io_cases(tmp):
    cases = []
    w, h = 64, 32
    for space in range(4):
        for to in (1, 0):
            for bd in (8, 10):
                seed = 1000 + space * 10 + to * 2 + bd
                x = io_inputs("color", w, h, bd, seed)
                a, b = os.path.join(tmp, "c_in.raw"), os.path.join(tmp, "c_out.raw")
                x.tofile(a)
                subprocess.check_call([IO_CHECKER, "color", str(space), str(to), str(bd), str(w), str(h), a, b])
                y = np.fromfile(b, np.uint16).reshape(3, h, w)
                cases.append({"kind": "color", "space": space, "to_ycbcr": to, "bd": bd, "w": w, "h": h, "seed": seed,
                              "input_md5": md5(x), "output_md5": md5(y), "output_head": y[:, 0, :8].tolist()})
    for bd in (8, 10, 12):
        seed = 2000 + bd
        x = io_inputs("range", w, h, bd, seed)
        a, b = os.path.join(tmp, "r_in.raw"), os.path.join(tmp, "r_out.raw")
        x.tofile(a)
        out = json.loads(subprocess.check_output([IO_CHECKER, "range", str(bd), str(w), str(h), a, b]).decode())
        y = np.fromfile(b, np.uint16).reshape(h, w)
        cases.append({"kind": "range", "bd": bd, "w": w, "h": h, "seed": seed, "input_md5": md5(x), "in_range": out["in_range"],
                      "output_md5": md5(y)})
    return cases


def md5(*arrays):
    h = hashlib.md5()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run_case(name, w, h, bd, seed, gkw, hopt, tmp):
    ref, tst = synth.pair420(w, h, bd, seed=seed, **gkw)
    a, b = os.path.join(tmp, "a.yuv"), os.path.join(tmp, "b.yuv")
    if bd == 8:
        ref.astype(np.uint8).tofile(a)
        tst.astype(np.uint8).tofile(b)
    else:
        ref.tofile(a)
        tst.tofile(b)
    cmd = [HARNESS, "-w", str(w), "-h", str(h), "-bd", str(bd), "-cf", "420", "-i0", a, "-i1", b, "-nth", "2",
           "-dump", os.path.join(tmp, "d")]
    if hopt.get("erp"):
        cmd += ["-erp", "-lat", str(hopt.get("lat", 180))]
    if "sr" in hopt:
        cmd += ["-sr", str(hopt["sr"])]
    if w < 16 or h < 16:  # the reference's MS-SSIM pyramid needs 4 halvings of at least 1 pixel
        cmd += ["-ssim", "0"]
    out = json.loads(subprocess.check_output(cmd).decode().splitlines()[0])
    cps = np.fromfile(os.path.join(tmp, "d_f0_cps.bin"), np.int8)
    scp = np.fromfile(os.path.join(tmp, "d_f0_scp.bin"), np.uint16)
    out.pop("frame", None)
    return {
        "name": name, "w": w, "h": h, "bd": bd, "seed": seed, "gen": {k: list(v) if isinstance(v, tuple) else v for k, v in gkw.items()},
        "opts": hopt, "input_md5": md5(ref, tst), "cps_md5": md5(cps), "scp_md5": md5(scp), "expected": out,
    }


def write_ssim_window(src=None):
    """tests/golden/ssim_window.json: the reference's 10x10 SSIM window table (c_FilterF,
    libs/pmbb-ivqm/src/xStructSimConsts.h:31-44) as the FP32 values its source spells out."""
    import re
    src = src or os.environ.get("QMIV_REFERENCE_DIR", "/root/reference")
    txt = open(os.path.join(src, "libs", "pmbb-ivqm", "src", "xStructSimConsts.h")).read()
    vals = [float(v) for v in re.findall(r"([0-9]\.[0-9]+)f", txt)][:121]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ssim_window.json")
    with open(path, "w") as f:
        json.dump({"source": "libs/pmbb-ivqm/src/xStructSimConsts.h:31-44 (c_FilterF, 11x11 storage, 10x10 used)",
                   "values": vals}, f)
    print("wrote", path)


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: oracle/build_ref.sh")
    write_ssim_window()
    tmp = tempfile.mkdtemp()
    cases = [run_case(*c, tmp) for c in CASES]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cases.json")
    with open(path, "w") as f:
        json.dump({"generator": "ivpsnr_gb300.synth.pair420", "reference": "pmbb-ivqm via oracle/ref_harness.cpp",
                   "cases": cases}, f, indent=1)
    print("wrote", path, len(cases), "cases")
    masked = [run_masked_case(*c, tmp) for c in MASKED_CASES]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "masked.json")
    with open(path, "w") as f:
        json.dump({"generator": "ivpsnr_gb300.synth.pair420 + make_golden.make_mask",
                   "reference": "pmbb-ivqm via oracle/ref_harness.cpp -im", "cases": masked}, f, indent=1)
    print("wrote", path, len(masked), "masked cases")
    io = run_io_cases(tmp)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io.json")
    with open(path, "w") as f:
        json.dump({"generator": "make_golden.io_inputs", "reference": "xColorSpace / xPixelOps via oracle/ref_io.cpp",
                   "cases": io}, f, indent=1)
    print("wrote", path, len(io), "input-side cases")


if __name__ == "__main__":
    main()
