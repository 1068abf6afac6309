"""Regenerates tests/golden/fencing/ and tests/golden/fencing.json from the reference itself.

The reference ships four 1920x1080 8-bit 4:2:0 pictures (the first frame of view 8 of the
Fencing multiview sequence: original, JPEG-compressed, synthesized from views 7 and 9, and an
object mask) together with its published PSNR-Y / IV-PSNR values (example/README.md:44-47,67-69).
They are the only real-content test vectors the reference holds for the metric path. This script
stores them LZMA-compressed (about 2.8 MB for the four) so that the GPU tests can reproduce the
published values on a machine without the reference sources, and records what the reference's own
build (oracle/build_ref.sh, driven by oracle/ref_harness.cpp) gives on them at full precision,
including the md5 of its CPS argmin maps and shift-compensated pictures.

    oracle/build_ref.sh && python tests/golden/make_fencing.py [REFERENCE_SOURCE_DIR]

(default: $QMIV_REFERENCE_DIR, else /root/reference)
"""
import hashlib
import json
import lzma
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "qmiv_ref_harness")
OUT = os.path.join(HERE, "fencing")
W, H = 1920, 1080
PICTURES = {
    "original": "Fencing_v8_original_1920x1080_yuv420p.yuv",
    "origJpgCompressed": "Fencing_v8_origJpgCompressed_1920x1080_yuv420p.yuv",
    "synthesized": "Fencing_v8_synthesized_1920x1080_yuv420p.yuv",
    "objectsMask": "Fencing_v8_objectsMask_1920x1080_yuv420p.yuv",
}


def md5(b):
    return hashlib.md5(b).hexdigest()


def harness(args, tmp):
    out = subprocess.check_output([HARNESS, "-w", str(W), "-h", str(H), "-bd", "8", "-cf", "420", "-nth", "8"] + args)
    return json.loads(out.decode().splitlines()[0])


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QMIV_REFERENCE_DIR", "/root/reference")
    example = os.path.join(src, "example")
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: oracle/build_ref.sh")
    os.makedirs(OUT, exist_ok=True)
    raw = {}
    for key, name in PICTURES.items():
        data = open(os.path.join(example, name), "rb").read()
        raw[key] = data
        with open(os.path.join(OUT, key + ".yuv.xz"), "wb") as f:
            f.write(lzma.compress(data, preset=9 | lzma.PRESET_EXTREME))
    tmp = tempfile.mkdtemp()
    path = lambda k: os.path.join(example, PICTURES[k])
    cases = []
    for tst in ("origJpgCompressed", "synthesized"):
        e = harness(["-i0", path("original"), "-i1", path(tst), "-dump", os.path.join(tmp, "d")], tmp)
        e.pop("frame", None)
        cps = np.fromfile(os.path.join(tmp, "d_f0_cps.bin"), np.int8)
        scp = np.fromfile(os.path.join(tmp, "d_f0_scp.bin"), np.uint16)
        cases.append({"pic0": "original", "pic1": tst, "expected": e,
                      "cps_md5": md5(cps.tobytes()), "scp_md5": md5(scp.tobytes())})
    e = harness(["-i0", path("original"), "-i1", path("synthesized"), "-im", path("objectsMask")], tmp)
    e.pop("frame", None)
    cases.append({"pic0": "original", "pic1": "synthesized", "mask": "objectsMask", "expected": e})
    doc = {
        "source": "reference example pictures (example/README.md), first frame of Fencing view 8, "
                  "1920x1080 8-bit 4:2:0; expected values from the reference build (oracle/build_ref.sh)",
        "width": W, "height": H, "bitdepth": 8,
        "md5": {k: md5(v) for k, v in raw.items()},
        "cases": cases,
    }
    with open(os.path.join(HERE, "fencing.json"), "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote", OUT, "and fencing.json")


if __name__ == "__main__":
    main()
