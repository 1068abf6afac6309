"""The reference's example pictures stored under tests/golden/fencing/ (see make_fencing.py):
loaders for the flat 8-bit 4:2:0 frames and the fixture of expected values."""
import hashlib
import json
import lzma
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = json.load(open(os.path.join(HERE, "fencing.json")))
W, H = FIXTURE["width"], FIXTURE["height"]


def raw(key):
    """The picture's file bytes (1920x1080 8-bit 4:2:0 planar), checked against its md5."""
    data = lzma.decompress(open(os.path.join(HERE, "fencing", key + ".yuv.xz"), "rb").read())
    assert hashlib.md5(data).hexdigest() == FIXTURE["md5"][key], key
    return data


def flat(key):
    """The picture as a flat uint16 array (Y, then Cb, then Cr), as ivpsnr_gb300.synth returns them."""
    return np.frombuffer(raw(key), np.uint8).astype(np.uint16)


def write(key, path):
    with open(path, "wb") as f:
        f.write(raw(key))
    return path
