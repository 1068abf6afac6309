"""The oracle's restatement of the input-side operations against the reference's own output
(tests/golden/io.json, made by tests/golden/make_golden.py through oracle/ref_io.cpp):
colour conversion (every colour space, both directions, 8 and 10 bit) and range
check / clipping; plus the raw 4:2:2 frame unpacking against its closed form."""
import json
import os

import numpy as np
import pytest

from .golden.make_golden import io_inputs, md5

IO = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "io.json")))


@pytest.mark.parametrize("case", IO["cases"], ids=["%s_%d" % (c["kind"], i) for i, c in enumerate(IO["cases"])])
def test_oracle_matches_reference_io(oq, case):
    x = io_inputs(case["kind"], case["w"], case["h"], case["bd"], case["seed"])
    assert md5(x) == case["input_md5"]
    if case["kind"] == "color":
        y = oq.color_convert(list(x), case["bd"], case["space"], case["to_ycbcr"])
        assert y[:, 0, :8].tolist() == case["output_head"]
        assert md5(y) == case["output_md5"]
    else:
        n, y = oq.range_clip(x, case["bd"])
        assert (n == 0) == bool(case["in_range"])
        assert md5(y) == case["output_md5"]


@pytest.mark.parametrize("bps,bd", [(1, 8), (2, 10)])
def test_oracle_unpacks_422(oq, bps, bd):
    w, h = 12, 6
    rng = np.random.default_rng(bd)
    y = rng.integers(0, 1 << bd, (h, w)).astype(np.uint16)
    cb = rng.integers(0, 1 << bd, (h, w // 2)).astype(np.uint16)
    cr = rng.integers(0, 1 << bd, (h, w // 2)).astype(np.uint16)
    dt = np.uint8 if bps == 1 else np.dtype("<u2")
    raw = np.concatenate([y.ravel(), cb.ravel(), cr.ravel()]).astype(dt).tobytes()
    out = oq.unpack_frame(raw, w, h, bps, 422)
    assert np.array_equal(out[0], y)
    assert np.array_equal(out[1], np.repeat(cb, 2, axis=1)) and np.array_equal(out[2], np.repeat(cr, 2, axis=1))
