"""The float-domain restatement used as the autograd reference (tests/loss_reference.py) is
pinned to the integer oracle: SSIM is scale invariant when C1, C2 scale with Max^2, so the
FP64 reference on samples / Max must reproduce the oracle's SSIM of the integer samples."""
import numpy as np
import pytest

from . import loss_reference as ref_impl


@pytest.mark.parametrize("w,h,bd,window", [(96, 64, 8, 0), (80, 48, 10, 0), (64, 40, 10, 1)])
def test_float_ssim_reproduces_integer_oracle(oq, w, h, bd, window):
    import torch
    from ivpsnr_gb300 import synth
    ref, tst = synth.pair420(w, h, bd, seed=900 + w)
    p0 = oq.upsample420(synth.split420(ref, w, h), w, h)
    p1 = oq.upsample420(synth.split420(tst, w, h), w, h)
    mx = float((1 << bd) - 1)
    x = torch.from_numpy(np.stack([p.astype(np.float64) for p in p1]))[None] / mx
    y = torch.from_numpy(np.stack([p.astype(np.float64) for p in p0]))[None] / mx
    got = ref_impl.ssim(x, y, win=11 if window else 10)[0].numpy()
    want = [oq.ssim_plane(p1[c], p0[c], bd, True, window) for c in range(3)]
    # the oracle uses the FP32 2-D table (xStructSimConsts.h); the restatement the FP32 1-D factor
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-7)


def test_reference_gradient_is_finite_and_nonzero():
    import torch
    from ivpsnr_gb300 import synth
    r, t = synth.float444(64, 48, seed=3)
    T = torch.from_numpy(t)[None].double().requires_grad_(True)
    sse, ss, _ = ref_impl.forward(T, torch.from_numpy(r)[None].double())
    (sse.sum() + ss.sum()).backward()
    assert torch.isfinite(T.grad).all() and T.grad.abs().max() > 0
