"""Plain-torch restatement of the differentiable IV-PSNR error and IV-SSIM (the float-domain
definitions documented with qmiv_loss_forward in include/qmiv_gb300.h), used by the tests as
the autograd reference (FP32 or FP64) and for FP64 central differences.

The corresponding-pixel search is evaluated in FP32 with the same operation order as the CUDA
kernel ((w0 d0^2 + w1 d1^2) + w2 d2^2 from separate tensor ops, argmin = first minimum, the
GCD rounded to FP32 as the kernel holds it), so both pick the same shifts; every other
quantity, the GCD included, is computed in the requested dtype. The SSIM
window is the FP32 factor g (normalised 11-tap Gaussian, sigma 1.5) as an outer product, the
valid region [5, W-5) x [5, H-5), and the sum divided by W*H (xSSIM.cpp:91-140).
"""
import math

import torch
import torch.nn.functional as F


def window_factor(win=10):
    g = torch.tensor([math.exp(-((i - 5) ** 2) / (2 * 1.5 * 1.5)) for i in range(11)], dtype=torch.float64)
    g = (g / g.sum()).to(torch.float32)
    return g[:win]


def _shifts(x, sr):
    """[n, 3, H, W] -> [n, 3, K, H, W]: x at (p + s), s row-major over [-sr, sr]^2, borders clamped."""
    h, w = x.shape[-2:]
    xp = F.pad(x, (sr, sr, sr, sr), mode="replicate")
    return torch.stack([xp[:, :, dy:dy + h, dx:dx + w] for dy in range(2 * sr + 1) for dx in range(2 * sr + 1)], dim=2)


def _werr(d, w):
    d32 = d.detach().float()
    return (w[0] * (d32[:, 0] * d32[:, 0]) + w[1] * (d32[:, 1] * d32[:, 1])) + w[2] * (d32[:, 2] * d32[:, 2])


def _gather(stack, k):
    n, c, _, h, w = stack.shape
    return torch.gather(stack, 2, k[:, None, None].expand(n, c, 1, h, w)).squeeze(2)


def ssim_map(x, y, win=10, c1=1e-4, c2=9e-4):
    """Per-position SSIM L*CS of each plane pair of [n, 3, H, W] tensors over the valid region
    [5, H-5) x [5, W-5) -> [n, 3, H-10, W-10] (Max = 1)."""
    n, c, h, w = x.shape
    g = window_factor(win).to(x.dtype).to(x.device)
    k2 = torch.outer(g, g)[None, None].expand(c, 1, win, win)
    conv = lambda t: F.conv2d(t, k2, groups=c)[:, :, :h - 10, :w - 10]
    mx, my = conv(x), conv(y)
    exx, eyy, exy = conv(x * x), conv(y * y), conv(x * y)
    vx, vy, cov = exx - mx * mx, eyy - my * my, exy - mx * my
    return ((2 * mx * my + c1) / (mx * mx + my * my + c1)) * ((2 * cov + c2) / (vx + vy + c2))


def ssim(x, y, win=10, c1=1e-4, c2=9e-4):
    """Picture SSIM of each plane pair of [n, 3, H, W] tensors -> [n, 3] (L*CS, Max = 1)."""
    h, w = x.shape[-2:]
    return ssim_map(x, y, win, c1, c2).sum(dim=(2, 3)) / (h * w)


def forward(tst, ref, sr=2, w_search=(4.0, 1.0, 1.0), unc=(0.01, 0.01, 0.01), win=10):
    """(sse[n, 2, 3], ssim[n, 2, 3]) in tst's dtype; differentiable with respect to tst."""
    e1, e0, s_r2t, s_t2r, ks = forward_maps(tst, ref, sr, w_search, unc, win)
    h, w = tst.shape[-2:]
    sse = torch.stack([(e1 * e1).sum(dim=(2, 3)), (e0 * e0).sum(dim=(2, 3))], dim=1)
    ss = torch.stack([s_r2t.sum(dim=(2, 3)), s_t2r.sum(dim=(2, 3))], dim=1) / (h * w)
    return sse, ss, ks


def forward_maps(tst, ref, sr=2, w_search=(4.0, 1.0, 1.0), unc=(0.01, 0.01, 0.01), win=10):
    """The terms before their picture sums: the R2T and T2R errors at the argmin [n, 3, H, W], the
    per-position SSIM of both directions [n, 3, H-10, W-10], and the argmin maps. Differences of
    two evaluations are taken term by term before summing, which keeps central differences of the
    picture sums free of the summation's rounding at large sizes."""
    dt = tst.dtype
    n, _, h, w = tst.shape
    m = (ref.double() - tst.double()).mean(dim=(2, 3)).to(dt)
    u = torch.tensor(unc, dtype=dt, device=tst.device)
    gcd = torch.clamp(m, -u, u)
    g4 = gcd[:, :, None, None]
    wt = torch.tensor(w_search, dtype=torch.float32, device=tst.device)
    rs, ts = _shifts(ref, sr), _shifts(tst, sr)
    # R2T: tested pixels (+ GCD) searched in the reference
    d1 = (tst + g4).unsqueeze(2) - rs
    d1_32 = (tst.float() + g4.float()).unsqueeze(2) - rs.float()
    k1 = _werr(d1_32, wt).argmin(dim=1)
    e1 = _gather(d1, k1)
    # T2R: reference pixels (- GCD) searched in the tested picture
    d0 = (ref - g4).unsqueeze(2) - ts
    d0_32 = (ref.float() - g4.float()).unsqueeze(2) - ts.float()
    k0 = _werr(d0_32, wt).argmin(dim=1)
    e0 = _gather(d0, k0)
    scp1 = torch.clamp(_gather(rs, k1) - g4, 0.0, 1.0)
    scp0 = torch.clamp(_gather(ts, k0) + g4, 0.0, 1.0)
    return e1, e0, ssim_map(ref, scp0, win), ssim_map(tst, scp1, win), (k1, k0)
