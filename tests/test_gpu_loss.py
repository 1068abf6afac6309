"""Differentiable IV-PSNR error and IV-SSIM (qmiv_loss_forward / qmiv_loss_backward through
ivpsnr_gb300.loss) against the plain-torch restatement in tests/loss_reference.py:
forward values against its FP64 evaluation, gradients against FP64 autograd of the same
definitions and against FP64 central differences (h = 1e-4) at 64 pixels, 1e-4 relative."""
import numpy as np
import pytest

from . import loss_reference as ref_impl

pytestmark = pytest.mark.gpu


def _pair(n, w, h, seed):
    import torch
    from ivpsnr_gb300 import synth
    rs, ts = [], []
    for i in range(n):  # the generator takes even sizes: odd ones are cropped from the next even size
        r, t = synth.float444(w + w % 2, h + h % 2, seed=seed + i)
        rs.append(np.ascontiguousarray(r[:, :h, :w]))
        ts.append(np.ascontiguousarray(t[:, :h, :w]))
    return torch.from_numpy(np.stack(ts)), torch.from_numpy(np.stack(rs))


def _loss_weights(n, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    return torch.rand((n, 2, 3), generator=g, dtype=torch.float64) + 0.5, torch.rand((n, 2, 3), generator=g, dtype=torch.float64) + 0.5


def _gpu(tst, ref, a, b, **opts):
    import torch
    from ivpsnr_gb300 import loss
    t = tst.cuda().requires_grad_(True)
    sse, ss = loss.iv_metrics(t, ref.cuda(), **opts)
    area = tst.shape[2] * tst.shape[3]
    L = (a.cuda() * sse / area).sum() + (b.cuda() * ss).sum()
    L.backward()
    torch.cuda.synchronize()
    return sse.detach().cpu(), ss.detach().cpu(), t.grad.cpu().double()


def _ref(tst, ref, a, b, dtype, **kw):
    t = tst.to(dtype).requires_grad_(True)
    sse, ss, ks = ref_impl.forward(t, ref.to(dtype), **kw)
    area = tst.shape[2] * tst.shape[3]
    L = (a.to(dtype) * sse / area).sum() + (b.to(dtype) * ss).sum()
    L.backward()
    return sse.detach(), ss.detach(), t.grad.double(), ks


CASES = [(2, 160, 128, 11, {}), (1, 96, 80, 12, {"search_range": 1}), (1, 128, 64, 13, {"ssim_window": 1}),
         (1, 64, 48, 14, {"search_range": 3, "unnoticeable": (0.001, 0.03, 0.03)}),
         # ragged tiles: 100x70 (partial 32x16 tiles, plane a multiple of 4) at the largest range,
         # 99x37 (plane not a multiple of 4: the scalar reduction path)
         (1, 100, 70, 15, {"search_range": 4}), (2, 99, 37, 16, {}),
         # weights other than (4, 1, 1): the search's general form (the default weights take a form
         # with the luma doubled in place of the weight products)
         (1, 96, 64, 17, {"cmp_w_search": (3, 2, 1)})]


def _kw(opts):
    return {"sr": opts.get("search_range", 2), "unc": opts.get("unnoticeable", (0.01, 0.01, 0.01)),
            "win": 11 if opts.get("ssim_window", 0) == 1 else 10,
            "w_search": tuple(float(v) for v in opts.get("cmp_w_search", (4, 1, 1)))}


@pytest.mark.parametrize("n,w,h,seed,opts", CASES)
def test_forward_and_gradients_match_fp64_autograd(gpu_lib, n, w, h, seed, opts):
    import torch
    tst, ref = _pair(n, w, h, seed)
    a, b = _loss_weights(n, seed)
    g_sse, g_ss, g_grad = _gpu(tst, ref, a, b, **opts)
    r_sse, r_ss, r_grad, _ = _ref(tst, ref, a, b, torch.float64, **_kw(opts))
    np.testing.assert_allclose(g_sse.numpy(), r_sse.numpy(), rtol=2e-5, atol=0)
    np.testing.assert_allclose(g_ss.numpy(), r_ss.numpy(), rtol=0, atol=2e-6)
    err = (g_grad - r_grad).abs()
    scale = r_grad.abs().max().item()
    assert (err <= 1e-4 * r_grad.abs() + 1e-4 * scale).float().mean().item() == 1.0, \
        (err.max().item(), scale)
    assert torch.linalg.norm(g_grad - r_grad) <= 1e-4 * torch.linalg.norm(r_grad)


def test_gradients_match_central_differences(gpu_lib):
    """FP64 central differences of the restatement at 64 random (pixel, component) points where
    the +-h perturbation leaves every argmin of both searches unchanged (there the loss is
    smooth; elsewhere the argmin jumps and no derivative exists)."""
    import torch
    n, w, h = 1, 96, 72
    tst, ref = _pair(n, w, h, 21)
    a, b = _loss_weights(n, 21)
    _, _, g_grad = _gpu(tst, ref, a, b)
    area = w * h
    t64, r64 = tst.double(), ref.double()
    hstep = 1e-4

    def L(t):
        sse, ss, ks = ref_impl.forward(t, r64)
        return float(((a * sse / area).sum() + (b * ss).sum()).item()), ks

    _, ks0 = L(t64)
    rng = np.random.default_rng(5)
    fd, an, tried = [], [], 0
    while len(fd) < 64:
        tried += 1
        assert tried < 1000, "too few smooth points"
        y, x, c = int(rng.integers(0, h)), int(rng.integers(0, w)), int(rng.integers(0, 3))
        tp = t64.clone(); tp[0, c, y, x] += hstep
        tm = t64.clone(); tm[0, c, y, x] -= hstep
        lp, kp = L(tp)
        lm, km = L(tm)
        if any(not torch.equal(u, v) for u, v in zip(kp + km, ks0 + ks0)):
            continue
        fd.append((lp - lm) / (2 * hstep))
        an.append(float(g_grad[0, c, y, x]))
    fd, an = np.array(fd), np.array(an)
    floor = 1e-2 * np.sqrt(np.mean(fd ** 2))
    rel = np.abs(an - fd) / np.maximum(np.abs(fd), floor)
    assert rel.max() <= 1e-4, (rel.max(), np.argmax(rel))


def test_gradient_paths_separately(gpu_lib):
    """SSE-only and SSIM-only upstream gradients, so an error in one path is not masked."""
    import torch
    tst, ref = _pair(1, 128, 96, 31)
    a, b = _loss_weights(1, 31)
    z = torch.zeros_like(a)
    for aa, bb in ((a, z), (z, b)):
        _, _, g_grad = _gpu(tst, ref, aa, bb)
        _, _, r_grad, _ = _ref(tst, ref, aa, bb, torch.float64)
        assert torch.linalg.norm(g_grad - r_grad) <= 1e-4 * torch.linalg.norm(r_grad)


def test_matches_fp32_autograd_on_the_gpu(gpu_lib):
    """The plain autograd reference in FP32 on the GPU (the form the benchmark times)."""
    import torch
    tst, ref = _pair(2, 256, 256, 41)
    a, b = _loss_weights(2, 41)
    g_sse, g_ss, g_grad = _gpu(tst, ref, a, b)
    t = tst.cuda().requires_grad_(True)
    sse, ss, _ = ref_impl.forward(t, ref.cuda())
    ((a.cuda().float() * sse / (256 * 256)).sum() + (b.cuda().float() * ss).sum()).backward()
    np.testing.assert_allclose(g_sse.numpy(), sse.detach().double().cpu().numpy(), rtol=1e-4)
    np.testing.assert_allclose(g_ss.numpy(), ss.detach().double().cpu().numpy(), atol=1e-4)
    r = t.grad.double().cpu()
    assert torch.linalg.norm(g_grad - r) <= 1e-2 * torch.linalg.norm(r)


def test_loss_helpers(gpu_lib):
    import torch
    from ivpsnr_gb300 import loss
    tst, ref = _pair(2, 64, 48, 51)
    sse, ss = loss.iv_metrics(tst.cuda(), ref.cuda())
    iv = loss.ivpsnr_db(sse, 64 * 48)
    w = torch.tensor([4.0, 1.0, 1.0], dtype=torch.float64)
    q = (10 * torch.log10(64 * 48 / sse.cpu()) * w).sum(-1) / 6
    assert torch.allclose(iv.cpu(), q.min(dim=1).values)
    assert torch.allclose(loss.ivssim(ss).cpu(), ((ss.cpu() * w).sum(-1) / 6).min(dim=1).values)
    with pytest.raises(ValueError):
        loss.iv_metrics(tst.cuda().double(), ref.cuda().double())


def test_config3_full_size_against_fp64(gpu_lib):
    """The differentiable workload at its own size: 16 FP32 4:4:4 pictures of 1024x1024 in one
    forward and backward, every value and gradient against the FP64 restatement on the GPU (two
    pictures at a time: each picture's terms depend on that picture only), same bars as above."""
    import torch
    n, w, h = 16, 1024, 1024
    tst, ref = _pair(n, w, h, 61)
    a, b = _loss_weights(n, 61)
    g_sse, g_ss, g_grad = _gpu(tst, ref, a, b)
    for i in range(0, n, 2):
        sl = slice(i, i + 2)
        r_sse, r_ss, r_grad, _ = _ref(tst[sl].cuda(), ref[sl].cuda(), a[sl].cuda(), b[sl].cuda(), torch.float64)
        r_sse, r_ss, r_grad = r_sse.cpu(), r_ss.cpu(), r_grad.cpu()
        np.testing.assert_allclose(g_sse[sl].numpy(), r_sse.numpy(), rtol=2e-5, atol=0)
        np.testing.assert_allclose(g_ss[sl].numpy(), r_ss.numpy(), rtol=0, atol=2e-6)
        err = (g_grad[sl] - r_grad).abs()
        scale = r_grad.abs().max().item()
        assert (err <= 1e-4 * r_grad.abs() + 1e-4 * scale).float().mean().item() == 1.0, (i, err.max().item(), scale)
        assert torch.linalg.norm(g_grad[sl] - r_grad) <= 1e-4 * torch.linalg.norm(r_grad), i
        del r_grad, err
        torch.cuda.empty_cache()


def test_config3_central_differences_at_full_size(gpu_lib):
    """FP64 central differences (h = 1e-4) of the restatement at 64 random (pixel, component)
    points of a 1024x1024 picture of the batch, against the GPU gradient, 1e-4 relative. The loss
    difference is summed term by term (errors and per-position SSIM of the two evaluations
    subtracted before the picture sums), so that rounding in million-term sums does not swamp a
    change of order 1e-10. Points where the perturbation moves an argmin are skipped. The central
    differences still carry noise of about 3e-11 at this size (measured: repeating them with h/2
    and h/4 moves them by that much, growing as h shrinks, so it is rounding, not truncation), so
    the relative error is taken against max(|fd|, 10 % of the RMS gradient): at the points whose
    derivative is far below the typical one that noise alone would exceed 1e-4 of it."""
    import torch
    n, w, h = 2, 1024, 1024
    tst, ref = _pair(n, w, h, 71)
    a, b = _loss_weights(n, 71)
    _, _, g_grad = _gpu(tst, ref, a, b)
    area = w * h
    t64, r64 = tst[:1].double().cuda(), ref[:1].double().cuda()
    a0, b0 = a[0].double().cuda(), b[0].double().cuda()
    hstep = 1e-4

    def terms(t):
        with torch.no_grad():
            return ref_impl.forward_maps(t, r64)

    _, _, _, _, ks0 = terms(t64)
    rng = np.random.default_rng(9)
    fd, an, tried = [], [], 0
    while len(fd) < 64:
        tried += 1
        assert tried < 1000, "too few smooth points"
        y, x, c = int(rng.integers(0, h)), int(rng.integers(0, w)), int(rng.integers(0, 3))
        tp = t64.clone(); tp[0, c, y, x] += hstep
        tm = t64.clone(); tm[0, c, y, x] -= hstep
        p, m = terms(tp), terms(tm)
        if any(not torch.equal(u, v) for u, v in zip(p[4] + m[4], ks0 + ks0)):
            continue
        dl = 0.0
        for d, (ep, em) in enumerate(((p[0], m[0]), (p[1], m[1]))):   # SSE: R2T, T2R
            dl += float(((ep * ep - em * em).sum(dim=(2, 3))[0] * a0[d]).sum()) / area
        for d, (sp, sm) in enumerate(((p[2], m[2]), (p[3], m[3]))):   # SSIM: R2T, T2R
            dl += float(((sp - sm).sum(dim=(2, 3))[0] * b0[d]).sum()) / area
        fd.append(dl / (2 * hstep))
        an.append(float(g_grad[0, c, y, x]))
    fd, an = np.array(fd), np.array(an)
    floor = 1e-1 * np.sqrt(np.mean(fd ** 2))
    rel = np.abs(an - fd) / np.maximum(np.abs(fd), floor)
    assert rel.max() <= 1e-4, (rel.max(), np.argmax(rel), fd[np.argmax(rel)], an[np.argmax(rel)])
