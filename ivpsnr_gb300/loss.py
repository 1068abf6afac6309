"""IV-PSNR error and IV-SSIM as differentiable functions of a tested picture (torch.autograd).

The forward and backward passes are the library's CUDA kernels (qmiv_loss_forward /
qmiv_loss_backward); this module only allocates the workspace and output tensors with torch
and wires the calls into autograd. Pictures are FP32 4:4:4 tensors [n, 3, H, W] in [0, 1] on
a CUDA device; `ref` is treated as a constant.

    sse, ssim = iv_metrics(tst, ref)          # [n, 2, 3] each, float64; direction 0 = R2T, 1 = T2R
    loss = -ivpsnr_db(sse, H * W).mean()      # or 1 - ivssim(ssim).mean()
    loss.backward()
"""
import ctypes

import torch

from . import _abi, default_options


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class IVMetricsFunction(torch.autograd.Function):
    """(tst, ref, options) -> (sse[n,2,3], ssim[n,2,3]); gradients flow to tst only."""

    @staticmethod
    def forward(ctx, tst, ref, opts):
        if tst.dim() != 4 or tst.shape[1] != 3 or tst.shape != ref.shape:
            raise ValueError("tst and ref must be [n, 3, H, W] tensors of the same shape")
        if tst.dtype != torch.float32 or ref.dtype != torch.float32 or not tst.is_cuda or not ref.is_cuda:
            raise ValueError("tst and ref must be float32 CUDA tensors")
        tst = tst.contiguous()
        ref = ref.contiguous()
        n, _, h, w = tst.shape
        lib = _abi.load()
        size = ctypes.c_size_t()
        _abi.check(lib.qmiv_loss_workspace_size(n, w, h, ctypes.byref(opts), ctypes.byref(size)), "qmiv_loss_workspace_size")
        ws = torch.empty(size.value, dtype=torch.uint8, device=tst.device)
        sse = torch.empty((n, 2, 3), dtype=torch.float64, device=tst.device)
        ssim = torch.empty((n, 2, 3), dtype=torch.float64, device=tst.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(tst.device).cuda_stream)
        _abi.check(lib.qmiv_loss_forward(_ptr(tst), _ptr(ref), n, w, h, ctypes.byref(opts), _ptr(ws), size.value,
                                         _ptr(sse), _ptr(ssim), stream), "qmiv_loss_forward")
        ctx.save_for_backward(tst, ref, ws)
        ctx.opts = opts
        return sse, ssim

    @staticmethod
    def backward(ctx, g_sse, g_ssim):
        tst, ref, ws = ctx.saved_tensors
        n, _, h, w = tst.shape
        g_sse = torch.zeros((n, 2, 3), dtype=torch.float64, device=tst.device) if g_sse is None else g_sse.contiguous().double()
        g_ssim = torch.zeros((n, 2, 3), dtype=torch.float64, device=tst.device) if g_ssim is None else g_ssim.contiguous().double()
        g_tst = torch.empty_like(tst)
        lib = _abi.load()
        stream = ctypes.c_void_p(torch.cuda.current_stream(tst.device).cuda_stream)
        _abi.check(lib.qmiv_loss_backward(_ptr(tst), _ptr(ref), n, w, h, ctypes.byref(ctx.opts), _ptr(ws), ws.numel(),
                                          _ptr(g_sse), _ptr(g_ssim), _ptr(g_tst), stream), "qmiv_loss_backward")
        return g_tst, None, None


def iv_metrics(tst, ref, **opts):
    """Per image, direction (0 = R2T, 1 = T2R) and component: SSE at the corresponding-pixel
    argmin and SSIM against the shift-compensated picture. Options as for Processor
    (search_range, cmp_w_search, unnoticeable, ssim_window)."""
    return IVMetricsFunction.apply(tst, ref, default_options(**opts))


def _wmean(x, w_avg):
    """Weighted mean over the last (component) axis with Python-scalar weights: no weight tensor
    is made on the device, so the helpers add no host-to-device copy to a training step."""
    w0, w1, w2 = (float(v) for v in w_avg)
    return (x[..., 0] * w0 + x[..., 1] * w1 + x[..., 2] * w2) / (w0 + w1 + w2)


def ivpsnr_db(sse, area, w_avg=(4, 1, 1)):
    """IV-PSNR per image from the [n, 2, 3] SSE: min over directions of the weighted
    10 log10(area / SSE_c) (Max = 1; xIVPSNR.cpp:100-133)."""
    return _wmean(10.0 * torch.log10(area / sse), w_avg).min(dim=1).values


def ivssim(ssim, w_avg=(4, 1, 1)):
    """IV-SSIM per image from the [n, 2, 3] SSIM values: min over directions of the weighted
    mean (xSSIM.cpp:192-210)."""
    return _wmean(ssim, w_avg).min(dim=1).values
