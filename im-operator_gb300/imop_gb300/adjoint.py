"""Differentiable calibration chain on the GPU: torch.autograd.Function wrappers over the C ABI.

    render(isp, desc, theta, raw)            -> t, shape (n_frames, h, w, 3), differentiable in theta
    l2_loss(isp, desc, theta, raw, target)   -> sum((t - target)^2), one fused adjoint launch

theta is a float32 CUDA tensor of imop_adjoint_param_count(desc) values (layout in
include/imop_isp.h: bl[4], wb[3], ccm[9], grid[gh][gw][4], knots[33]); raw holds the n_frames input
frames back to back (uint8 CUDA tensor).  The kernels run on torch's current stream.
"""
import ctypes as C

import torch

from . import abi, check, lib


def param_count(desc):
    return lib().imop_adjoint_param_count(C.byref(desc))


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _check_inputs(desc, theta, raw):
    if theta.dtype != torch.float32 or not theta.is_cuda or not theta.is_contiguous():
        raise ValueError("theta must be a contiguous float32 CUDA tensor")
    if theta.numel() != param_count(desc):
        raise ValueError(f"theta has {theta.numel()} values, the chain takes {param_count(desc)}")
    if raw.dtype != torch.uint8 or not raw.is_cuda or not raw.is_contiguous():
        raise ValueError("raw must be a contiguous uint8 CUDA tensor")


def render_forward(isp, desc, theta, raw):
    _check_inputs(desc, theta, raw)
    out = torch.empty((desc.n_frames, desc.height, desc.width, 3), dtype=torch.float32, device=theta.device)
    check(lib().imop_isp_render_device(isp.h, C.byref(desc), theta.data_ptr(), raw.data_ptr(), out.data_ptr(),
                                       _stream()))
    return out


def backward(isp, desc, theta, raw, ref, mode):
    """(loss, grad) as CUDA tensors: loss is sum (t - ref)^2 (mode ADJ_TARGET) or sum t * ref
    (mode ADJ_UPSTREAM, ref = dL/dt); grad = d loss / d theta."""
    _check_inputs(desc, theta, raw)
    ref = ref.contiguous()
    if ref.dtype != torch.float32 or ref.numel() != desc.n_frames * desc.height * desc.width * 3:
        raise ValueError("ref must be float32 with n_frames * h * w * 3 values")
    loss = torch.empty(1, dtype=torch.float32, device=theta.device)
    grad = torch.empty_like(theta)
    check(lib().imop_isp_backward_device(isp.h, C.byref(desc), theta.data_ptr(), raw.data_ptr(), ref.data_ptr(),
                                         mode, loss.data_ptr(), grad.data_ptr(), _stream()))
    return loss[0], grad


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, raw, isp, desc):
        ctx.isp, ctx.desc = isp, desc
        ctx.save_for_backward(theta, raw)
        return render_forward(isp, desc, theta.detach().contiguous(), raw)

    @staticmethod
    def backward(ctx, grad_t):
        theta, raw = ctx.saved_tensors
        _, g = backward(ctx.isp, ctx.desc, theta.detach().contiguous(), raw, grad_t.float(), abi.ADJ_UPSTREAM)
        return g, None, None, None


class _L2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, raw, target, isp, desc):
        loss, g = backward(isp, desc, theta.detach().contiguous(), raw, target, abi.ADJ_TARGET)
        ctx.save_for_backward(g)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        (g,) = ctx.saved_tensors
        return g * grad_loss, None, None, None, None


def render(isp, desc, theta, raw):
    return _Render.apply(theta, raw, isp, desc)


def l2_loss(isp, desc, theta, raw, target):
    return _L2.apply(theta, raw, target, isp, desc)
