"""torch.autograd binding of the differentiable fp32 Floyd-Warshall
(fw_forward_f32 / fw_backward in libfw103.so).

    D = shortest_paths(W)          # W: float32 CUDA tensor, (n, n) or (B, n, n); +inf = no edge
    D.backward(G)                  # W.grad[u, v] = sum of G[i, j] over the pairs whose
                                   # recorded shortest path uses edge (u, v)

The forward records int32 next hops (kept for the backward; also returned by
``forward_with_next_hops``). Gradients flow to present edges only.
"""
from __future__ import annotations

import ctypes

import torch

from . import _check, _ptr, lib


def _setup():
    L = lib()
    if not getattr(L, "_fw_diff_ready", False):
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        L.fw_forward_f32.argtypes = [vp, vp, i64, i64, vp]
        L.fw_forward_f32.restype = ctypes.c_int
        L.fw_backward.argtypes = [vp, vp, vp, i64, i64, vp, vp]
        L.fw_backward.restype = ctypes.c_int
        L._fw_diff_ready = True
    return L


def _shape(W: torch.Tensor):
    if W.dim() == 2:
        return 1, W.shape[0]
    if W.dim() == 3:
        return W.shape[0], W.shape[1]
    raise ValueError("expected (n, n) or (B, n, n)")


def forward_with_next_hops(W: torch.Tensor, stream=None):
    """(D, nh) without autograd: distances and next hops of fp32 weights W."""
    if W.dtype != torch.float32 or not W.is_cuda:
        raise ValueError("W must be a float32 CUDA tensor")
    batch, n = _shape(W)
    if W.shape[-1] != n:
        raise ValueError("W must be square")
    D = W.contiguous().clone()
    nh = torch.empty(D.shape, dtype=torch.int32, device=D.device)
    s = (stream or torch.cuda.current_stream()).cuda_stream
    _check(_setup().fw_forward_f32(_ptr(D), _ptr(nh), n, batch, s))
    return D, nh


def backward_from_next_hops(G: torch.Tensor, nh: torch.Tensor, stream=None, check_walks: bool = False):
    """dL/dW from dL/dD = G and the forward's next hops."""
    batch, n = _shape(nh)
    if nh.dtype != torch.int32 or not nh.is_cuda or nh.shape[-1] != n:
        raise ValueError("nh must be the forward's square int32 CUDA next-hop tensor")
    if tuple(G.shape) != tuple(nh.shape) or G.device != nh.device:
        raise ValueError(f"G must have nh's shape {tuple(nh.shape)} and device, got {tuple(G.shape)} on {G.device}")
    nh = nh.contiguous()
    G = G.contiguous().to(torch.float32)
    dW = torch.empty(nh.shape, dtype=torch.float32, device=nh.device)
    bad = torch.zeros(1, dtype=torch.int32, device=nh.device) if check_walks else None
    s = (stream or torch.cuda.current_stream()).cuda_stream
    _check(_setup().fw_backward(_ptr(G), _ptr(nh), _ptr(dW), n, batch, _ptr(bad) if bad is not None else None, s))
    if check_walks:
        return dW, int(bad.item())
    return dW


class FloydWarshall(torch.autograd.Function):
    @staticmethod
    def forward(ctx, W):
        D, nh = forward_with_next_hops(W)
        ctx.save_for_backward(nh)
        ctx.mark_non_differentiable(nh)
        return D, nh

    @staticmethod
    def backward(ctx, gD, gnh):
        (nh,) = ctx.saved_tensors
        return backward_from_next_hops(gD, nh)


def shortest_paths(W: torch.Tensor) -> torch.Tensor:
    """Differentiable all-pairs shortest-path distances of fp32 weights W."""
    D, _ = FloydWarshall.apply(W)
    return D
