"""PyTorch autograd boundary for the GB300 permanent.

``permanent(A)`` takes a square complex128 CUDA tensor and returns perm(A) as
a 0-dim complex tensor.  The forward pass runs the fused permanent+gradient
sweep of libgbperm (gbperm_perm_grad_dev) on the tensor's current stream and
keeps dperm/dA for the backward pass, which returns grad_out * conj(dperm/dA)
(PyTorch's convention for holomorphic functions).  ``permanent_fwd`` is the
forward-only plain kernel.  Tensors stay on the device; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat

_P = ctypes.c_void_p


def _stream_ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _check_input(A: torch.Tensor) -> torch.Tensor:
    if not A.is_cuda:
        raise ValueError("permanent: the matrix must be a CUDA tensor (no CPU path)")
    if A.dim() != 2 or A.shape[0] != A.shape[1]:
        raise ValueError("permanent: square 2-D matrix required")
    return A.to(torch.complex128).contiguous()


def permanent_fwd(A: torch.Tensor, mode: str = "fp64") -> torch.Tensor:
    """Forward-only permanent on the device (gbperm_perm_dev)."""
    A = _check_input(A)
    lib = nat.load()
    n = A.shape[0]
    out = torch.empty(2, dtype=torch.float64, device=A.device)
    ws_bytes = int(lib.gbperm_perm_workspace_size(n, n))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=A.device)
    with torch.cuda.device(A.device):
        nat.check(lib.gbperm_perm_dev(_P(A.data_ptr()), n, n, n, nat.arith_of(mode), _P(out.data_ptr()), None,
                                      _P(ws.data_ptr()), ws_bytes, _stream_ptr(A)))
    return torch.complex(out[0], out[1])


def permanent_and_grad(A: torch.Tensor):
    """(perm, dperm/dA) on the device in one sweep (n <= 32)."""
    A = _check_input(A)
    lib = nat.load()
    n = A.shape[0]
    perm = torch.empty(2, dtype=torch.float64, device=A.device)
    grad = torch.empty((n, n), dtype=torch.complex128, device=A.device)
    ws_bytes = int(lib.gbperm_perm_grad_workspace_size(n))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=A.device)
    with torch.cuda.device(A.device):
        nat.check(lib.gbperm_perm_grad_dev(_P(A.data_ptr()), n, n, _P(perm.data_ptr()), None, _P(grad.data_ptr()),
                                           _P(ws.data_ptr()), ws_bytes, _stream_ptr(A)))
    return torch.complex(perm[0], perm[1]), grad


class Permanent(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A):
        p, g = permanent_and_grad(A)
        ctx.save_for_backward(g)
        return p

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g.conj()


def permanent(A: torch.Tensor) -> torch.Tensor:
    """Differentiable permanent of a square complex CUDA matrix."""
    return Permanent.apply(A)


def clements_unitary(phases: torch.Tensor, m: int) -> torch.Tensor:
    """m x m unitary of a Clements rectangular mesh of m(m-1)/2 Mach-Zehnder
    interferometers, two phases (theta, phi) each: phases has m(m-1) entries.
    Built with differentiable torch ops (complex128, on phases.device)."""
    dev = phases.device
    U = torch.eye(m, dtype=torch.complex128, device=dev)
    k = 0
    for layer in range(m):
        for i in range(layer % 2, m - 1, 2):
            theta, phi = phases[k], phases[k + 1]
            k += 2
            e_phi = torch.exp(1j * phi.to(torch.complex128))
            c = torch.cos(theta).to(torch.complex128)
            s = torch.sin(theta).to(torch.complex128)
            # 2x2 block acting on modes i, i+1
            T = torch.stack([torch.stack([e_phi * c, -s]), torch.stack([e_phi * s, c])])
            rows = U[i:i + 2, :]
            U = torch.cat([U[:i, :], T @ rows, U[i + 2:, :]], dim=0)
    return U
