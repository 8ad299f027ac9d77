"""PyTorch autograd boundary for the GB300 permanent.

``permanent(A)`` takes a square complex128 CUDA tensor and returns perm(A) as
a 0-dim complex tensor; given a (B, n, n) stack it returns the B permanents
from one set of launches.  The forward pass runs the fused
permanent+gradient sweep of libgbperm (gbperm_perm_grad_dev /
gbperm_perm_grad_batched_dev) on the tensor's current stream and keeps
dperm/dA for the backward pass, which returns grad_out * conj(dperm/dA)
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


def permanents_and_grads(A: torch.Tensor):
    """(perms[B], dperm/dA[B, n, n]) of a (B, n, n) stack in one sweep per
    matrix and one set of launches (n <= 32)."""
    if not A.is_cuda:
        raise ValueError("permanent: the matrices must be a CUDA tensor (no CPU path)")
    if A.dim() != 3 or A.shape[1] != A.shape[2]:
        raise ValueError("permanent: a (B, n, n) stack of square matrices is required")
    A = A.to(torch.complex128).contiguous()
    lib = nat.load()
    count, n = A.shape[0], A.shape[1]
    perms = torch.empty((count, 2), dtype=torch.float64, device=A.device)
    grads = torch.empty((count, n, n), dtype=torch.complex128, device=A.device)
    if count == 0:
        return torch.complex(perms[:, 0], perms[:, 1]), grads
    ws_bytes = int(lib.gbperm_perm_grad_batched_workspace_size(n, count))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=A.device)
    with torch.cuda.device(A.device):
        nat.check(lib.gbperm_perm_grad_batched_dev(_P(A.data_ptr()), n, count, n, n * n, _P(perms.data_ptr()),
                                                   _P(grads.data_ptr()), _P(ws.data_ptr()), ws_bytes,
                                                   _stream_ptr(A)))
    return torch.complex(perms[:, 0], perms[:, 1]), grads


class PermanentBatched(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A):
        p, g = permanents_and_grads(A)
        ctx.save_for_backward(g)
        return p

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out[:, None, None] * g.conj()


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
    """Differentiable permanent of a square complex CUDA matrix, or the
    permanents of a (B, n, n) stack."""
    if A.dim() == 3:
        return PermanentBatched.apply(A)
    return Permanent.apply(A)


class ClementsMesh(torch.autograd.Function):
    """The mesh unitary (gbperm_mesh_unitary_dev) and its phase adjoint
    (gbperm_mesh_unitary_backward_dev); the layer states stay in a device
    workspace from the forward pass to the backward pass."""

    @staticmethod
    def forward(ctx, phases, m):
        lib = nat.load()
        ws_bytes = int(lib.gbperm_mesh_workspace_size(m))
        if ws_bytes == 0:
            raise ValueError("clements_unitary: modes must be in 1..64")
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=phases.device)
        U = torch.empty((m, m), dtype=torch.complex128, device=phases.device)
        with torch.cuda.device(phases.device):
            nat.check(lib.gbperm_mesh_unitary_dev(_P(phases.data_ptr()), m, _P(U.data_ptr()), _P(ws.data_ptr()),
                                                  ws_bytes, _stream_ptr(phases)))
        ctx.save_for_backward(phases)
        ctx.ws = ws
        ctx.m = m
        return U

    @staticmethod
    def backward(ctx, gU):
        (phases,) = ctx.saved_tensors
        lib = nat.load()
        gU = gU.to(torch.complex128).contiguous()
        g = torch.empty_like(phases)
        with torch.cuda.device(phases.device):
            nat.check(lib.gbperm_mesh_unitary_backward_dev(_P(phases.data_ptr()), ctx.m, _P(gU.data_ptr()),
                                                           _P(g.data_ptr()), _P(ctx.ws.data_ptr()), ctx.ws.numel(),
                                                           _stream_ptr(phases)))
        return g, None


def clements_unitary(phases: torch.Tensor, m: int) -> torch.Tensor:
    """m x m unitary (complex128) of a Clements rectangular mesh of m(m-1)/2
    Mach-Zehnder interferometers, two phases (theta, phi) each: phases has
    m(m-1) entries, on a CUDA device.  Layer l holds the interferometers on
    mode pairs (i, i+1), i = l mod 2, l mod 2 + 2, ...; each maps rows
    (i, i+1) of the running matrix by
    [[e^{i phi} cos theta, -sin theta], [e^{i phi} sin theta, cos theta]],
    so U = L_{m-1} ... L_1 L_0.  Differentiable with respect to the phases
    (hand-written forward and adjoint kernels; no CPU path)."""
    if not phases.is_cuda:
        raise ValueError("clements_unitary: the phases must be a CUDA tensor (no CPU path)")
    if phases.dim() != 1 or phases.numel() != m * (m - 1):
        raise ValueError("clements_unitary: phases must hold m(m-1) entries")
    return ClementsMesh.apply(phases.to(torch.float64).contiguous(), int(m))


def capture_graph(fn, warmup: int = 3):
    """Capture ``fn()`` -- e.g. a forward + backward step built from
    ``clements_unitary``, ``permanent`` and torch ops over static input
    tensors -- as one CUDA graph.  The library's device entry points only
    enqueue on the current stream and allocate through torch, so such a step
    captures whole; one-time setup runs in the ``warmup`` eager calls, which
    go to a side stream as torch's capture rules ask.  Returns
    ``(graph, outputs)``: copy new inputs into the same tensors and call
    ``graph.replay()``; ``outputs`` are then overwritten in place."""
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):
            fn()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        outputs = fn()
    return graph, outputs
