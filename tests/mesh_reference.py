"""Plain-torch construction of the Clements mesh unitary, the numerical
reference for the hand-written mesh kernels: the m layer matrices are built
in one scatter and multiplied in a binary tree of batched products, all in
differentiable complex128 torch ops (CPU or CUDA), so torch autograd gives
the reference phase gradient.  Same conventions as
``piquassoboost_gb300.torch_perm.clements_unitary``."""
import torch


def clements_unitary_torch(phases: torch.Tensor, m: int) -> torch.Tensor:
    dev = phases.device
    lay, top = [], []
    for layer in range(m):
        for i in range(layer % 2, m - 1, 2):
            lay.append(layer)
            top.append(i)
    lay = torch.tensor(lay, dtype=torch.long, device=dev)
    top = torch.tensor(top, dtype=torch.long, device=dev)
    base = torch.eye(m, dtype=torch.complex128, device=dev).repeat(m, 1, 1)
    base[lay, top, top] = 0
    base[lay, top + 1, top + 1] = 0
    theta = phases[0::2]
    phi = phases[1::2]
    e_phi = torch.exp(1j * phi.to(torch.complex128))
    c = torch.cos(theta).to(torch.complex128)
    s = torch.sin(theta).to(torch.complex128)
    li = torch.cat([lay, lay, lay, lay])
    ri = torch.cat([top, top, top + 1, top + 1])
    ci = torch.cat([top, top + 1, top, top + 1])
    vals = torch.cat([e_phi * c, -s, e_phi * s, c])
    D = base.index_put((li, ri, ci), vals, accumulate=True)
    while D.shape[0] > 1:   # U = D[m-1] @ ... @ D[0]
        k = D.shape[0]
        even = k - (k % 2)
        prod = torch.bmm(D[1:even:2], D[0:even:2])
        D = torch.cat([prod, D[even:]]) if k % 2 else prod
    return D[0]
