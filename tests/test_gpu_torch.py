"""PyTorch boundary: the differentiable permanent inside a Clements-mesh
log-likelihood, backpropagated to the mesh phases and checked against FP64
central finite differences of the same loss."""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _modes(seed, m, k, count):
    rng = np.random.default_rng(seed)
    ins = [np.sort(rng.choice(m, size=k, replace=False)) for _ in range(count)]
    outs = [np.sort(rng.choice(m, size=k, replace=False)) for _ in range(count)]
    return ins, outs


@pytest.mark.parametrize("m", [1, 2, 3, 9, 16, 40, 64])
def test_mesh_kernel_matches_torch_reference(m):
    # forward: the native mesh against the plain-torch construction;
    # backward: the phase adjoint against torch autograd through it, for a
    # real loss with a random complex upstream weight
    from piquassoboost_gb300.torch_perm import clements_unitary
    from tests.mesh_reference import clements_unitary_torch
    rng = np.random.default_rng(100 + m)
    ph0 = rng.uniform(0, 2 * np.pi, m * (m - 1))
    W = torch.tensor(rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m)), device="cuda")
    pa = torch.tensor(ph0, device="cuda", requires_grad=True)
    Ua = clements_unitary(pa, m)
    pb = torch.tensor(ph0, device="cuda", requires_grad=True)
    Ub = clements_unitary_torch(pb, m)
    assert (Ua - Ub).abs().max().item() <= 1e-13
    if m == 1:
        return
    (Ua * W).sum().abs().pow(2).backward()
    (Ub * W).sum().abs().pow(2).backward()
    scale = pb.grad.abs().max().item()
    assert (pa.grad - pb.grad).abs().max().item() <= 1e-12 * max(1.0, scale)


def test_mesh_kernel_deterministic_and_checked():
    from piquassoboost_gb300.torch_perm import clements_unitary
    m = 40
    ph0 = np.random.default_rng(5).uniform(0, 2 * np.pi, m * (m - 1))
    grads = []
    for _ in range(2):
        ph = torch.tensor(ph0, device="cuda", requires_grad=True)
        U = clements_unitary(ph, m)
        (U.real.sum() + U[3, 7].imag).backward()
        grads.append(ph.grad.clone())
    assert torch.equal(grads[0], grads[1])
    with pytest.raises(ValueError):
        clements_unitary(torch.zeros(65 * 64, device="cuda", dtype=torch.float64), 65)
    with pytest.raises(ValueError):
        clements_unitary(torch.zeros(12, dtype=torch.float64), 4)
    with pytest.raises(ValueError):
        clements_unitary(torch.zeros(11, device="cuda", dtype=torch.float64), 4)


def test_clements_unitary_is_unitary():
    from piquassoboost_gb300.torch_perm import clements_unitary
    m = 10
    ph = torch.tensor(np.random.default_rng(0).uniform(0, 2 * np.pi, m * (m - 1)), device="cuda")
    U = clements_unitary(ph, m)
    eye = U @ U.conj().T
    assert torch.allclose(eye, torch.eye(m, dtype=torch.complex128, device="cuda"), atol=1e-12)


def _loss(ph, m, ins, outs, diff=True):
    from piquassoboost_gb300.torch_perm import clements_unitary, permanent, permanent_fwd
    U = clements_unitary(ph, m)
    total = 0.0
    for i, o in zip(ins, outs):
        sub = U[torch.as_tensor(o, device="cuda")][:, torch.as_tensor(i, device="cuda")]
        p = permanent(sub) if diff else permanent_fwd(sub)
        total = total + torch.log((p * p.conj()).real)
    return total


def test_clements_batch_backprop_vs_finite_differences():
    m, k, count = 16, 6, 12
    rng = np.random.default_rng(7)
    ph0 = rng.uniform(0, 2 * np.pi, m * (m - 1))
    ins, outs = _modes(3, m, k, count)
    ph = torch.tensor(ph0, device="cuda", requires_grad=True)
    loss = _loss(ph, m, ins, outs)
    loss.backward()
    g = ph.grad.cpu().numpy()
    h = 1e-6
    for idx in rng.choice(len(ph0), size=6, replace=False):
        p1 = ph0.copy(); p1[idx] += h
        p2 = ph0.copy(); p2[idx] -= h
        with torch.no_grad():
            l1 = _loss(torch.tensor(p1, device="cuda"), m, ins, outs, diff=False).item()
            l2 = _loss(torch.tensor(p2, device="cuda"), m, ins, outs, diff=False).item()
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, g[idx])


def test_permanent_fwd_matches_host_api():
    from piquassoboost_gb300.torch_perm import permanent_fwd
    from piquassoboost_gb300.workloads import haar_block
    A = haar_block(14, seed=2)
    for mode in ("fp64", "fast"):
        v = permanent_fwd(torch.tensor(A, device="cuda"), mode=mode).item()
        ref = nat.perm(A)
        assert abs(v - ref) <= 1e-10 * abs(ref)


def _batched_loss(ph, m, ins, outs, diff=True):
    from piquassoboost_gb300.torch_perm import clements_unitary, permanent, permanent_fwd
    U = clements_unitary(ph, m)
    o = torch.as_tensor(np.asarray(outs), device="cuda")
    i = torch.as_tensor(np.asarray(ins), device="cuda")
    subs = U[o[:, :, None], i[:, None, :]]          # (terms, k, k)
    if diff:
        p = permanent(subs)
    else:
        p = torch.stack([permanent_fwd(s) for s in subs])
    return torch.log((p * p.conj()).real).sum()


def test_batched_permanent_matches_per_term_loss_and_grad():
    m, k, count = 16, 6, 12
    rng = np.random.default_rng(11)
    ph0 = rng.uniform(0, 2 * np.pi, m * (m - 1))
    ins, outs = _modes(5, m, k, count)
    pa = torch.tensor(ph0, device="cuda", requires_grad=True)
    la = _loss(pa, m, ins, outs)
    la.backward()
    pb = torch.tensor(ph0, device="cuda", requires_grad=True)
    lb = _batched_loss(pb, m, ins, outs)
    lb.backward()
    assert abs(la.item() - lb.item()) <= 1e-11 * abs(la.item())
    assert torch.allclose(pa.grad, pb.grad, rtol=1e-9, atol=1e-11)


def test_mesh_batch_backprop_vs_finite_differences():
    # the 40-mode / 12-photon mesh shape with 32 terms
    from piquassoboost_gb300.workloads import mesh_instance
    ph0, ins, outs = mesh_instance(seed=3, modes=40, photons=12, terms=32)
    ph = torch.tensor(ph0, device="cuda", requires_grad=True)
    loss = _batched_loss(ph, 40, ins, outs)
    loss.backward()
    g = ph.grad.cpu().numpy()
    rng = np.random.default_rng(4)
    h = 1e-6
    for idx in rng.choice(len(ph0), size=5, replace=False):
        p1 = ph0.copy(); p1[idx] += h
        p2 = ph0.copy(); p2[idx] -= h
        with torch.no_grad():
            l1 = _batched_loss(torch.tensor(p1, device="cuda"), 40, ins, outs, diff=False).item()
            l2 = _batched_loss(torch.tensor(p2, device="cuda"), 40, ins, outs, diff=False).item()
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, g[idx])


def test_mesh_step_replays_as_cuda_graph():
    # the whole forward + backward step (mesh, gather, batched permanents,
    # loss, phase gradient) captured once and replayed on new inputs equals
    # the eager step on the same inputs
    from piquassoboost_gb300.torch_perm import capture_graph, clements_unitary, permanent
    from piquassoboost_gb300.workloads import mesh_instance
    m, k, terms = 16, 6, 40
    insts = [mesh_instance(seed=500 + s, modes=m, photons=k, terms=terms) for s in range(3)]
    s_ph = torch.zeros(m * (m - 1), dtype=torch.float64, device="cuda")
    s_o = torch.zeros((terms, k), dtype=torch.long, device="cuda")
    s_i = torch.zeros((terms, k), dtype=torch.long, device="cuda")

    def load(q):
        ph, ins, outs = insts[q]
        s_ph.copy_(torch.tensor(ph, device="cuda"))
        s_o.copy_(torch.tensor(outs, device="cuda"))
        s_i.copy_(torch.tensor(ins, device="cuda"))

    def step():
        ph = s_ph.detach().requires_grad_(True)
        U = clements_unitary(ph, m)
        p = permanent(U[s_o[:, :, None], s_i[:, None, :]])
        loss = torch.log((p * p.conj()).real).sum()
        (g,) = torch.autograd.grad(loss, ph)
        return loss.detach(), g

    load(0)
    graph, (g_loss, g_grad) = capture_graph(step)
    for q in (1, 2):
        load(q)
        e_loss, e_grad = step()
        graph.replay()
        torch.cuda.synchronize()
        assert abs(e_loss.item() - g_loss.item()) <= 1e-12 * abs(e_loss.item())
        assert torch.allclose(e_grad, g_grad, rtol=1e-12, atol=1e-12)

