"""GPU gradient of the permanent: checked against minor permanents from the
oracle and against FP64 central finite differences (the permanent is linear
in each entry, so differences are exact up to rounding)."""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu


def _minor(A, k, l):
    return np.delete(np.delete(A, k, axis=0), l, axis=1)


@pytest.mark.parametrize("n", [2, 3, 5, 8, 12, 16])
def test_grad_all_minors(n):
    A = haar_block(n, seed=700 + n)
    p, G = nat.perm_grad(A)
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(p, q) <= 1e-10
    gnorm = np.abs(G).max()
    for k in range(n):
        for l in range(n):
            ref, _ = orc.bbfg(_minor(A, k, l), prec=1) if n > 1 else (1.0, None)
            assert abs(G[k, l] - ref) <= 1e-10 * max(abs(ref), 1e-3 * gnorm), (k, l, G[k, l], ref)


@pytest.mark.parametrize("n", [20, 24])
def test_grad_sampled_minors(n):
    A = haar_block(n, seed=800 + n)
    p, G = nat.perm_grad(A)
    rng = np.random.default_rng(n)
    gnorm = np.abs(G).max()
    for _ in range(6):
        k, l = rng.integers(0, n, size=2)
        ref, _ = orc.bbfg(_minor(A, k, l), prec=0)
        assert abs(G[k, l] - ref) <= 1e-10 * max(abs(ref), 1e-3 * gnorm)


@pytest.mark.parametrize("n", [2, 5, 9, 12])
def test_grad_fx_all_minors(n):
    # the integer-mantissa sweep: every entry against binary128 minors
    A = haar_block(n, seed=1700 + n)
    st = nat.Stats()
    p, G = nat.perm_grad(A, mode="fx", stats=st)
    assert st.arith == nat.ARITH_FX64
    _, q = orc.bbfg(A, prec=1)
    assert orc.rel_err(p, q) <= 1e-10
    gnorm = np.abs(G).max()
    for k in range(n):
        for l in range(n):
            ref, _ = orc.bbfg(_minor(A, k, l), prec=1) if n > 1 else (1.0, None)
            assert abs(G[k, l] - ref) <= 1e-10 * max(abs(ref), 1e-3 * gnorm), (k, l, G[k, l], ref)


@pytest.mark.parametrize("n", [20, 24])
def test_grad_fx_more_accurate_than_fast(n):
    # worst entry error against the FP64 kernel's minors, fx vs double-float
    A = haar_block(n, seed=1800 + n)
    _, Gf = nat.perm_grad(A, mode="fast")
    _, Gx = nat.perm_grad(A, mode="fx")
    rng = np.random.default_rng(n)
    gnorm = np.abs(Gx).max()
    worst = {"fast": 0.0, "fx": 0.0}
    for _ in range(8):
        k, l = (int(x) for x in rng.integers(0, n, size=2))
        m = nat.perm(_minor(A, k, l), mode="fx")
        d = max(abs(m), 1e-3 * gnorm)
        worst["fast"] = max(worst["fast"], abs(Gf[k, l] - m) / d)
        worst["fx"] = max(worst["fx"], abs(Gx[k, l] - m) / d)
    assert worst["fx"] <= 1e-12 and worst["fast"] <= 1e-10, worst


def test_grad_wide_column_range():
    # columns scaled by 2^-300 .. 2^300: each column is normalised by its own
    # power of two, so the double-float sweep keeps the bar
    rng = np.random.default_rng(51)
    n = 10
    A = haar_block(n, seed=51) * np.exp2(rng.integers(-300, 300, n))[None, :]
    p, G = nat.perm_grad(A)
    ref = nat.perm(A, mode="fx")
    assert abs(p - ref) <= 1e-10 * abs(ref)
    for k, l in ((0, 0), (3, 7), (9, 2)):
        m = nat.perm(_minor(A, k, l), mode="fx")
        assert abs(G[k, l] - m) <= 1e-10 * abs(m), (k, l)


def test_grad_range_check_failure_runs_fx_twin():
    # a zero column fails the double-float range check (no scale for it):
    # the device hands the matrix to the integer-mantissa twin, which used
    # to be an error.  The permanent is 0; the minors without that column
    # survive.
    n = 8
    A = haar_block(n, seed=8).copy()
    A[:, 3] = 0.0
    st = nat.Stats()
    p, G = nat.perm_grad(A, stats=st)
    assert st.arith == nat.ARITH_FX64
    assert p == 0
    gnorm = np.abs(G).max()
    assert gnorm > 0
    for k in range(n):
        for l in range(n):
            m = nat.perm(_minor(A, k, l), mode="fx")
            assert abs(G[k, l] - m) <= 1e-10 * max(abs(m), 1e-3 * gnorm)


def test_grad_escalates_above_error_bar():
    # positive entries: the Gray terms dwarf the permanent, the double-float
    # estimate exceeds 1e-10 and the twin recomputes on the device
    rng = np.random.default_rng(28)
    G0 = np.abs(rng.standard_normal((28, 28))) + 0.1
    st = nat.Stats()
    p, G = nat.perm_grad(G0, stats=st)
    assert st.arith == nat.ARITH_FX64
    px, Gx = nat.perm_grad(G0, mode="fx")
    assert abs(p - px) <= 1e-12 * abs(px)
    assert np.max(np.abs(G - Gx)) <= 1e-12 * np.max(np.abs(Gx))
    ref = nat.perm(G0, mode="fx")
    assert abs(p - ref) <= 1e-10 * abs(ref)
    # a Haar block stays on the double-float sweep, with its estimate reported
    st2 = nat.Stats()
    nat.perm_grad(haar_block(16, seed=16), stats=st2)
    assert st2.arith == nat.ARITH_DF32 and 0.0 < st2.err_est <= 1e-10


def test_grad_batched_mixed_escalation():
    # one launch: Haar members stay double-float, a positive member and an
    # out-of-range member go to the twin; each matches its own single call
    rng = np.random.default_rng(9)
    mats = [haar_block(12, seed=s) for s in range(3)]
    mats.append(np.abs(rng.standard_normal((12, 12))) + 0.1)
    zc = haar_block(12, seed=77).copy()
    zc[:, 5] = 0.0
    mats.append(zc)
    mats = np.stack(mats)
    perms, grads = nat.perm_grad_batched(mats)
    for b in range(len(mats)):
        ref = nat.perm(mats[b], mode="fx")
        assert abs(perms[b] - ref) <= 1e-10 * abs(ref) or perms[b] == ref == 0, b
        _, G = nat.perm_grad(mats[b], mode="fx")
        assert np.max(np.abs(grads[b] - G)) <= 1e-10 * np.max(np.abs(G)), b


@pytest.mark.parametrize("mode", ["fast", "fx"])
@pytest.mark.parametrize("n", [28, 32])
def test_grad_large_sampled_minors_and_differences(n, mode):
    # the gradient sizes of the differentiable-permanent configuration:
    # 16 seeded entries against their minors (n - 1 permanents on the FP64
    # kernel, itself pinned to the oracle) and 3 against FP64 central
    # differences (the permanent is linear in each entry, so the difference
    # quotient is exact up to rounding)
    A = haar_block(n, seed=900 + n)
    p, G = nat.perm_grad(A, mode=mode)
    ref = nat.perm(A, mode="fp64")
    assert abs(p - ref) <= 1e-10 * abs(ref)
    gnorm = np.abs(G).max()
    rng = np.random.default_rng(n)
    for _ in range(16):
        k, l = (int(x) for x in rng.integers(0, n, size=2))
        m = nat.perm(_minor(A, k, l), mode="fp64")
        assert abs(G[k, l] - m) <= 1e-10 * max(abs(m), 1e-3 * gnorm), (k, l, G[k, l], m)
    for _ in range(3):
        k, l = (int(x) for x in rng.integers(0, n, size=2))
        h = 1e-2
        Ap = A.copy()
        Ap[k, l] += h
        Am = A.copy()
        Am[k, l] -= h
        fd = (nat.perm(Ap, mode="fp64") - nat.perm(Am, mode="fp64")) / (2 * h)
        assert abs(fd - G[k, l]) <= 1e-8 * max(abs(G[k, l]), 1e-3 * gnorm), (k, l, fd, G[k, l])


def test_grad_finite_differences():
    n = 10
    A = haar_block(n, seed=31)
    _, G = nat.perm_grad(A)
    rng = np.random.default_rng(1)
    for _ in range(5):
        k, l = rng.integers(0, n, size=2)
        h = 1e-3
        Ap = A.copy(); Ap[k, l] += h
        Am = A.copy(); Am[k, l] -= h
        fd = (nat.perm(Ap) - nat.perm(Am)) / (2 * h)
        assert abs(fd - G[k, l]) <= 1e-8 * max(abs(G[k, l]), 1e-12)


def test_grad_forward_matches_plain():
    for n in (6, 14, 22):
        A = haar_block(n, seed=n)
        p, _ = nat.perm_grad(A)
        ref = nat.perm(A)
        assert abs(p - ref) <= 1e-10 * abs(ref)


def test_torch_autograd():
    torch = pytest.importorskip("torch")
    from piquassoboost_gb300.torch_perm import permanent
    n = 8
    A = haar_block(n, seed=3)
    At = torch.tensor(A, device="cuda", requires_grad=True)
    p = permanent(At)
    loss = (p * p.conj()).real  # |perm|^2
    loss.backward()
    _, G = nat.perm_grad(A)
    perm = nat.perm(A)
    # d|p|^2 / d conj(a) convention: grad = 2 * p * conj(G)... torch gives grad_out*conj(dp/dA) chain
    expected = 2 * perm * np.conj(G)
    assert np.allclose(At.grad.cpu().numpy(), expected, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("n,count", [(12, 37), (20, 3), (1, 5), (5, 64)])
def test_grad_batched_matches_single(n, count):
    rng = np.random.default_rng(n * 100 + count)
    mats = np.stack([haar_block(n, seed=int(s)) for s in rng.integers(0, 10**6, size=count)])
    perms, grads = nat.perm_grad_batched(mats)
    for b in range(count):
        p, G = nat.perm_grad(mats[b])
        assert abs(perms[b] - p) <= 1e-11 * abs(p)
        assert np.max(np.abs(grads[b] - G)) <= 1e-11 * np.max(np.abs(G))


def test_grad_batched_nonfinite_instance_isolated():
    mats = np.stack([haar_block(8, seed=s) for s in range(4)])
    mats[2, 3, 1] = np.nan
    perms, grads = nat.perm_grad_batched(mats)
    assert np.isnan(perms[2]) and np.all(np.isnan(grads[2]))
    for b in (0, 1, 3):
        p, G = nat.perm_grad(mats[b])
        assert abs(perms[b] - p) <= 1e-11 * abs(p)
        assert np.allclose(grads[b], G, rtol=1e-11, atol=0)


def test_grad_batched_minors():
    # every gradient entry of a few batch members against oracle minors
    mats = np.stack([haar_block(9, seed=900 + s) for s in range(6)])
    perms, grads = nat.perm_grad_batched(mats)
    for b in range(len(mats)):
        _, q = orc.bbfg(mats[b], prec=1)
        assert orc.rel_err(perms[b], q) <= 1e-10
        gnorm = np.abs(grads[b]).max()
        for k in range(9):
            for l in range(9):
                ref, _ = orc.bbfg(_minor(mats[b], k, l), prec=1)
                assert abs(grads[b, k, l] - ref) <= 1e-10 * max(abs(ref), 1e-3 * gnorm)


def test_grad_row_scaled_matrix():
    # rows scaled by factors up to ~10: the rows are balanced by exact powers
    # of two before the sweep, and each entry's exponent drops its row's
    # factor; permanent and minors against the binary128 oracle
    rng = np.random.default_rng(9)
    n = 14
    A = np.exp(rng.uniform(-2.3, 2.3, n))[:, None] * haar_block(n, seed=9)
    p, G = nat.perm_grad(A)
    _, ref = orc.bbfg(A, prec=1)
    assert orc.rel_err(p, ref) <= 1e-10
    for r, c in [(0, 0), (3, 7), (n - 1, 2), (5, n - 1), (9, 9)]:
        _, m = orc.bbfg(np.delete(np.delete(A, r, 0), c, 1), prec=1)
        assert orc.rel_err(G[r, c], m) <= 1e-10, (r, c)
