"""GPU parity of the batched persistent kernel."""
import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import batched_instances
from tests import oracle_bind as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("mode", ["fp64", "fast", "fx"])
def test_batched_uneven_vs_oracle(mode):
    mats = batched_instances(96, seed=5, modes=40, kmin=1, kmax=16)
    vals = nat.perm_batched(mats, mode=mode)
    for m, v in zip(mats, vals):
        _, q = orc.bbfg(m, prec=1)
        assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "fast", "fx"])
def test_batched_matches_single_kernel(mode):
    mats = batched_instances(24, seed=9, modes=60, kmin=16, kmax=22)
    vals = nat.perm_batched(mats, mode=mode)
    for m, v in zip(mats, vals):
        ref = nat.perm(m, mode="fp64")
        assert abs(v - ref) <= TOL * abs(ref)


@pytest.mark.parametrize("mode", ["fp64", "fx"])
def test_batched_trivial_and_rectangular(mode):
    rng = np.random.default_rng(2)
    mats = [np.zeros((0, 0)), np.ones((5, 2)), rng.standard_normal((3, 5)) + 1j, rng.standard_normal((4, 3)),
            rng.standard_normal((1, 1)), rng.standard_normal((2, 9)) + 1j, rng.standard_normal((7, 48)) + 0.5j]
    vals = nat.perm_batched(mats, mode=mode)
    assert vals[0] == 1 and vals[1] == 0
    for m, v in zip(mats[2:], vals[2:]):
        ref, q = orc.bbfg(m, prec=1)
        assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("mode", ["fast", "fx"])
def test_batched_nan_instance_isolated(mode):
    a = np.ones((4, 4)); b = np.ones((4, 4)); b[1, 2] = np.nan
    vals = nat.perm_batched([a, b, a], mode=mode)
    assert abs(vals[0] - 24) < 1e-9 and abs(vals[2] - 24) < 1e-9
    assert np.isnan(vals[1].real)


def test_batched_plan_reuse_and_item_sizes():
    mats = batched_instances(40, seed=21, modes=50, kmin=8, kmax=18)
    plan = nat.BatchPlan([m.shape for m in mats], mode="fast")
    first = plan.run(mats)
    for item_log2 in (6, 10, 14):
        plan.set_item_log2(item_log2)
        again = plan.run(mats)
        for a, b in zip(first, again):
            assert abs(a - b) <= TOL * abs(b)
    other = batched_instances(40, seed=22, modes=50, kmin=8, kmax=18)
    # same shapes are required; rebuild for the other draw
    plan2 = nat.BatchPlan([m.shape for m in other], mode="fast")
    vals = plan2.run(other)
    for m, v in zip(other, vals):
        ref = nat.perm(m, mode="fp64")
        assert abs(v - ref) <= TOL * abs(ref)
    plan.close(); plan2.close()


def test_dropin_list_branch_uses_batched():
    from piquassoboost_gb300.sampling.Boson_Sampling_Utilities import BBFGPermanentDouble
    mats = batched_instances(10, seed=3, modes=20, kmin=4, kmax=10)
    vals = BBFGPermanentDouble(mats).calculate()
    assert isinstance(vals, list) and len(vals) == 10
    for m, v in zip(mats, vals):
        _, q = orc.bbfg(m, prec=1)
        assert orc.rel_err(v, q) <= TOL


@pytest.mark.parametrize("mode", ["fast", "fx"])
def test_batched_autotune_keeps_results(mode):
    from piquassoboost_gb300.workloads import batched_instances
    mats = batched_instances(96, seed=12, modes=40, kmin=4, kmax=16)
    plan = nat.BatchPlan([m.shape for m in mats], mode=mode)
    before = plan.run(mats)
    ms = plan.autotune(mats)
    assert ms > 0.0
    grp, cpl = plan.shape()
    assert grp in (2, 4) and grp * cpl >= 16
    after = plan.run(mats)
    for a, b in zip(before, after):
        assert abs(a - b) <= 1e-10 * abs(b)
    plan.close()


def test_batched_device_pointer_run_with_trivial_slots():
    torch = pytest.importorskip("torch")
    import ctypes
    rng = np.random.default_rng(21)
    mats = [rng.standard_normal((k, k)) + 1j * rng.standard_normal((k, k)) for k in (5, 9, 12)]
    mats.insert(1, np.zeros((0, 0), dtype=np.complex128))          # empty -> 1
    mats.append(rng.standard_normal((6, 3)) + 0j)                   # rows >= cols + 2 -> 0
    plan = nat.BatchPlan([m.shape for m in mats], mode="fast")
    host = plan.run(mats)
    packed = torch.from_numpy(plan.pack(mats)).to("cuda")
    out = torch.full((2 * len(mats),), 7.0, dtype=torch.float64, device="cuda")
    P = ctypes.c_void_p
    nat.check(nat.load().gbperm_batch_plan_run_dev(plan._h, P(packed.data_ptr()), P(out.data_ptr()),
                                                   P(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    dev = out.cpu().numpy().reshape(-1, 2)
    for (re, im), h in zip(dev, host):
        assert abs(complex(re, im) - h) <= 1e-12 * max(abs(h), 1.0)
    assert complex(*dev[1]) == 1.0 and complex(*dev[-1]) == 0.0
    plan.close()


def test_batched_fast_within_bar_of_fp64():
    # the bench's uneven k = 8..28 instances (rows and columns drawn with
    # repetition): every double-float result whose error estimate is above
    # 1e-10 is recomputed with the FP64 product, so all are within the bar
    from piquassoboost_gb300.workloads import batched_instances
    mats = batched_instances(4096, seed=36)
    st = nat.Stats()
    f = np.array(nat.perm_batched(mats, mode="fast", stats=st))
    d = np.array(nat.perm_batched(mats, mode="fp64"))
    assert np.max(np.abs(f - d) / np.abs(d)) <= 1e-10
    assert 0.0 < st.err_est <= 1e-10
    x = np.array(nat.perm_batched(mats, mode="fx", stats=st))
    assert st.arith == nat.ARITH_FX64
    assert np.max(np.abs(x - d) / np.abs(d)) <= 1e-10


# ------------------------------------------------ multiplicity batch plan
def _pairs_batch(count, seed, modes, kmin, kmax):
    from piquassoboost_gb300.workloads import batched_index_sets, index_sets_to_states
    U, rows, cols = batched_index_sets(count, seed=seed, modes=modes, kmin=kmin, kmax=kmax)
    return U, rows, cols, index_sets_to_states(rows, cols, modes)


def test_rep_batch_matches_expanded_submatrices():
    # the draws of the batched configuration (rows and columns with
    # repetition from one Haar unitary) as state pairs: every permanent
    # against the integer-mantissa plain kernel on its expanded submatrix
    U, rows, cols, pairs = _pairs_batch(96, seed=7, modes=60, kmin=4, kmax=20)
    plan = nat.RepBatchPlan(U, pairs)
    got = plan.run()
    assert plan.info()["steps"] > 0
    for i, (r, c) in enumerate(zip(rows, cols)):
        ref = nat.perm(U[np.ix_(r, c)], mode="fx")
        assert abs(got[i] - ref) <= TOL * abs(ref), (i, got[i], ref)
    # a second run of the same plan gives the same bits
    assert np.array_equal(plan.run(), got)
    plan.close()


def test_rep_batch_vs_oracle_and_edge_pairs():
    from piquassoboost_gb300.workloads import haar_unitary
    m = 12
    U = haar_unitary(m, 3)
    rng = np.random.default_rng(12)
    pairs = []
    for _ in range(20):
        k = int(rng.integers(1, 9))
        pairs.append((rng.multinomial(k, np.ones(m) / m), rng.multinomial(k, np.ones(m) / m)))
    pairs.append((np.zeros(m, dtype=np.int64), np.zeros(m, dtype=np.int64)))   # no photons -> 1
    pairs.append((np.eye(m, dtype=np.int64)[2] * 3, np.eye(m, dtype=np.int64)[5] * 3))  # one mode each side
    plan = nat.RepBatchPlan(U, pairs)
    got = plan.run()
    for i, (cin, rout) in enumerate(pairs):
        ref, dref = orc.bbfg_repeated(U, cin, rout, prec=1)
        if abs(ref) < 1e-300:
            assert abs(got[i]) < 1e-12
        else:
            assert orc.rel_err(got[i], dref) <= TOL, (i, got[i], ref)
    # the batched entry point with the integer-mantissa product runs the plan
    many = nat.perm_repeated_many(U, pairs, mode="fx")
    assert np.allclose(many, got, rtol=0, atol=0)


def test_rep_batch_device_form_and_limits():
    torch = pytest.importorskip("torch")
    U, rows, cols, pairs = _pairs_batch(40, seed=8, modes=50, kmin=6, kmax=16)
    plan = nat.RepBatchPlan(U, pairs)
    host = plan.run()
    d_out = torch.zeros(2 * len(pairs), dtype=torch.float64, device="cuda")
    plan.run_dev(d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    dev = d_out.cpu().numpy()
    assert np.array_equal(dev[0::2] + 1j * dev[1::2], host)
    plan.close()
    # more than 40 occupied modes on both sides: rejected by the plan
    from piquassoboost_gb300.workloads import haar_unitary
    big = haar_unitary(44, 1)
    ones = np.ones(44, dtype=np.int64)
    with pytest.raises(nat.GBPermError) as ei:
        nat.RepBatchPlan(big, [(ones, ones)])
    assert ei.value.code == nat.GBPERM_ERR_TOO_LARGE
