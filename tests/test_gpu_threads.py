"""Concurrent host-API calls from several Python threads: ctypes drops the
GIL around each call, and the library gives every calling thread its own
stream and device workspace, so the calls overlap on the GPU without
sharing buffers."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from piquassoboost_gb300 import _native as nat
from piquassoboost_gb300.workloads import haar_block, repeated_instance

pytestmark = pytest.mark.gpu


def test_threads_get_their_own_results():
    mats = [haar_block(n, seed=900 + n) for n in range(14, 22)]
    reps = [repeated_instance(seed=s, modes=20, photons=10, max_mult=3) for s in range(8)]
    ref_plain = [nat.perm(m, mode="fast") for m in mats]
    ref_rep = [nat.perm_repeated(u, i, o, mode="fast") for u, i, o in reps]

    def work(k):
        out = []
        for _ in range(3):
            out.append(nat.perm(mats[k], mode="fast"))
            u, i, o = reps[k]
            out.append(nat.perm_repeated(u, i, o, mode="fast"))
        return out

    with ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(work, range(8)))
    for k, res in enumerate(results):
        for t in range(3):
            assert res[2 * t] == ref_plain[k]          # bitwise: fixed-order reductions
            assert res[2 * t + 1] == ref_rep[k]


def test_threads_mixed_shapes_share_kernels():
    # different table sizes on the same kernels from several threads at once:
    # each launch's dynamic shared memory differs, and none may fail
    from piquassoboost_gb300.workloads import pmf_layer_instance
    reps = [repeated_instance(seed=50 + s, modes=24, photons=8 + s, max_mult=3) for s in range(6)]
    layers = [pmf_layer_instance(seed=70 + s, modes=16, photons=6 + s) for s in range(6)]
    ref_rep = [nat.perm_repeated(u, i, o, mode=m) for (u, i, o) in reps for m in ("fast", "fp64")]
    ref_pmf = [nat.compute_pmf(u, s, c, mode=m)[0] for (u, s, c) in layers for m in ("fast", "fp64")]

    def work(k):
        out = []
        for it in range(4):
            u, i, o = reps[(k + it) % 6]
            for m in ("fast", "fp64"):
                out.append(("rep", (k + it) % 6, m, nat.perm_repeated(u, i, o, mode=m)))
            u, s, c = layers[(k + it) % 6]
            for m in ("fast", "fp64"):
                out.append(("pmf", (k + it) % 6, m, nat.compute_pmf(u, s, c, mode=m)[0]))
        return out

    with ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(work, range(8)))
    for res in results:
        for kind, idx, m, v in res:
            j = 2 * idx + (0 if m == "fast" else 1)
            if kind == "rep":
                assert v == ref_rep[j]
            else:
                assert np.array_equal(v, ref_pmf[j])
