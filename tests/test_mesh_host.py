"""Host-side Clements mesh (the numpy copy used for host baselines) against
the plain-torch reference construction, on CPU."""
import numpy as np
import pytest

from piquassoboost_gb300.workloads import mesh_unitary

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("m", [1, 2, 3, 8, 13, 40])
def test_mesh_unitary_matches_torch_reference(m):
    from tests.mesh_reference import clements_unitary_torch
    ph = np.random.default_rng(m).uniform(0, 2 * np.pi, m * (m - 1))
    U = mesh_unitary(ph, m)
    R = clements_unitary_torch(torch.tensor(ph), m).numpy()
    assert np.abs(U - R).max() <= 1e-13
    assert np.abs(U @ U.conj().T - np.eye(m)).max() <= 1e-13
