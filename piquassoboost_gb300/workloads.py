"""Seeded synthetic inputs with the shapes of the reference's permanent workloads.

All generators are deterministic in their seed (numpy default_rng).  Haar
unitaries are drawn as the QR factor of a complex Gaussian matrix with the
phases of R's diagonal divided out of Q's columns.
"""
from __future__ import annotations

import numpy as np


def haar_unitary(m: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))[None, :]


def haar_block(n: int, seed: int, m: int | None = None) -> np.ndarray:
    """Top-left n x n block of a seeded Haar m x m unitary (m = 2n by default)."""
    u = haar_unitary(m if m is not None else 2 * n, seed)
    return np.ascontiguousarray(u[:n, :n])


def repeated_instance(seed: int, modes: int = 60, photons: int = 30, max_mult: int = 4):
    """Haar `modes`-mode unitary, one photon in each of modes 0..photons-1,
    output occupation from a seeded multinomial over all modes with every
    multiplicity <= max_mult (redrawn otherwise)."""
    u = haar_unitary(modes, seed)
    rng = np.random.default_rng(seed + 7919)
    inp = np.zeros(modes, dtype=np.int64)
    inp[:photons] = 1
    while True:
        out = rng.multinomial(photons, np.ones(modes) / modes).astype(np.int64)
        if out.max() <= max_mult:
            break
    return u, inp, out


def batched_instances(count: int, seed: int, modes: int = 100, kmin: int = 8, kmax: int = 28):
    """`count` square k x k submatrices (k uniform in kmin..kmax) of one seeded
    Haar `modes`-mode unitary, rows and columns drawn with repetition."""
    u = haar_unitary(modes, seed)
    rng = np.random.default_rng(seed + 104729)
    ks = rng.integers(kmin, kmax + 1, size=count)
    mats = []
    for k in ks:
        r = rng.integers(0, modes, size=k)
        c = rng.integers(0, modes, size=k)
        mats.append(np.ascontiguousarray(u[np.ix_(r, c)]))
    return mats


def batched_index_sets(count: int, seed: int, modes: int = 100, kmin: int = 8, kmax: int = 28):
    """The draws behind batched_instances (same seed, same stream): the
    unitary and, per instance, its row and column index draws; instance i of
    batched_instances is u[np.ix_(rows[i], cols[i])]."""
    u = haar_unitary(modes, seed)
    rng = np.random.default_rng(seed + 104729)
    ks = rng.integers(kmin, kmax + 1, size=count)
    rows, cols = [], []
    for k in ks:
        rows.append(rng.integers(0, modes, size=k))
        cols.append(rng.integers(0, modes, size=k))
    return u, rows, cols


def index_sets_to_states(rows, cols, modes: int):
    """Occupation form of index draws: (input_state, output_state) pairs,
    input = column multiplicities, output = row multiplicities (the
    reference's (input, output) convention of the repeated calculators)."""
    return [(np.bincount(c, minlength=modes).astype(np.int64), np.bincount(r, minlength=modes).astype(np.int64))
            for r, c in zip(rows, cols)]


def pmf_layer_instance(seed: int, modes: int = 60, photons: int = 30):
    """The last probability layer of a Clifford & Clifford run: Haar
    `modes`-mode unitary, one input photon in each of modes 0..photons-1, and
    a sample of photons - 1 output photons from a seeded uniform multinomial
    over all modes (a Haar interferometer spreads photons near uniformly)."""
    u = haar_unitary(modes, seed)
    rng = np.random.default_rng(seed + 15485863)
    inp = np.zeros(modes, dtype=np.int64)
    inp[:photons] = 1
    sample = rng.multinomial(photons - 1, np.ones(modes) / modes).astype(np.int64)
    return u, sample, inp


def mesh_instance(seed: int, modes: int = 40, photons: int = 12, terms: int = 512):
    """Phases of a `modes`-mode Clements mesh (modes (modes-1) entries,
    uniform in [0, 2 pi)) and `terms` pairs of sorted input / output mode
    sets of `photons` distinct modes each, all seeded."""
    rng = np.random.default_rng(seed)
    phases = rng.uniform(0.0, 2.0 * np.pi, modes * (modes - 1))
    ins = np.stack([np.sort(rng.choice(modes, size=photons, replace=False)) for _ in range(terms)])
    outs = np.stack([np.sort(rng.choice(modes, size=photons, replace=False)) for _ in range(terms)])
    return phases, ins.astype(np.int64), outs.astype(np.int64)


def mesh_unitary(phases: np.ndarray, m: int) -> np.ndarray:
    """Host (numpy) copy of the Clements mesh unitary that
    ``torch_perm.clements_unitary`` builds on the device, for host-side
    baselines: layer l holds the pairs (i, i+1), i = l mod 2, l mod 2 + 2, ...,
    interferometer t (layer by layer, then by i) maps rows (i, i+1) by
    [[e^{i phi} cos theta, -sin theta], [e^{i phi} sin theta, cos theta]]
    with (theta, phi) = (phases[2t], phases[2t+1]); U = L_{m-1} ... L_0."""
    u = np.eye(m, dtype=np.complex128)
    t = 0
    for layer in range(m):
        for i in range(layer % 2, m - 1, 2):
            th, ph = phases[2 * t], phases[2 * t + 1]
            e = np.exp(1j * ph)
            a, b, c, d = e * np.cos(th), -np.sin(th), e * np.sin(th), np.cos(th)
            ri, ri1 = u[i].copy(), u[i + 1].copy()
            u[i] = a * ri + b * ri1
            u[i + 1] = c * ri + d * ri1
            t += 1
    return u
