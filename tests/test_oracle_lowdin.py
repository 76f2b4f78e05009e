"""The oracle's Lowdin restatement (oracle/lowdin.py) on a small Hermitian
pair: with a positive-definite S it is the generalized eigenproblem
H c = S c eps with c^H S c = 1; with an eigenvalue below 1e-4 the dropped
count and the column shift follow diagonalize_S."""
import numpy as np

from oracle import lowdin


def _herm(rng, n):
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return 0.5 * (a + a.conj().T)


def test_positive_definite_overlap_is_generalized_eigenproblem():
    rng = np.random.default_rng(1)
    n = 12
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    S = a @ a.conj().T / n + np.eye(n)
    H = _herm(rng, n)
    eps, cl, c, S12, m = lowdin.solve_k(H, S)
    assert m == 0
    assert np.abs(H @ c - S @ c * eps).max() < 1e-10
    assert np.abs(c.conj().T @ S @ c - np.eye(n)).max() < 1e-10
    assert np.abs(S12 @ S @ S12 - np.eye(n)).max() < 1e-10


def test_linear_dependence_drops_and_shifts():
    rng = np.random.default_rng(2)
    n = 8
    q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    lam = np.array([-0.3, 5e-5, 0.2, 0.5, 1.0, 1.5, 2.0, 3.0])
    S = (q * lam) @ q.conj().T
    S12, m = lowdin.s12_of(S)
    assert m == 2
    # kept: lam[2:], plus the trailing two columns again (the top two)
    l2, u2 = np.linalg.eigh(S)
    cols = list(range(2, 8)) + [6, 7]
    want = sum(np.outer(u2[:, j], u2[:, j].conj()) / np.sqrt(l2[j]) for j in cols)
    assert np.abs(S12 - want).max() < 1e-10
