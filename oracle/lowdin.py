"""numpy restatement of the reference's k-point Lowdin solver.

TEST INFRASTRUCTURE ONLY: the checker of the library's GPU eigensolver
(fb_solve_k), imported by the tests and the benchmark's check leg, never by
the product path.  Parity status: unpinned (the reference's Fortran cannot
be built here); LAPACK's zheev is replaced by numpy.linalg.eigh, which
returns the same ascending eigenvalues and eigenvectors up to a phase per
column.

Follows h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:
  diagonalize_S (:145-251): eigenpairs of S(k); the eigenvalues below
    overtol = 1e-4 count as a linear dependence: with mineig the number of
    them, columns mineig+1..n are moved to 1..n-mineig (:222-233), the
    trailing mineig columns keep what they held;
  diagonalize_H_Lowdin (:264-403): every column j of the shifted eigenvector
    matrix is scaled by lambda_j^(-1/4) and S12 = W W^H (:336-343; the
    routine takes norbitals_new = size(eigen) = n, so the trailing columns
    enter too); Z = S12 H S12 (:352-357); eigenpairs of Z (:372-379):
    the band energies and c_Lowdin; c = S12 c_Lowdin (:386-388).
"""
from __future__ import annotations

import numpy as np

OVERTOL = 1.0e-4


def s12_of(Sk):
    """(S^-1/2 as the reference forms it, number of dropped eigenvalues)."""
    lam, U = np.linalg.eigh(Sk)
    n = len(lam)
    m = int(np.count_nonzero(lam < OVERTOL))
    # mineig = the last index with lam < overtol (ascending order), +1
    if m:
        last = int(np.nonzero(lam < OVERTOL)[0].max()) + 1
        m = last
        lam = lam.copy()
        U = U.copy()
        lam[:n - m] = lam[m:]
        U[:, :n - m] = U[:, m:]
    W = U * lam ** (-0.25)
    return W @ W.conj().T, m


def solve_k(Hk, Sk):
    """(eigenvalues ascending, c_Lowdin, c, S12, dropped) of one k-point."""
    S12, m = s12_of(Sk)
    Z = S12 @ Hk @ S12
    eps, cl = np.linalg.eigh(Z)
    return eps, cl, S12 @ cl, S12, m
