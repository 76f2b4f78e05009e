"""Properties of the oracle's Bloch sums (the reference's Hmatrix /
Smatrix build, h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:413-442),
CPU only: S(k) and H(k) Hermitian; at Gamma real and equal to the plain
sum over images; under k -> k + G (G a reciprocal lattice vector) element
(i, j) changes only by the phase exp(i G . (r_j - r_i))."""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc


@pytest.fixture(scope="module")
def bloch_system(fdata_root):
    path, nZ, st = workload("si_vac", fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    S, T, vb, vbo = s.assemble()
    norb = np.array([fd.norb(int(q)) for q in st.imass])
    return s, st, norb, S, T + vb + vbo


def _slots(norb):
    return np.concatenate([[0], np.cumsum(norb)])


def test_bloch_hermitian(bloch_system):
    s, st, norb, S, H = bloch_system
    rng = np.random.default_rng(3)
    k = rng.uniform(-1.0, 1.0, (3, 3))
    for B, tol in ((S, 1e-12), (H, 1e-10)):
        M = s.bloch(k, B)
        for m in M:
            assert np.abs(m - m.conj().T).max() < tol


def test_bloch_gamma_is_image_sum(bloch_system):
    s, st, norb, S, H = bloch_system
    slot = _slots(norb)
    n = slot[-1]
    want = np.zeros((n, n))
    for i in range(st.natoms):
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            j = s.neigh_j[p]
            blk = S[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
            want[slot[i]:slot[i + 1], slot[j]:slot[j + 1]] += blk
    M = s.bloch(np.zeros((1, 3)), S)[0]
    assert np.abs(M.imag).max() == 0.0
    assert np.abs(M.real - want).max() < 1e-13


def test_bloch_reciprocal_shift_is_a_gauge(bloch_system):
    s, st, norb, S, H = bloch_system
    G = 2.0 * np.pi * np.linalg.inv(np.asarray(st.lattice, float)).T  # rows b_i, a_i . b_j = 2 pi delta
    k = np.array([0.11, -0.07, 0.23])
    g = G[0] - 2.0 * G[2]
    M0, M1 = s.bloch(np.stack([k, k + g]), H)
    slot = _slots(norb)
    ph = np.exp(1j * (st.ratom @ g))             # exp(i g . r_i) per atom
    d = np.repeat(ph, np.diff(slot))
    want = np.conj(d)[:, None] * M0 * d[None, :]  # exp(i g . (r_j - r_i))
    assert np.abs(M1 - want).max() < 1e-9 * max(1.0, np.abs(M0).max())
