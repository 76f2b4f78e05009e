"""The oracle's restatement of assemble_ewald (j.ASSEMBLERS/
M_assemble_ewald_DOGS.f90:633-918), pinned to a known answer: with charges
+1/-1 on the rock-salt lattice, 1/2 q . ewald . q is the Madelung energy
-4 M / r0 of the conventional cell (M = 1.747564594633, r0 = a/2).  Also:
the matrix is symmetric, a cluster keeps the bare Coulomb 1/z, and the
ewaldsr / ewaldlr blocks vanish with the charges."""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc

MADELUNG_NACL = 1.747564594633


@pytest.fixture(scope="module")
def fd(fdata_root):
    path, nZ, _ = workload("sic_vac", fdata_root, dogs=True)
    return orc.Fdata(path, nZ)


def _ewald(fd, pos, imass, lattice, icluster=0):
    s = orc.System(fd, pos, np.asarray(imass, np.int32), lattice, icluster=icluster)
    L = orc.lib()
    n = len(imass)
    ew = np.zeros(n * n)
    L.or_assemble_ewald(s.h, ew)
    return ew.reshape(n, n)


@pytest.mark.parametrize("a", [5.64, 4.2])
def test_rock_salt_madelung(fd, a):
    base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    pos = np.vstack([base, base + [.5, 0, 0]]) * a
    ew = _ewald(fd, pos, [1] * 4 + [2] * 4, np.eye(3) * a)
    q = np.array([1.0] * 4 + [-1.0] * 4)
    assert abs(0.5 * q @ ew @ q - (-4 * MADELUNG_NACL / (a / 2))) < 1e-8
    assert np.abs(ew - ew.T).max() == 0.0


def test_cluster_is_bare_coulomb(fd):
    rng = np.random.default_rng(1)
    pos = rng.uniform(0, 6, (5, 3))
    ew = _ewald(fd, pos, [1, 2, 1, 2, 1], np.eye(3) * 50, icluster=1)
    d = np.linalg.norm(pos[:, None] - pos[None], axis=2)
    want = np.where(d > 1e-4, 1.0 / np.where(d > 0, d, 1), 0.0)
    assert np.abs(ew - want).max() < 1e-14


def test_ewald_blocks_vanish_without_charges(fdata_root):
    path, nZ, st = workload("sic_vac", fdata_root, dogs=True)
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors()
    ew, sr, lr = s.assemble_ewald(np.zeros((len(st.imass), 3)))
    assert np.abs(sr).max() == 0.0 and np.abs(lr).max() == 0.0
    ew, sr, lr = s.assemble_ewald(np.random.default_rng(3).uniform(-0.3, 0.3, (len(st.imass), 3)))
    assert np.abs(sr).max() > 1e-3 and np.abs(lr).max() > 1e-3


@pytest.fixture(scope="module")
def ew_system(fdata_root):
    from conftest import symmetric_denmat
    path, nZ, st = workload("sic_vac", fdata_root, dogs=True)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    norb = np.array([fd.norb(int(q)) for q in st.imass])
    rho, _ = symmetric_denmat(s, norb, 5)
    dq = np.random.default_rng(2).uniform(-0.3, 0.3, (len(st.imass), 3))
    return fd, s, st, rho, dq


def test_ewald_forces_are_minus_gradients(ew_system):
    """Dassemble_ewald's dewald(:, i, j) is d ewald(i, j) / d r_i; its Ewald
    energy force is -d/dR sum_ij (Q_i Q_j - Q0_i Q0_j) ewald(i, j); and the
    build_forces sum of the ewaldsr / ewaldlr forces is -d/dR sum rho .
    (ewaldlr - ewaldsr), all by central differences."""
    fd, s, st, rho, dq = ew_system
    N = len(st.imass)
    d = s.dassemble_ewald(rho, dq)
    Q0 = np.array([fd.norb(1) * 0 + 4.0] * N)  # the synthetic Si and C: Qneutral 2 + 2
    Q = Q0 + dq[:, :2].sum(1)
    qq = np.outer(Q, Q) - np.outer(Q0, Q0)
    h = 1e-5

    def at(r):
        t = orc.System(fd, r, st.imass, st.lattice).neighbors()
        assert t.npairs == s.npairs
        ew, sr, lr = t.assemble_ewald(dq)
        return ew, float(rho @ (lr - sr))

    for i in (1, 4):
        for k in range(3):
            rp, rm = st.ratom.copy(), st.ratom.copy()
            rp[i, k] += h
            rm[i, k] -= h
            (ep, Ep), (em, Em) = at(rp), at(rm)
            dew = (ep - em) / (2 * h)
            off = np.arange(N) != i
            assert np.abs(dew[i, off] - d["dewald"][i, off, k]).max() < 1e-8
            g = -((qq * ep).sum() - (qq * em).sum()) / (2 * h)
            assert abs(g - d["fewald"][3 * i + k]) < 1e-6 * max(1.0, abs(g))
            g = -(Ep - Em) / (2 * h)
            assert abs(g - d["ftot_add"][3 * i + k]) < 1e-6 * max(1.0, abs(g))
