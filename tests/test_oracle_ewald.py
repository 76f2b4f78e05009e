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
