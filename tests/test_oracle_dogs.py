"""The oracle's DOGS restatement (j.ASSEMBLERS/M_assemble_2c_DOGS.f90,
M_assemble_3c_DOGS.f90) on the synthetic DOGS Fdata: with zero shell
charges it is the Harris assembly exactly, the charged terms are linear in
the shell charges while S, T and the z-dipole blocks do not depend on them,
and the z-dipole blocks are finite."""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc

TOL = 1e-10


@pytest.fixture(scope="module", params=["sic_vac", "cho_small"])
def systems(request, fdata_root):
    name = request.param
    path, nZ, st = workload(name, fdata_root, dogs=True)
    path0, _, _ = workload(name, fdata_root)
    fd, fd0 = orc.Fdata(path, nZ), orc.Fdata(path0, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    s0 = orc.System(fd0, st.ratom, st.imass, st.lattice).neighbors()
    return s, s0, st


def test_zero_charges_are_harris(systems):
    s, s0, st = systems
    H = s0.assemble()
    D = s.assemble_dogs(np.zeros((len(st.imass), 3)))
    for a, b in zip(H, D[:4]):
        assert np.array_equal(a, b)


def test_charged_terms_linear(systems):
    s, _, st = systems
    rng = np.random.default_rng(5)
    dq = rng.uniform(-0.3, 0.3, (len(st.imass), 3))
    z = s.assemble_dogs(np.zeros_like(dq))
    a = s.assemble_dogs(dq)
    b = s.assemble_dogs(2.0 * dq)
    for k in (2, 3):  # vna, vnao
        d1, d2 = a[k] - z[k], b[k] - z[k]
        assert np.abs(d1).max() > 1e-3
        assert np.abs(d2 - 2.0 * d1).max() <= TOL * max(1.0, np.abs(d2).max())
    for k in (0, 1, 4):  # S, T and the dipole do not depend on the charges
        assert np.array_equal(a[k], z[k])


def test_dipole_finite(systems):
    s, _, st = systems
    D = s.assemble_dogs(np.zeros((len(st.imass), 3)))
    assert np.isfinite(D[4]).all() and np.abs(D[4]).max() > 0
