"""Neighbor and common-neighbor decisions at the cutoff, against the oracle.

The GPU neighbor kernels pre-test distances in float (positions and, in the
common-neighbor search, the pairs' relative vectors) and take the
reference's FP64 test only in a band around the cutoff rc_i + rc_j - 0.01.
Random structures almost never land in the band; these do: an atom A with
two neighbors B and C whose distance |B - C| is set to the cutoff plus or
minus a tiny or a moderate offset, so that the pair (B, C) and the triplet
(A; B, C) are decided by the FP64 test (or by the float pre-test just outside
its margins).  Neighbor maps and triplet lists must be bit-exact.
"""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc
from fbgpu import synth

pytestmark = pytest.mark.gpu

# offsets of |B - C| from the cutoff (Angstrom): inside and outside the FP64
# band (within 1e-9, 1e-6, 5e-3 of it) and outside the float pre-test's
# margins (-0.03, +0.02)
OFFSETS = [-1e-9, 1e-9, -1e-6, 1e-6, -5e-3, 5e-3, -0.03, 0.02]


def _structure(offset):
    rc = 2.0 * synth.si().rcA - 0.01
    d = (rc + offset) / np.sqrt(2.0)
    e1 = np.array([1.0, 0.3, -0.2])
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(e1, [0.0, 0.0, 1.0])
    e2 /= np.linalg.norm(e2)
    A = np.array([20.0, 21.0, 19.0])
    B = A + d * e1
    C = A + d * e2
    # |B - C| = sqrt(2) d = rc + offset
    return synth.Structure(np.array([A, B, C]), np.array([1, 1, 1]), np.diag([60.0, 60.0, 60.0]), 0,
                           "band%+g" % offset)


@pytest.mark.parametrize("offset", OFFSETS)
def test_cutoff_band_decisions_bit_exact(fdata_root, offset):
    import fbgpu
    path, nZ, _ = workload("si64", fdata_root)
    st = _structure(offset)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    ctx = fbgpu.Context(0)
    try:
        ctx.read_Fdata(path, nZ)
        ctx.set_structure(st.ratom, st.imass, st.lattice)
        P, T, NB = ctx.driver_neighbors()
        assert (P, T, NB) == (s.npairs, s.ntrip, s.nblock)
        # inside the cutoff: B and C are neighbors and (A; B, C) a triplet
        assert (T > 0) == (offset < 0.0)
        nb = ctx.neighbors()
        assert np.array_equal(nb["neighn"], np.diff(s.pair_off))
        assert np.array_equal(nb["neigh_j"], s.neigh_j[:P] + 1)
        assert np.array_equal(nb["neigh_b"], s.neigh_b[:P])
        assert np.array_equal(nb["neigh_back"], s.neigh_back[:P] + 1)
        cm = ctx.common_neighbors()
        assert np.array_equal(cm["ncommon"], np.diff(s.trip_off))
        assert np.array_equal(cm["iatom_common_j"], s.ci_j[:T] + 1)
        assert np.array_equal(cm["jatom_common_j"], s.cj_j[:T] + 1)
        assert np.array_equal(cm["neigh_common"], s.cneigh[:T] + 1)
    finally:
        ctx.close()
