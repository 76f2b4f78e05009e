"""Forces in epsilon's collinear fallback frames, against the oracle.

The force kernels take the frame derivatives through the rotation rates of
the frame.  Where epsilon falls back to its collinear frame while Depsilon
still returns non-zero derivatives, the reference's derivatives are not a
rotation of that frame: the three-center kernels add closed-form extra terms
(frame_extra_3c) and the two-center kernel takes its literal path.  Random
structures never reach these geometries; this one is built to:

- three Si atoms on a line through c + t e (c a 2e-3 A offset from the
  origin, perpendicular to e), so that the pair B-C has r2 nearly parallel to
  its bond (two-center fallback frame, |r2 x r1| >= 1e-3);
- the third atom A a little off that line (9.5e-5 of its distance to the
  bond midpoint), so that the triplet (A; B, C) has rhat nearly parallel to
  sighat (three-center fallback frame, |r21 x rnabc| >= 1e-3).
"""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc
from fbgpu import synth

pytestmark = pytest.mark.gpu


def _unit(v):
    return v / np.linalg.norm(v)


def _structure():
    e = _unit(np.array([1.0, 1.0, 1.0]))
    n1 = _unit(np.cross(e, [1.0, 0.0, 0.0]))
    n2 = np.cross(e, n1)
    c = 2.0e-3 * n1
    z, x = 4.4, 2.8
    tb = 25.0
    B = c + tb * e
    C = c + (tb + z) * e
    A = c + (tb + 0.5 * z + x) * e + 9.5e-5 * x * n2
    pos = np.array([B, C, A])
    lat = np.diag([80.0, 80.0, 80.0])
    return synth.Structure(pos, np.array([1, 1, 1]), lat, 0, "collinear3"), (A, B, C)


def _ypm(r1, r2):
    # epsilon's |r2hat x r1hat| (y axis magnitude before normalisation)
    return np.linalg.norm(np.cross(_unit(r2), _unit(r1)))


def test_geometry_reaches_the_fallback_frames():
    st, (A, B, C) = _structure()
    # two-center frame epsilon(r2, sighat) of the pair (B, C)
    sig = _unit(C - B)
    assert _ypm(C, sig) < 1.0e-4
    assert np.linalg.norm(np.cross(C, B)) >= 1.0e-3
    # three-center frame epsilon(rhat, sighat) of the triplet (A; B, C)
    rn = A - 0.5 * (B + C)
    assert _ypm(_unit(rn), sig) < 1.0e-4
    assert np.linalg.norm(np.cross(C - B, rn)) >= 1.0e-3


@pytest.mark.parametrize("prec", [0, 1])
def test_forces_in_fallback_frames_match_oracle(fdata_root, prec):
    import fbgpu
    path, nZ, _ = workload("si64", fdata_root)
    st, _ = _structure()
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    assert s.ntrip > 0
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 5)
    ref = s.dassemble(rho, cape)
    ctx = fbgpu.Context(0)
    try:
        ctx.set_precision(prec)
        ctx.read_Fdata(path, nZ)
        ctx.set_structure(st.ratom, st.imass, st.lattice)
        ctx.driver_neighbors()
        ctx.set_denmat(rho, cape)
        ctx.Dassemble()
        # The fallback frames' derivatives are large (1 / |r21 x rnabc| ~ 1e3)
        # and the forces ill-conditioned: the oracle itself, built with and
        # without FMA contraction, differs on this structure by 3.5e-10 of the
        # largest ftot component (7.8e-10 for f3naa).  The tolerance is 2e-9 of
        # each array's largest component; a missing fallback term is off by
        # ~1e-2 of it.
        for key in ("ftot", "kinetic", "vna", "f3naa", "f3nab", "f3nac", "vna_ontop", "vna_atom"):
            got, want = ctx.forces(key), ref[key]
            scale = max(1.0, float(np.abs(want).max()))
            err = float(np.abs(got - want).max())
            assert err <= 2e-9 * scale, (key, err, scale)
    finally:
        ctx.close()
