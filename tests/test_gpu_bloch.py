"""Bloch sums into dense H(k), S(k) (h.SOLVESH/M_kspace_Lowdin.f90) on the
GPU against the oracle's restatement: the same matrices to FP64 rounding
(the GPU adds with atomics, in another order), Hermitian, real at Gamma."""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_ctx():
    import fbgpu
    ctx = fbgpu.Context(0)
    yield ctx
    ctx.close()


KPTS = np.array([[0.0, 0.0, 0.0], [0.11, -0.23, 0.31], [0.5, 0.5, 0.0]])


@pytest.mark.parametrize("name", ["si64", "cho_small", "sic_small"])
def test_bloch_matches_oracle(gpu_ctx, fdata_root, name):
    path, nZ, st = workload(name, fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    S0, T0, vb0, vbo0 = s.assemble()
    Href = s.bloch(KPTS, T0 + vb0 + vbo0)
    Sref = s.bloch(KPTS, S0)
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.assemble()
    Hk, Sk = ctx.bloch(KPTS)
    for got, ref in ((Hk, Href), (Sk, Sref)):
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= 1e-12 * scale
        assert np.abs(got - np.conj(np.transpose(got, (0, 2, 1)))).max() <= 1e-12 * scale
    assert np.abs(Hk[0].imag).max() <= 1e-13 * np.abs(Hk[0]).max()


def test_bloch_needs_blocks(gpu_ctx, fdata_root):
    import fbgpu
    path, nZ, st = workload("si64", fdata_root)
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError):
        ctx.bloch(KPTS[:1])
