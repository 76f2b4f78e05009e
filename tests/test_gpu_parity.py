"""GPU parity: libfbgpu (through its C ABI) against the CPU oracle.

Neighbor maps and block indices must be bit-exact; matrix elements and
forces must agree to 1e-10 eV (and eV/Angstrom) per element, which is tighter
than the 1e-10 Ha (2.7e-9 eV) the assembly is required to hold.
"""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL_BLOCK = 1e-10   # eV per matrix element
TOL_FORCE = 1e-10   # eV/Angstrom per component


@pytest.fixture(scope="module")
def gpu_ctx():
    import fbgpu
    ctx = fbgpu.Context(0)
    yield ctx
    ctx.close()


def _oracle(path, nZ, st, threads=1):
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, threads=threads).neighbors()
    return fd, s


CASES = ["si64", "cho_small", "sic_small", "si_vac", "sic_vac"]


@pytest.mark.parametrize("name", CASES)
def test_neighbors_bit_exact(gpu_ctx, fdata_root, name):
    path, nZ, st = workload(name, fdata_root)
    fd, s = _oracle(path, nZ, st)
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, NB = ctx.driver_neighbors()
    assert (P, T, NB) == (s.npairs, s.ntrip, s.nblock)
    nb = ctx.neighbors()
    assert np.array_equal(nb["neighn"], np.diff(s.pair_off))
    assert np.array_equal(nb["neigh_j"], s.neigh_j[:P] + 1)
    assert np.array_equal(nb["neigh_b"], s.neigh_b[:P])
    assert np.array_equal(nb["neigh_back"], s.neigh_back[:P] + 1)
    assert np.array_equal(nb["neigh_self"], s.neigh_self + 1)
    assert np.array_equal(nb["blk_off"], s.blk_off)
    cm = ctx.common_neighbors()
    assert np.array_equal(cm["ncommon"], np.diff(s.trip_off))
    assert np.array_equal(cm["iatom_common_j"], s.ci_j[:T] + 1)
    assert np.array_equal(cm["iatom_common_b"], s.ci_b[:T])
    assert np.array_equal(cm["jatom_common_j"], s.cj_j[:T] + 1)
    assert np.array_equal(cm["jatom_common_b"], s.cj_b[:T])
    assert np.array_equal(cm["neigh_common"], s.cneigh[:T] + 1)


PRECS = [0, 1]  # FB_PREC_FP64, FB_PREC_DF (double-float three-center kernels)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", CASES)
def test_blocks_match_oracle(gpu_ctx, fdata_root, name, prec):
    path, nZ, st = workload(name, fdata_root)
    fd, s = _oracle(path, nZ, st)
    S0, T0, vb0, vbo0 = s.assemble()
    ctx = gpu_ctx
    ctx.set_precision(prec)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.assemble_S()
    ctx.assemble_T()
    ctx.assemble_vna_2c()
    ctx.assemble_vna_3c()
    for key, ref in (("S", S0), ("T", T0), ("vna", vb0), ("vnao", vbo0)):
        got = ctx.blocks(key)
        err = np.abs(got - ref).max()
        assert err <= TOL_BLOCK, "%s prec %d %s max |diff| %.3e" % (name, prec, key, err)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", CASES)
def test_forces_match_oracle(gpu_ctx, fdata_root, name, prec):
    path, nZ, st = workload(name, fdata_root)
    fd, s = _oracle(path, nZ, st)
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 42)
    ref = s.dassemble(rho, cape)
    ctx = gpu_ctx
    ctx.set_precision(prec)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_denmat(rho, cape)
    ctx.Dassemble(keep_dblocks=True)
    for key in ("ftot", "kinetic", "vna", "pulay", "f3naa", "f3nab", "f3nac", "vna_ontop", "vna_atom"):
        got = ctx.forces(key)
        err = np.abs(got - ref[key]).max()
        assert err <= TOL_FORCE, "%s prec %d %s max |diff| %.3e" % (name, prec, key, err)
    for key in ("dS", "dT"):
        err = np.abs(ctx.blocks(key) - ref[key]).max()
        assert err <= TOL_FORCE, "%s %s max |diff| %.3e" % (name, key, err)


def test_step_through_host_buffers(gpu_ctx, fdata_root):
    """fb_assemble_step: positions in, four block sets out (host buffers)."""
    path, nZ, st = workload("si64", fdata_root)
    fd, s = _oracle(path, nZ, st)
    S0, T0, vb0, vbo0 = s.assemble()
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    outs = [np.zeros(s.nblock) for _ in range(4)]
    ctx.assemble_step(np.ascontiguousarray(st.ratom.ravel()), *outs)
    for got, ref in zip(outs, (S0, T0, vb0, vbo0)):
        assert np.abs(got - ref).max() <= TOL_BLOCK


@pytest.mark.slow
def test_si512_full_size_parity(gpu_ctx, fdata_root):
    """Configuration 2 at full size: neighbor maps bit-exact, blocks and
    forces within tolerance, both precision modes."""
    path, nZ, st = workload("si512", fdata_root)
    fd, s = _oracle(path, nZ, st, threads=16)
    S0, T0, vb0, vbo0 = s.assemble()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 7)
    ref = s.dassemble(rho, cape)
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    assert ctx.driver_neighbors() == (s.npairs, s.ntrip, s.nblock)
    nb = ctx.neighbors()
    assert np.array_equal(nb["neigh_j"], s.neigh_j[:s.npairs] + 1)
    assert np.array_equal(ctx.common_neighbors()["neigh_common"], s.cneigh[:s.ntrip] + 1)
    for prec in PRECS:
        ctx.set_precision(prec)
        ctx.assemble()
        for key, r in (("S", S0), ("T", T0), ("vna", vb0), ("vnao", vbo0)):
            assert np.abs(ctx.blocks(key) - r).max() <= TOL_BLOCK, (prec, key)
        ctx.set_denmat(rho, cape)
        ctx.Dassemble()
        assert np.abs(ctx.forces("ftot") - ref["ftot"]).max() <= TOL_FORCE, prec
    ctx.set_precision(1)
