"""Persistent launch shapes, the autotuner and the CUDA-graph step: every
launch shape and the graph replay must give the oracle's blocks and forces
(1e-10 eV, eV/Angstrom), like the default launches."""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10
FORCE_KEYS = ("ftot", "kinetic", "vna", "pulay", "f3naa", "f3nab", "f3nac", "vna_ontop", "vna_atom")


@pytest.fixture(scope="module")
def gpu_ctx():
    import fbgpu
    ctx = fbgpu.Context(0)
    yield ctx
    ctx.close()


def _reference(name, fdata_root, seed):
    path, nZ, st = workload(name, fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, seed)
    return path, nZ, st, s.assemble(), rho, cape, s.dassemble(rho, cape)


def _check(ctx, blocks, fref, tag):
    for key, ref in zip(("S", "T", "vna", "vnao"), blocks):
        err = np.abs(ctx.blocks(key) - ref).max()
        assert err <= TOL, "%s %s %.3e" % (tag, key, err)
    for key in FORCE_KEYS:
        err = np.abs(ctx.forces(key) - fref[key]).max()
        assert err <= TOL, "%s %s %.3e" % (tag, key, err)


SHAPES = [(64, 0, 1), (256, 0, 1), (64, 4, 1), (128, 2, 4), (256, 8, 16)]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", ["si64", "cho_small", "sic_small"])
def test_launch_shapes(gpu_ctx, fdata_root, name, prec):
    import fbgpu
    path, nZ, st, blocks, rho, cape, fref = _reference(name, fdata_root, 3)
    ctx = gpu_ctx
    ctx.set_precision(prec)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_denmat(rho, cape)
    for shape in SHAPES:
        for k in fbgpu.TUNABLE:
            ctx.set_launch(k, *shape)
        ctx.assemble()
        ctx.Dassemble()
        _check(ctx, blocks, fref, "%s prec %d shape %s" % (name, prec, shape))
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 128, 0, 1)
    ctx.set_precision(1)


@pytest.mark.parametrize("prec", [0, 1])
def test_graph_step_and_replay(gpu_ctx, fdata_root, prec):
    """The graph gives the separate calls' results, and a replay after a new
    density matrix gives that matrix's forces."""
    import fbgpu
    path, nZ, st, blocks, rho, cape, fref = _reference("sic_small", fdata_root, 5)
    _, _, _, _, rho2, cape2, fref2 = _reference("sic_small", fdata_root, 6)
    ctx = gpu_ctx
    ctx.set_precision(prec)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 128, 2, 4)
    ctx.set_denmat(rho, cape)
    l0 = ctx.kernel_launches()
    ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    per_graph = ctx.kernel_launches() - l0
    # 2c value, 2c force, three-center force (which also adds the
    # three-center value terms) and build_forces at least
    assert per_graph >= 4
    _check(ctx, blocks, fref, "graph prec %d" % prec)
    ctx.set_denmat(rho2, cape2)
    ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    assert ctx.kernel_launches() - l0 == 2 * per_graph
    _check(ctx, blocks, fref2, "replay prec %d" % prec)
    # same sizes after a neighbor rebuild: the graph is replayed, not re-captured
    ctx.driver_neighbors()
    ctx.set_denmat(rho, cape)
    ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    _check(ctx, blocks, fref, "after rebuild prec %d" % prec)
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 128, 0, 1)
    ctx.set_precision(1)


def test_autotune_then_results(gpu_ctx, fdata_root):
    import fbgpu
    path, nZ, st, blocks, rho, cape, fref = _reference("si64", fdata_root, 7)
    ctx = gpu_ctx
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_denmat(rho, cape)
    best = ctx.autotune(fbgpu.FB_ALL | fbgpu.FB_FORCES, reps=1)
    assert set(best) == set(fbgpu.TUNABLE)
    for k, (ms, shape) in best.items():
        assert ms > 0 and shape["threads"] in (64, 128, 256)
    ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    _check(ctx, blocks, fref, "autotuned")
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 128, 0, 1)


def test_launch_shape_rejects(gpu_ctx):
    import fbgpu
    with pytest.raises(fbgpu.FBError):
        gpu_ctx.set_launch("assemble_3c", 48, 0, 1)
    with pytest.raises(fbgpu.FBError):
        gpu_ctx.set_launch("no_such_kernel", 128, 0, 1)
