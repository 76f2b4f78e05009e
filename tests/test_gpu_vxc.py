"""The McWEDA exchange-correlation value pass on the GPU (fb_assemble with
FB_VXC) against the oracle's restatement of assemble_vxc
(j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90) and the input densities
(j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90): the vxc, rho_in and
rho_bond blocks and the shell-level weighted densities to 1e-10 per element
on cells of one and two species, with s-only hydrogen, vacancies and a
cluster, plain and as one graph; the call-order and table errors."""
import numpy as np
import pytest

import fbgpu
from conftest import workload
from fbgpu import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    c = fbgpu.Context(0)
    yield c
    c.close()


def case(fdata_root, name):
    if name == "sic_cluster":
        path, nZ, _ = workload("sic_small", fdata_root, vxc=True)
        st = synth.diamond((1, 1, 1), 4.36, 0.1, 41, sp_a=1, sp_b=2, name="SiC8cluster")
        st.icluster = 1
        return path, [14, 6], st
    return workload(name, fdata_root, vxc=True)


def _check(ctx, ref, P):
    assert np.abs(ctx.blocks("rho_in") - ref["rho_in"]).max() <= TOL
    assert np.abs(ctx.blocks("rho_bond") - ref["rho_bond"]).max() <= TOL
    assert np.abs(ctx.blocks("wrho_in").reshape(P, 9) - ref["wrho_in"]).max() <= TOL
    assert np.abs(ctx.blocks("wrho_bond").reshape(P, 9) - ref["wrho_bond"]).max() <= TOL
    assert np.abs(ctx.blocks("vxc") - ref["vxc"]).max() <= TOL


@pytest.mark.parametrize("prec", [0, 1])  # FP64 kernels, double-float three-center densities
@pytest.mark.parametrize("name", ["si64", "sic_small", "cho_small", "si_vac", "sic_vac", "sic_cluster"])
def test_vxc_matches_oracle(ctx, fdata_root, name, prec):
    ctx.set_precision(prec)
    path, nZ, st = case(fdata_root, name)
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
    ref = s.assemble_vxc()
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    what = fbgpu.FB_ALL | fbgpu.FB_VXC
    try:
        ctx.assemble(what)
        assert np.abs(ctx.blocks("S") - ref["S"]).max() <= TOL
        _check(ctx, ref, s.npairs)
        for _ in range(2):  # as one graph, captured then replayed
            ctx.assemble_graph(what)
            _check(ctx, ref, s.npairs)
    finally:
        ctx.set_precision(1)


def test_vxc_after_overlap(ctx, fdata_root):
    """FB_VXC alone reads the overlap of an earlier call."""
    path, nZ, st = case(fdata_root, "sic_small")
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors()
    ref = s.assemble_vxc()
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.assemble(fbgpu.FB_S)
    ctx.assemble(fbgpu.FB_VXC)
    _check(ctx, ref, s.npairs)


@pytest.mark.parametrize("prec", [0, 1])  # FP64 kernels, double-float three-center kernels
@pytest.mark.parametrize("name", ["sic_small", "si64", "cho_small", "sic_vac", "sic_cluster"])
def test_vxc_forces_match_oracle(ctx, fdata_root, name, prec):
    """Dassemble_vxc: the pair forces vxc_off_site / vxc_on_site, f3xca/b/c,
    the vxc pair sums and their addition to ftot, plain and as one graph."""
    from conftest import symmetric_denmat
    path, nZ, st = case(fdata_root, name)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
    rho, cape = symmetric_denmat(s, np.array([fd.norb(int(q)) for q in st.imass]), 5)
    ref = s.dassemble_vxc(rho)
    harris = s.dassemble(rho, cape)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.set_denmat(rho, cape)
    ctx.set_precision(prec)
    what = fbgpu.FB_ALL | fbgpu.FB_VXC
    try:
        ctx.assemble(what)
        ctx.Dassemble(what)
        for k in ("vxc_off_site", "vxc_on_site", "f3xca", "f3xcb", "f3xcc", "vxc"):
            assert np.abs(ctx.forces(k) - ref[k]).max() <= TOL, k
        want = harris["ftot"] + ref["ftot_add"]
        assert np.abs(ctx.forces("ftot") - want).max() <= TOL
        for _ in range(2):  # value and force pass as one graph
            ctx.assemble_graph(what | fbgpu.FB_FORCES)
            assert np.abs(ctx.forces("ftot") - want).max() <= TOL
            assert np.abs(ctx.forces("vxc_on_site") - ref["vxc_on_site"]).max() <= TOL
    finally:
        ctx.set_precision(1)


def test_vxc_batch_matches_oracle(ctx, fdata_root):
    """A batch of three structures (one a cluster, one with a vacancy) in
    one FB_VXC assembly: each structure's densities and vxc blocks as the
    oracle gives them for that structure alone."""
    path = synth.fdata_dir_for("batch256", root=fdata_root, vxc=True)
    nZ = [14, 6]
    structs = [synth.diamond((1, 1, 2), 4.36, 0.1, 31, sp_a=1, sp_b=2, name="SiC16"),
               synth.diamond((2, 2, 1), 5.43, 0.1, 32, vacancy=0.05, name="Si32v"),
               synth.diamond((1, 1, 1), 4.36, 0.1, 33, sp_a=1, sp_b=2, name="SiC8cluster")]
    structs[2].icluster = 1
    fd = orc.Fdata(path, nZ)
    ctx.read_Fdata(path, nZ)
    ctx.set_batch([(st.ratom, st.imass, st.lattice, st.icluster) for st in structs])
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.assemble(fbgpu.FB_ALL | fbgpu.FB_VXC)
    got = {w: ctx.blocks(w) for w in ("rho_in", "rho_bond", "vxc")}
    off = ctx.batch_offsets()["block"]
    for k, st in enumerate(structs):
        s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
        ref = s.assemble_vxc()
        for w in ("rho_in", "rho_bond", "vxc"):
            assert np.abs(got[w][off[k]:off[k + 1]] - ref[w]).max() <= TOL, (k, w)


def test_all_terms_in_one_graph(ctx, fdata_root):
    """Harris S, T, vna, the vnl terms and McWEDA vxc, value and force
    pass as one graph: ftot is the sum of the oracle's three contributions."""
    from conftest import symmetric_denmat
    path, nZ, st = case(fdata_root, "sic_small")
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    rho, cape = symmetric_denmat(s, np.array([fd.norb(int(q)) for q in st.imass]), 6)
    harris = s.dassemble(rho, cape)
    vxc = s.dassemble_vxc(rho)
    s.neighbors_pp()
    from test_oracle_pp import _sym_rho
    rho_pp = _sym_rho(s, fd, st, 12)
    vnl = s.dassemble_pp(rho_pp)
    want = harris["ftot"] + vxc["ftot_add"] + vnl["ftot_vnl"]
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.driver_neighbors_PP()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.set_denmat(rho, cape)
    ctx.set_denmat_pp(rho_pp)
    what = fbgpu.FB_ALL | fbgpu.FB_VXC | fbgpu.FB_VNL | fbgpu.FB_FORCES
    for _ in range(2):
        ctx.assemble_graph(what)
        assert np.abs(ctx.forces("ftot") - want).max() <= TOL
        assert np.abs(ctx.blocks("vxc") - vxc["values"]["vxc"]).max() <= TOL


def test_vxc_errors(ctx, fdata_root):
    path, nZ, st = case(fdata_root, "sic_small")
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError) as e:      # the overlap first
        ctx.assemble(fbgpu.FB_VXC)
    assert e.value.code == 11
    both, _, _ = workload("sic_small", fdata_root, dogs=True, vxc=True)  # DOGS and McWEDA tables
    ctx.read_Fdata(both, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    with pytest.raises(fbgpu.FBError) as e:      # McWEDA Harris only
        ctx.assemble(fbgpu.FB_S | fbgpu.FB_VXC)
    assert e.value.code == 13
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    plain, nZ2, st2 = workload("sic_small", fdata_root)  # no McWEDA tables
    ctx.read_Fdata(plain, nZ2)
    ctx.set_structure(st2.ratom, st2.imass, st2.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError) as e:
        ctx.assemble(fbgpu.FB_S | fbgpu.FB_VXC)
    assert e.value.code == 3
