"""The DOGS Ewald terms on the GPU (fb_assemble with FB_EWALD) against the
oracle's restatement of assemble_ewald / assemble_ewaldsr / assemble_ewaldlr
(j.ASSEMBLERS/M_assemble_ewald_DOGS.f90): the N x N matrix to 1e-10 1/A and
the ewaldsr / ewaldlr blocks to 1e-10 eV per element, periodic cells of one
and two species, a vacancy cell, a cluster and the 512-atom Si cell (343
lattice vectors, most of them inside the screened cutoff), plain and as one
graph, with the lattice and reciprocal sums in FP64 (precision 0) and in
double-float (precision 1, the default); the call-order errors."""
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
        path, nZ, _ = workload("sic_small", fdata_root, dogs=True)
        st = synth.diamond((1, 1, 1), 4.36, 0.1, 41, sp_a=1, sp_b=2, name="SiC8cluster")
        st.icluster = 1
        return path, [14, 6], st
    return workload(name, fdata_root, dogs=True)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", ["sic_small", "si64", "sic_vac", "cho_small", "sic_cluster", "si512"])
def test_ewald_matches_oracle(ctx, fdata_root, name, prec):
    ctx.set_precision(prec)
    path, nZ, st = case(fdata_root, name)
    dq = np.random.default_rng(13).uniform(-0.3, 0.3, (len(st.imass), 3))
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
    ew, sr, lr = s.assemble_ewald(dq)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(dq)
    what = fbgpu.FB_ALL | fbgpu.FB_EWALD
    ctx.assemble(what)
    assert np.abs(ctx.ewald() - ew).max() <= TOL
    assert np.abs(ctx.blocks("ewaldsr") - sr).max() <= TOL
    assert np.abs(ctx.blocks("ewaldlr") - lr).max() <= TOL
    for _ in range(2):  # as one graph, captured then replayed
        ctx.assemble_graph(what)
        assert np.abs(ctx.blocks("ewaldsr") - sr).max() <= TOL
        assert np.abs(ctx.blocks("ewaldlr") - lr).max() <= TOL


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", ["sic_small", "sic_vac", "cho_small", "sic_cluster", "si512"])
def test_ewald_forces_match_oracle(ctx, fdata_root, name, prec):
    from conftest import symmetric_denmat
    ctx.set_precision(prec)
    path, nZ, st = case(fdata_root, name)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
    norb = np.array([fd.norb(int(q)) for q in st.imass])
    rho, cape = symmetric_denmat(s, norb, 5)
    dq = np.random.default_rng(2).uniform(-0.3, 0.3, (len(st.imass), 3))
    ref = s.dassemble_ewald(rho, dq)
    dogs = s.dassemble_dogs(rho, cape, dq)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(dq)
    ctx.set_denmat(rho, cape)
    what = fbgpu.FB_ALL | fbgpu.FB_EWALD
    ctx.assemble(what)
    ctx.Dassemble(what)
    assert np.abs(ctx.forces("ewald") - ref["fewald"]).max() <= TOL
    assert np.abs(ctx.forces("ewaldsr") - ref["ewaldsr"]).max() <= TOL
    assert np.abs(ctx.forces("ewaldlr") - ref["ewaldlr"]).max() <= TOL
    want = dogs["ftot"] + ref["ftot_add"]
    assert np.abs(ctx.forces("ftot") - want).max() <= TOL
    for _ in range(2):  # value and force pass as one graph
        ctx.assemble_graph(what | fbgpu.FB_FORCES)
        assert np.abs(ctx.forces("ftot") - want).max() <= TOL


def test_harris_ewald_is_zero(ctx, fdata_root):
    """The Harris assemble_ewaldsr / assemble_ewaldlr allocate zero blocks and
    Dassemble_ewaldsr zero pair forces (j.ASSEMBLERS/M_assemble_ewald_Harris.f90,
    k.DASSEMBLERS/M_Dassemble_ewald_Harris.f90); there is no Ewald matrix, and
    ftot is the Harris one."""
    from conftest import symmetric_denmat
    path, nZ, st = case(fdata_root, "sic_small")
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    rho, cape = symmetric_denmat(s, np.array([fd.norb(int(q)) for q in st.imass]), 3)
    ref = s.dassemble(rho, cape)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.set_denmat(rho, cape)
    what = fbgpu.FB_ALL | fbgpu.FB_EWALD
    ctx.assemble(what)
    assert not ctx.blocks("ewaldsr").any() and not ctx.blocks("ewaldlr").any()
    with pytest.raises(fbgpu.FBError) as e:
        ctx.ewald()
    assert e.value.code == 11
    ctx.Dassemble(what)
    for k in ("ewaldsr", "ewaldlr", "ewald"):
        assert not ctx.forces(k).any()
    assert np.abs(ctx.forces("ftot") - ref["ftot"]).max() <= TOL
    ctx.assemble_graph(what | fbgpu.FB_FORCES)
    assert np.abs(ctx.forces("ftot") - ref["ftot"]).max() <= TOL


def test_ewald_errors(ctx, fdata_root):
    path, nZ, st = case(fdata_root, "sic_small")
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    with pytest.raises(fbgpu.FBError) as e:      # no Ewald matrix yet
        ctx.ewald()
    assert e.value.code == 11
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(np.zeros((len(st.imass), 3)))
    with pytest.raises(fbgpu.FBError) as e:      # the overlap and dipole blocks first
        ctx.assemble(fbgpu.FB_EWALD)
    assert e.value.code == 11
