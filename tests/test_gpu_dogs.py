"""DOGS on the GPU (fb_set_theory(FB_THEORY_DOGS)) against the oracle's
restatement of assemble_vna_2c / assemble_vna_3c / assemble_dipole_z
(j.ASSEMBLERS/M_assemble_{2c,3c}_DOGS.f90) and Dassemble_vna_2c /
Dassemble_vna_3c (k.DASSEMBLERS/M_Dassemble_{2c,3c}_DOGS.f90): every block
set to 1e-10 eV per element and every force array to 1e-10 eV/Angstrom per
component, for one- and two-species systems and for a batch, plain and as
one CUDA graph; zero charges give the Harris results; the call-order and
capability errors the interface states."""
import numpy as np
import pytest

import fbgpu
from conftest import workload
from fbgpu import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10   # eV per matrix element
TOL_FORCE = 1e-10   # eV/Angstrom per component
FORCES = ("ftot", "kinetic", "vna", "pulay", "f3naa", "f3nab", "f3nac", "vna_ontop", "vna_atom")


@pytest.fixture(scope="module")
def ctx():
    c = fbgpu.Context(0)
    yield c
    c.close()


def charges(n, seed):
    return np.random.default_rng(seed).uniform(-0.3, 0.3, (n, 3))


def gpu_dogs(ctx, path, nZ, st, dq, graph=False):
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(dq)
    if graph:
        ctx.assemble_graph(fbgpu.FB_ALL)
    else:
        ctx.assemble()
    return [ctx.blocks(w) for w in ("S", "T", "vna", "vnao", "dip")]


def gpu_dogs_forces(ctx, rho, cape, graph=False):
    ctx.set_denmat(rho, cape)
    if graph:
        ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    else:
        ctx.Dassemble()
    return {k: ctx.forces(k) for k in FORCES}


@pytest.mark.parametrize("prec", [0, 1])  # FP64, double-float three-center kernels
@pytest.mark.parametrize("name", ["sic_small", "cho_small", "si64", "sic_vac"])
def test_dogs_forces_match_oracle(ctx, fdata_root, name, prec):
    from conftest import symmetric_denmat
    path, nZ, st = workload(name, fdata_root, dogs=True)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    norb = np.array([fd.norb(int(q)) for q in st.imass])
    rho, cape = symmetric_denmat(s, norb, 23)
    dq = charges(len(st.imass), 29)
    ref = s.dassemble_dogs(rho, cape, dq)
    ctx.set_precision(prec)
    try:
        gpu_dogs(ctx, path, nZ, st, dq)
        got = gpu_dogs_forces(ctx, rho, cape)
        for k in FORCES:
            assert np.abs(got[k] - ref[k]).max() <= TOL_FORCE, (k, np.abs(got[k] - ref[k]).max())
        # the same step as one graph (value and force pass), replayed
        for _ in range(2):
            g = gpu_dogs_forces(ctx, rho, cape, graph=True)
            for k in FORCES:
                assert np.abs(g[k] - ref[k]).max() <= TOL_FORCE, ("graph", k)
    finally:
        ctx.set_precision(fbgpu.FB_PREC_DF)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", ["sic_small", "cho_small", "si64", "sic_vac"])
def test_dogs_matches_oracle(ctx, fdata_root, name, prec):
    path, nZ, st = workload(name, fdata_root, dogs=True)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    dq = charges(len(st.imass), 17)
    ref = s.assemble_dogs(dq)
    ctx.set_precision(prec)
    try:
        got = gpu_dogs(ctx, path, nZ, st, dq)
    finally:
        ctx.set_precision(fbgpu.FB_PREC_DF)
    for g, r, w in zip(got, ref, ("S", "T", "vna", "vnao", "dip")):
        assert g.shape == r.shape, w
        assert np.abs(g - r).max() <= TOL, (w, np.abs(g - r).max())


def test_dogs_graph_equals_plain(ctx, fdata_root):
    path, nZ, st = workload("sic_small", fdata_root, dogs=True)
    dq = charges(len(st.imass), 3)
    a = gpu_dogs(ctx, path, nZ, st, dq)
    b = gpu_dogs(ctx, path, nZ, st, dq, graph=True)
    b2 = gpu_dogs(ctx, path, nZ, st, dq, graph=True)  # replay
    for x, y, y2 in zip(a, b, b2):
        assert np.abs(x - y).max() <= TOL and np.abs(x - y2).max() <= TOL


def test_zero_charges_are_harris(ctx, fdata_root):
    path, nZ, st = workload("sic_small", fdata_root, dogs=True)
    n = len(st.imass)
    d = gpu_dogs(ctx, path, nZ, st, np.zeros((n, 3)))
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.set_precision(fbgpu.FB_PREC_FP64)
    ctx.assemble()
    h = [ctx.blocks(w) for w in ("S", "T", "vna", "vnao")]
    ctx.set_precision(fbgpu.FB_PREC_DF)
    for x, y in zip(d[:4], h):
        assert np.abs(x - y).max() <= TOL


def test_dogs_batch_matches_oracle(ctx, fdata_root):
    path = synth.fdata_dir_for("batch256", root=fdata_root, dogs=True)
    nZ = [14, 6]
    structs = [synth.diamond((1, 1, 2), 4.36, 0.1, 31, sp_a=1, sp_b=2, name="SiC16"),
               synth.diamond((2, 2, 1), 5.43, 0.1, 32, vacancy=0.05, name="Si32v"),
               synth.diamond((1, 1, 1), 4.36, 0.1, 33, sp_a=1, sp_b=2, name="SiC8cluster")]
    structs[2].icluster = 1
    fd = orc.Fdata(path, nZ)
    dqs = [charges(len(st.imass), 40 + k) for k, st in enumerate(structs)]
    ctx.read_Fdata(path, nZ)
    ctx.set_batch([(st.ratom, st.imass, st.lattice, st.icluster) for st in structs])
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    ctx.set_charges(np.concatenate(dqs))
    ctx.assemble()
    got = {w: ctx.blocks(w) for w in ("S", "T", "vna", "vnao", "dip")}
    off = ctx.batch_offsets()["block"]
    for k, st in enumerate(structs):
        s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
        ref = s.assemble_dogs(dqs[k])
        for r, w in zip(ref, ("S", "T", "vna", "vnao", "dip")):
            g = got[w][off[k]:off[k + 1]]
            assert np.abs(g - r).max() <= TOL, (k, w)


def test_dogs_errors(ctx, fdata_root):
    path0, nZ, st = workload("sic_small", fdata_root)
    ctx.read_Fdata(path0, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError) as e:      # Harris Fdata: no sub-cells
        ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    assert e.value.code == 3
    with pytest.raises(fbgpu.FBError) as e:      # no dipole_z table
        ctx.assemble_dipole_z()
    assert e.value.code == 3
    path, nZ, st = workload("sic_small", fdata_root, dogs=True)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_theory(fbgpu.FB_THEORY_DOGS)
    with pytest.raises(fbgpu.FBError) as e:      # charges first
        ctx.assemble()
    assert e.value.code == 11
    with pytest.raises(fbgpu.FBError) as e:      # at most 3 shells
        ctx.set_charges(np.zeros((len(st.imass), 4)))
    assert e.value.code == 12
    ctx.set_charges(charges(len(st.imass), 1))
    ctx.assemble()
    # the z-dipole blocks alone, in either theory
    ctx.set_theory(fbgpu.FB_THEORY_HARRIS)
    ctx.assemble_dipole_z()
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    ref = s.assemble_dogs(np.zeros((len(st.imass), 3)))[4]
    assert np.abs(ctx.blocks("dip") - ref).max() <= TOL
