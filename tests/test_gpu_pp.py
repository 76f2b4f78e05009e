"""Non-local pseudopotential (vnl) on the GPU against the oracle's
restatement of driver_neighbors_PP (c.SYSTEM/M_neighbors_PP.f90),
assemble_svnl / assemble_vnl_2c / assemble_vnl_3c
(j.ASSEMBLERS/M_assemble_PP_{2c,3c}.f90), Dassemble_svnl / Dassemble_vnl_2c
/ Dassemble_vnl_3c (k.DASSEMBLERS/M_Dassemble_PP_{2c,3c}.f90) and the vnl
terms of build_forces: the PP, PPx and PPp maps, maps, points and common
triplets bit-exact (1-based, as the reference numbers them), svnl and vnl
blocks to 1e-10 eV per element, every vnl force array to 1e-10 eV/Angstrom,
plain and as one CUDA graph, and the call-order errors."""
import numpy as np
import pytest

import fbgpu
from conftest import workload, symmetric_denmat
from fbgpu import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    c = fbgpu.Context(0)
    yield c
    c.close()


def cases(fdata_root):
    out = {}
    for name in ("sic_small", "cho_small", "si64", "sic_vac"):
        path, nZ, st = workload(name, fdata_root)
        out[name] = (path, nZ, st)
    path, _, _ = workload("sic_small", fdata_root)
    cl = synth.diamond((1, 1, 1), 4.36, 0.1, 41, sp_a=1, sp_b=2, name="SiC8cluster")
    cl.icluster = 1
    out["sic_cluster"] = (path, [14, 6], cl)
    return out


def rho_pp_for(s, st, fd, seed):
    """a density over PPp, symmetric across the reverse pair as the
    solver's s%denmat_PP is"""
    from test_oracle_pp import _sym_rho
    return _sym_rho(s, fd, st, seed)


def run_both(ctx, path, nZ, st, graph=False):
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors().neighbors_pp()
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice, st.icluster)
    ctx.driver_neighbors()
    sizes = ctx.driver_neighbors_PP()
    return fd, s, sizes


@pytest.mark.parametrize("name", ["sic_small", "cho_small", "si64", "sic_vac", "sic_cluster"])
def test_pp_maps_match_oracle(ctx, fdata_root, name):
    path, nZ, st = cases(fdata_root)[name]
    fd, s, sizes = run_both(ctx, path, nZ, st)
    assert (sizes["npp"], sizes["nppx"], sizes["nppp"], sizes["ntrip"]) == (s.npp, s.nppx, s.nppp, s.ntrip_pp)
    assert (sizes["nsvnl"], sizes["nvnl"]) == (s.nsvnl, s.nvnl)
    for which, key in ((fbgpu.FB_PP_MAP, "PP"), (fbgpu.FB_PPX_MAP, "PPx"), (fbgpu.FB_PPP_MAP, "PPp")):
        g, r = ctx.pp_neighbors(which), s.pp[key]
        assert np.array_equal(g["neighn"], np.diff(r["off"]))
        assert np.array_equal(g["neigh_j"], r["j"] + 1)
        assert np.array_equal(g["neigh_b"], r["b"])
        assert np.array_equal(g["self"], r["self"] + 1)
        if key != "PPp":
            assert np.array_equal(g["map"], r["map"] + 1)
        if key == "PPx":
            assert np.array_equal(g["point"], r["point"] + 1)
    g, r = ctx.pp_common(), s.pp["common"]
    assert np.array_equal(g["ncommon"], np.diff(r["off"]))
    for gk, rk, add in (("iatom_j", "i", 1), ("iatom_b", "ib", 0), ("jatom_j", "j", 1), ("jatom_b", "jb", 0),
                        ("neigh_common", "m", 1), ("m31", "m31", 1), ("m32", "m32", 1)):
        assert np.array_equal(g[gk], r[rk] + add), gk


@pytest.mark.parametrize("name", ["sic_small", "cho_small", "si64", "sic_vac", "sic_cluster"])
def test_vnl_blocks_and_forces_match_oracle(ctx, fdata_root, name):
    path, nZ, st = cases(fdata_root)[name]
    fd, s, _ = run_both(ctx, path, nZ, st)
    svnl, vnl = s.assemble_pp()
    ctx.assemble(fbgpu.FB_VNL)
    assert np.abs(ctx.blocks("svnl") - svnl).max() <= TOL
    assert np.abs(ctx.blocks("vnl") - vnl).max() <= TOL
    rho_pp = rho_pp_for(s, st, fd, 5)
    ref = s.dassemble_pp(rho_pp)
    ctx.set_denmat_pp(rho_pp)
    ctx.Dassemble(fbgpu.FB_VNL2C | fbgpu.FB_VNL3C)
    assert np.abs(ctx.blocks("dsvnl") - ref["dsvnl"]).max() <= TOL
    for k in ("vnl_atom", "vnl_ontop", "f3nla", "f3nlb", "f3nlc", "vnl"):
        assert np.abs(ctx.forces(k) - ref[k]).max() <= TOL, k
    # only vnl terms requested: ftot is the vnl addition of build_forces
    assert np.abs(ctx.forces("ftot") - ref["ftot_vnl"]).max() <= TOL


def test_vnl_with_harris_forces_and_graph(ctx, fdata_root):
    path, nZ, st = cases(fdata_root)["sic_small"]
    fd, s, _ = run_both(ctx, path, nZ, st)
    norb = np.array([fd.norb(int(q)) for q in st.imass])
    rho, cape = symmetric_denmat(s, norb, 7)
    rho_pp = rho_pp_for(s, st, fd, 9)
    href = s.dassemble(rho, cape)["ftot"]
    vref = s.dassemble_pp(rho_pp)["ftot_vnl"]
    ctx.set_precision(fbgpu.FB_PREC_FP64)
    ctx.set_denmat(rho, cape)
    ctx.set_denmat_pp(rho_pp)
    what = fbgpu.FB_ALL | fbgpu.FB_VNL
    ctx.assemble(what)
    ctx.Dassemble(what)
    assert np.abs(ctx.forces("ftot") - (href + vref)).max() <= TOL
    _, vnl = s.assemble_pp()
    for _ in range(2):  # capture, then replay
        ctx.assemble_graph(what | fbgpu.FB_FORCES)
        assert np.abs(ctx.blocks("vnl") - vnl).max() <= TOL
        assert np.abs(ctx.forces("ftot") - (href + vref)).max() <= TOL
    ctx.set_precision(fbgpu.FB_PREC_DF)


def test_vnl_call_order_errors(ctx, fdata_root):
    path, nZ, st = cases(fdata_root)["sic_small"]
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError) as e:      # maps first
        ctx.assemble(fbgpu.FB_SVNL)
    assert e.value.code == 11
    ctx.driver_neighbors_PP()
    with pytest.raises(fbgpu.FBError) as e:      # svnl before vnl
        ctx.assemble(fbgpu.FB_VNL2C)
    assert e.value.code == 11
    ctx.assemble(fbgpu.FB_SVNL | fbgpu.FB_VNL2C)
    with pytest.raises(fbgpu.FBError) as e:      # the PP density first
        ctx.Dassemble(fbgpu.FB_VNL2C)
    assert e.value.code == 11
    ctx.update_positions(st.ratom)
    with pytest.raises(fbgpu.FBError) as e:      # new positions: the maps are stale
        ctx.pp_sizes()
    assert e.value.code == 11
    structs = [(st.ratom, st.imass, st.lattice, 0), (st.ratom, st.imass, st.lattice, 0)]
    ctx.set_batch(structs)
    with pytest.raises(fbgpu.FBError) as e:      # single structures
        ctx.driver_neighbors_PP()
    assert e.value.code == 13
