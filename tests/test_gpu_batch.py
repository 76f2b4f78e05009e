"""Batched assembly: several structures of uneven size (periodic Si, SiC
with vacancies, and a cluster) set as one batch.  Every structure's slice of
the batch must equal the oracle run on that structure alone: neighbor maps
bit-exact in the reference's per-structure numbering, blocks and forces to
1e-10 eV (eV/Angstrom)."""
import numpy as np
import pytest

from conftest import symmetric_denmat
from fbgpu import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10


def batch_cases():
    st = [
        synth.diamond((2, 2, 1), 5.43, 0.1, 21, vacancy=0.05, name="Si32v"),
        synth.diamond((1, 1, 2), 4.36, 0.1, 22, sp_a=1, sp_b=2, name="SiC16"),
        synth.diamond((2, 2, 2), 4.36, 0.1, 23, sp_a=1, sp_b=2, vacancy=0.04, name="SiC64v"),
        synth.diamond((1, 1, 1), 4.36, 0.1, 24, sp_a=1, sp_b=2, name="SiC8cluster"),
        synth.diamond((1, 2, 2), 5.43, 0.1, 25, name="Si32"),
    ]
    st[3].icluster = 1
    return st


@pytest.fixture(scope="module")
def batch(fdata_root):
    import fbgpu
    path = synth.fdata_dir_for("batch256", root=fdata_root)
    nZ = [14, 6]
    structs = batch_cases()
    fd = orc.Fdata(path, nZ)
    refs = []
    for k, st in enumerate(structs):
        s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=st.icluster).neighbors()
        norb = np.array([fd.norb(int(q)) for q in st.imass])
        rho, cape = symmetric_denmat(s, norb, 100 + k)
        refs.append((s, s.assemble(), rho, cape, s.dassemble(rho, cape)))
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_batch([(st.ratom, st.imass, st.lattice, st.icluster) for st in structs])
    yield ctx, structs, refs
    ctx.close()


def test_batch_neighbors(batch):
    ctx, structs, refs = batch
    P, T, NB = ctx.driver_neighbors()
    assert P == sum(r[0].npairs for r in refs)
    assert T == sum(r[0].ntrip for r in refs)
    assert NB == sum(r[0].nblock for r in refs)
    off = ctx.batch_offsets()
    nb = ctx.neighbors()
    cm = ctx.common_neighbors()
    for k, (s, *_rest) in enumerate(refs):
        a0, a1 = off["atom"][k], off["atom"][k + 1]
        p0, p1 = off["pair"][k], off["pair"][k + 1]
        t0, t1 = off["trip"][k], off["trip"][k + 1]
        assert a1 - a0 == structs[k].natoms
        assert (p1 - p0, t1 - t0) == (s.npairs, s.ntrip)
        assert off["block"][k + 1] - off["block"][k] == s.nblock
        assert np.array_equal(nb["neighn"][a0:a1], np.diff(s.pair_off))
        assert np.array_equal(nb["neigh_j"][p0:p1], s.neigh_j[:s.npairs] + 1)
        assert np.array_equal(nb["neigh_b"][p0:p1], s.neigh_b[:s.npairs])
        assert np.array_equal(nb["neigh_back"][p0:p1], s.neigh_back[:s.npairs] + 1)
        assert np.array_equal(nb["neigh_self"][a0:a1], s.neigh_self + 1)
        assert np.array_equal(nb["blk_off"][p0:p1 + 1] - off["block"][k], s.blk_off)
        assert np.array_equal(cm["ncommon"][a0:a1], np.diff(s.trip_off))
        assert np.array_equal(cm["iatom_common_j"][t0:t1], s.ci_j[:s.ntrip] + 1)
        assert np.array_equal(cm["jatom_common_j"][t0:t1], s.cj_j[:s.ntrip] + 1)
        assert np.array_equal(cm["iatom_common_b"][t0:t1], s.ci_b[:s.ntrip])
        assert np.array_equal(cm["jatom_common_b"][t0:t1], s.cj_b[:s.ntrip])
        assert np.array_equal(cm["neigh_common"][t0:t1], s.cneigh[:s.ntrip] + 1)


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_blocks_and_forces(batch, prec):
    ctx, structs, refs = batch
    ctx.set_precision(prec)
    ctx.driver_neighbors()
    off = ctx.batch_offsets()
    ctx.assemble()
    got = {k: ctx.blocks(k) for k in ("S", "T", "vna", "vnao")}
    rho = np.concatenate([r[2] for r in refs])
    cape = np.concatenate([r[3] for r in refs])
    ctx.set_denmat(rho, cape)
    ctx.Dassemble()
    f = {k: ctx.forces(k) for k in ("ftot", "f3naa", "f3nab", "f3nac", "kinetic", "vna", "pulay")}
    for k, (s, blocks, _rho, _cape, fref) in enumerate(refs):
        b0, b1 = off["block"][k], off["block"][k + 1]
        for key, ref in zip(("S", "T", "vna", "vnao"), blocks):
            err = np.abs(got[key][b0:b1] - ref).max()
            assert err <= TOL, "%s prec %d %s %.3e" % (structs[k].name, prec, key, err)
        a0, a1 = off["atom"][k], off["atom"][k + 1]
        for key, arr in f.items():
            err = np.abs(arr[3 * a0:3 * a1] - fref[key]).max()
            assert err <= TOL, "%s prec %d %s %.3e" % (structs[k].name, prec, key, err)
    ctx.set_precision(1)


def test_batch_graph_persistent(batch):
    """The batch through one graph launch with persistent launch shapes."""
    import fbgpu
    ctx, structs, refs = batch
    ctx.set_precision(1)
    ctx.driver_neighbors()
    off = ctx.batch_offsets()
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 64, 4, 2)
    rho = np.concatenate([r[2] for r in refs])
    cape = np.concatenate([r[3] for r in refs])
    ctx.set_denmat(rho, cape)
    ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
    got = {k: ctx.blocks(k) for k in ("S", "T", "vna", "vnao")}
    ftot = ctx.forces("ftot")
    for k, (s, blocks, _rho, _cape, fref) in enumerate(refs):
        b0, b1 = off["block"][k], off["block"][k + 1]
        for key, ref in zip(("S", "T", "vna", "vnao"), blocks):
            assert np.abs(got[key][b0:b1] - ref).max() <= TOL
        a0, a1 = off["atom"][k], off["atom"][k + 1]
        assert np.abs(ftot[3 * a0:3 * a1] - fref["ftot"]).max() <= TOL
    for k in fbgpu.TUNABLE:
        ctx.set_launch(k, 128, 0, 1)
