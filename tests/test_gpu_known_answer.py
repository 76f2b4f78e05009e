"""Known answers for whole assembled blocks on the GPU path: the S blocks and
the three-center vna terms of a three-atom Si cluster on polynomial Fdata,
against their closed form (known_answer.py), through the C ABI, in both
precision modes of the three-center kernels, and through the graph step
whose force kernel also adds the value-pass three-center terms."""
import numpy as np
import pytest

import known_answer as ka
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def poly(tmp_path_factory):
    path = str(tmp_path_factory.mktemp("ka_gpu") / "poly")
    coef2, coef3 = ka.write_poly_fdata(path)
    return path, coef2, coef3


@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_blocks_known_answer(poly, prec):
    import fbgpu
    path, coef2, coef3 = poly
    r, imass, lat = ka.cluster()
    s = orc.System(orc.Fdata(path, [14]), r, imass, lat, icluster=1).neighbors()
    vb2 = s.assemble(with3c=False)[2]
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, [14])
    ctx.set_precision(prec)
    ctx.set_structure(r, imass, lat, icluster=1)
    assert ctx.driver_neighbors() == (s.npairs, s.ntrip, s.nblock)
    nb = ctx.neighbors()
    pair_off = np.concatenate([[0], np.cumsum(nb["neighn"])])
    nj0 = nb["neigh_j"] - 1
    for step in ("calls", "graph"):
        if step == "calls":
            ctx.assemble()
        else:
            rng = np.random.default_rng(1)
            ctx.set_denmat(rng.normal(0.0, 0.1, s.nblock), rng.normal(0.0, 0.05, s.nblock))
            ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
        S = ctx.blocks("S")
        vb3 = ctx.blocks("vna") - vb2
        for i in range(3):
            for j in range(3):
                if i == j:
                    continue
                k = 3 - i - j
                want = ka.bcna_block(coef3, r[i], r[j], r[k])
                got = ka.block_of(vb3, nb["blk_off"], pair_off, nj0, i, j)
                assert np.abs(got - want).max() < 1e-9 * max(1.0, np.abs(want).max()), (step, i, j)
                want = ka.overlap_block(coef2, r[i], r[j])
                got = ka.block_of(S, nb["blk_off"], pair_off, nj0, i, j)
                assert np.abs(got - want).max() < 1e-10 * max(1.0, np.abs(want).max()), (step, i, j)
    ctx.close()
