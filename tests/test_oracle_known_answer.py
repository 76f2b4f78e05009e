"""Known answers for whole assembled blocks (CPU, oracle).

The reference ships no golden data and cannot be built here, so these
tests pin the oracle's assemblers to a closed-form evaluation of the
reference's formulas: polynomial tables that the interpolators reproduce
exactly, and the blocks of a three-atom cluster computed directly from the
geometry, the Legendre sum and the Slater-Koster transformation
(known_answer.py).  Every off-diagonal pair block of the cluster receives
exactly one three-center term, from the third atom."""
import numpy as np
import pytest

import known_answer as ka
from oracle import oracle as orc


@pytest.fixture(scope="module")
def poly(tmp_path_factory):
    path = str(tmp_path_factory.mktemp("ka") / "poly")
    coef2, coef3 = ka.write_poly_fdata(path)
    return path, coef2, coef3


def _system(path):
    r, imass, lat = ka.cluster()
    s = orc.System(orc.Fdata(path, [14]), r, imass, lat, icluster=1).neighbors()
    return s, r


def test_three_center_blocks_known_answer(poly):
    path, coef2, coef3 = poly
    s, r = _system(path)
    assert s.npairs == 9 and s.ntrip == 6
    vb3 = s.assemble_3c_only()
    for i in range(3):
        for j in range(3):
            if i == j:
                continue
            k = 3 - i - j
            want = ka.bcna_block(coef3, r[i], r[j], r[k])
            got = ka.block_of(vb3, s.blk_off, s.pair_off, s.neigh_j, i, j)
            assert np.abs(got - want).max() < 1e-9 * max(1.0, np.abs(want).max()), (i, j)


def test_overlap_blocks_known_answer(poly):
    path, coef2, coef3 = poly
    s, r = _system(path)
    S = s.assemble()[0]
    for i in range(3):
        for j in range(3):
            if i == j:
                continue
            want = ka.overlap_block(coef2, r[i], r[j])
            got = ka.block_of(S, s.blk_off, s.pair_off, s.neigh_j, i, j)
            assert np.abs(got - want).max() < 1e-10 * max(1.0, np.abs(want).max()), (i, j)
