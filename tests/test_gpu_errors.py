"""The reference's `stop` conditions on the GPU path, as status codes.

The reference stops the process when two atoms are closer than 0.5 A
(c.SYSTEM/M_neighbors.f90:421-430) and when a two-center interpolation is
asked for a distance beyond its table (e.FDATA/M_Fdata_2c.f90:347-353).  The
library's kernels set a device status flag instead; the host reads it after
the launch and returns FB_ERR_ATOMS_CLOSE or FB_ERR_X_TOO_LARGE.  Nothing
faults: the kernels finish, and the context stays usable afterwards.  The
oracle reports the same conditions with the same codes.
"""
import os
import shutil

import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

FB_ERR_X_TOO_LARGE = 5
FB_ERR_ATOMS_CLOSE = 6


def test_atoms_too_close_is_a_status(fdata_root):
    import fbgpu
    path, nZ, st = workload("si64", fdata_root)
    r = st.ratom.copy()
    r[1] = r[0] + np.array([0.4, 0.0, 0.0])
    with pytest.raises(orc.OracleError) as eo:
        orc.System(orc.Fdata(path, nZ), r, st.imass, st.lattice).neighbors()
    assert eo.value.code == FB_ERR_ATOMS_CLOSE
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(r, st.imass, st.lattice)
    with pytest.raises(fbgpu.FBError) as eg:
        ctx.driver_neighbors()
    assert eg.value.code == FB_ERR_ATOMS_CLOSE
    # the context is usable again with valid positions
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors()
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    assert ctx.driver_neighbors() == (s.npairs, s.ntrip, s.nblock)
    ctx.assemble()
    assert np.abs(ctx.blocks("S") - s.assemble()[0]).max() <= 1e-10
    ctx.close()


def _shrink_overlap_table(src, dst, xmax_new):
    """A copy of an Fdata set whose overlap table (interaction 1) claims a
    shorter range: the pair cutoff then reaches beyond the table."""
    shutil.copytree(src, dst)
    fn = os.path.join(dst, "2c.14.14.dir")
    lines = open(fn).read().splitlines()
    out = []
    for ln in lines:
        f = ln.split()
        if len(f) == 7 and f[1] == "1":
            f[6] = "%.6f" % xmax_new
            ln = "%5s %3s %3s %-28s %3s %4s %9s" % tuple(f)
        out.append(ln)
    open(fn, "w").write("\n".join(out) + "\n")


def test_distance_beyond_table_is_a_status(fdata_root, tmp_path):
    import fbgpu
    path, nZ, st = workload("si64", fdata_root)
    dst = str(tmp_path / "short_overlap")
    _shrink_overlap_table(path, dst, 3.0)
    s = orc.System(orc.Fdata(dst, nZ), st.ratom, st.imass, st.lattice).neighbors()
    with pytest.raises(orc.OracleError) as eo:
        s.assemble()
    assert eo.value.code == FB_ERR_X_TOO_LARGE
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(dst, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    assert ctx.driver_neighbors() == (s.npairs, s.ntrip, s.nblock)
    with pytest.raises(fbgpu.FBError) as eg:
        ctx.assemble(fbgpu.FB_S)
    assert eg.value.code == FB_ERR_X_TOO_LARGE
    # the kinetic table keeps its full range: that call succeeds afterwards
    ctx.assemble(fbgpu.FB_T)
    ref_t = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors().assemble()[1]
    assert np.abs(ctx.blocks("T") - ref_t).max() <= 1e-10
    ctx.close()
