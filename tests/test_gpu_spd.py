"""The d-orbital paths of the kernels (s, p, d basis; the HASD
instantiations): a Ti/Si cell with a Ti s + p + d basis against the oracle,
the Harris blocks and forces and the McWEDA vxc blocks and forces, to 1e-10
per element.  The double-float three-center kernels serve s and sp bases
only, so a system with d orbitals runs the FP64 kernels in both precision
settings."""
import os

import numpy as np
import pytest

import fbgpu
from conftest import symmetric_denmat
from fbgpu import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10


def spd_case(root, vxc=False):
    path = os.path.join(root, "TiSi_rc50" + ("_VXC" if vxc else ""))
    stamp = os.path.join(path, ".complete")
    if not os.path.exists(stamp):
        synth.write_fdata(path, [synth.ti(), synth.si()], vxc=vxc)
        with open(stamp, "w") as f:
            f.write("ok\n")
    st = synth.diamond((1, 1, 1), 5.2, 0.1, 17, sp_a=1, sp_b=2, name="TiSi8")
    return path, [22, 14], st


@pytest.fixture(scope="module")
def ctx():
    c = fbgpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_spd_blocks_and_forces(ctx, fdata_root, prec):
    path, nZ, st = spd_case(fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    assert fd.norb(1) == 9
    S0, T0, vb0, vbo0 = s.assemble()
    rho, cape = symmetric_denmat(s, np.array([fd.norb(int(k)) for k in st.imass]), 9)
    ref = s.dassemble(rho, cape)
    ctx.set_precision(prec)
    try:
        ctx.read_Fdata(path, nZ)
        ctx.set_structure(st.ratom, st.imass, st.lattice)
        ctx.driver_neighbors()
        ctx.assemble(fbgpu.FB_ALL)
        for key, want in (("S", S0), ("T", T0), ("vna", vb0), ("vnao", vbo0)):
            assert np.abs(ctx.blocks(key) - want).max() <= TOL, key
        ctx.set_denmat(rho, cape)
        ctx.Dassemble(fbgpu.FB_ALL)
        for key in ("ftot", "kinetic", "vna", "pulay", "f3naa", "f3nab", "f3nac", "vna_ontop", "vna_atom"):
            assert np.abs(ctx.forces(key) - ref[key]).max() <= TOL, key
        ctx.assemble_graph(fbgpu.FB_ALL | fbgpu.FB_FORCES)
        assert np.abs(ctx.forces("ftot") - ref["ftot"]).max() <= TOL
    finally:
        ctx.set_precision(1)


def test_spd_vxc(ctx, fdata_root):
    path, nZ, st = spd_case(fdata_root, vxc=True)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    rho, cape = symmetric_denmat(s, np.array([fd.norb(int(k)) for k in st.imass]), 4)
    ref = s.dassemble_vxc(rho)
    vals = ref["values"]
    harris = s.dassemble(rho, cape)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.set_denmat(rho, cape)
    what = fbgpu.FB_ALL | fbgpu.FB_VXC
    ctx.assemble(what)
    for key in ("rho_in", "rho_bond", "vxc"):
        assert np.abs(ctx.blocks(key) - vals[key]).max() <= TOL, key
    assert np.abs(ctx.blocks("wrho_in").reshape(-1, 9) - vals["wrho_in"]).max() <= TOL
    ctx.Dassemble(what)
    for key in ("vxc_off_site", "vxc_on_site", "f3xca", "f3xcb", "f3xcc"):
        assert np.abs(ctx.forces(key) - ref[key]).max() <= TOL, key
    assert np.abs(ctx.forces("ftot") - (harris["ftot"] + ref["ftot_add"])).max() <= TOL
