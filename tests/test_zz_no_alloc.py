"""The allocation-free force entry point, fb_dassemble_noalloc.

Some callers cannot allocate GPU memory while they run the force pass (a
driver that gives the whole device to a pre-sized pool, an MD loop that may
not touch the CUDA allocator between steps).  fb_dassemble_noalloc keeps its
intermediate terms in a statically sized device array of the library instead
of allocating them.  These tests call it through the C ABI and check it
against the allocating path (fb_dassemble + fb_get_forces), twice in a row,
because every call reuses the same static array.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-10  # eV/Angstrom per component, as the other force parity tests


def _setup(name, fdata_root):
    import fbgpu
    path, nZ, st = workload(name, fdata_root)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 1234)
    return ctx, st, rho, cape


@pytest.mark.parametrize("name", ["si64", "cho_small"])
def test_noalloc_matches_allocating_path(fdata_root, name):
    torch = pytest.importorskip("torch")
    import fbgpu
    ctx, st, rho, cape = _setup(name, fdata_root)
    ctx.set_denmat(rho, cape)
    ctx.Dassemble(fbgpu.FB_ALL)
    ref = ctx.forces("ftot")
    d_rho = torch.from_numpy(rho).cuda()
    d_cape = torch.from_numpy(cape).cuda()
    for call in range(2):
        d_f = torch.full((3 * st.natoms,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st_code = ctx.L.fb_dassemble_noalloc(ctx.h, C.c_void_p(d_rho.data_ptr()), C.c_void_p(d_cape.data_ptr()),
                                             C.c_void_p(d_f.data_ptr()))
        assert st_code == 0, ctx.L.fb_last_error(ctx.h).decode()
        got = d_f.cpu().numpy()
        err = np.abs(got - ref).max()
        assert err <= TOL, "call %d: max |diff| %.3e" % (call, err)
    ctx.close()


def test_noalloc_without_cape_drops_pulay(fdata_root):
    torch = pytest.importorskip("torch")
    import fbgpu
    ctx, st, rho, cape = _setup("si64", fdata_root)
    ctx.set_denmat(rho, None)
    ctx.Dassemble(fbgpu.FB_ALL)
    ref = ctx.forces("ftot")
    d_rho = torch.from_numpy(rho).cuda()
    d_f = torch.zeros(3 * st.natoms, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert ctx.L.fb_dassemble_noalloc(ctx.h, C.c_void_p(d_rho.data_ptr()), None, C.c_void_p(d_f.data_ptr())) == 0
    assert np.abs(d_f.cpu().numpy() - ref).max() <= TOL
    ctx.close()


def test_noalloc_rejects_oversized_system(fdata_root):
    torch = pytest.importorskip("torch")
    import fbgpu
    path, nZ, st = workload("sic4096", fdata_root)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    P, T, NB = ctx.driver_neighbors()
    assert P > 65536
    d_rho = torch.zeros(NB, dtype=torch.float64, device="cuda")
    d_f = torch.zeros(3 * st.natoms, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    code = ctx.L.fb_dassemble_noalloc(ctx.h, C.c_void_p(d_rho.data_ptr()), None, C.c_void_p(d_f.data_ptr()))
    assert code == 12  # FB_ERR_CAPACITY
    assert b"at most" in ctx.L.fb_last_error(ctx.h)
    ctx.close()
