"""The allocation-free force entry point, fb_dassemble_noalloc.

Some callers cannot allocate GPU memory while they run the force pass (a
driver that gives the whole device to a pre-sized pool, an MD loop that may
not touch the CUDA allocator between steps).  fb_dassemble_noalloc keeps its
intermediate terms in a statically sized device array of the library instead
of allocating them.  These tests call it through the C ABI, twice in a row
(every call reuses the same static array), and check it against the oracle
and against the allocating path (fb_dassemble + fb_get_forces).  The density
matrix stored on the context (fb_set_denmat) differs from the one passed to
the entry point, so a call that read the stored one would fail.
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
    return ctx, st, s, norb


def _call(ctx, d_rho, d_cape, d_f):
    return ctx.L.fb_dassemble_noalloc(ctx.h, C.c_void_p(d_rho.data_ptr()),
                                      None if d_cape is None else C.c_void_p(d_cape.data_ptr()),
                                      C.c_void_p(d_f.data_ptr()))


@pytest.mark.parametrize("name", ["si64", "cho_small"])
def test_noalloc_matches_oracle_and_allocating_path(fdata_root, name):
    torch = pytest.importorskip("torch")
    import fbgpu
    ctx, st, s, norb = _setup(name, fdata_root)
    rho_a, cape_a = symmetric_denmat(s, norb, 1234)
    rho_b, cape_b = symmetric_denmat(s, norb, 4321)
    ref_b = s.dassemble(rho_b, cape_b)["ftot"]
    # the allocating path with the density matrix the entry point is given
    ctx.set_denmat(rho_b, cape_b)
    ctx.Dassemble(fbgpu.FB_ALL)
    alloc_b = ctx.forces("ftot")
    # then a different density matrix stored on the context
    ctx.set_denmat(rho_a, cape_a)
    d_rho = torch.from_numpy(rho_b).cuda()
    d_cape = torch.from_numpy(cape_b).cuda()
    for call in range(2):
        d_f = torch.full((3 * st.natoms,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        code = _call(ctx, d_rho, d_cape, d_f)
        assert code == 0, ctx.L.fb_last_error(ctx.h).decode()
        got = d_f.cpu().numpy()
        err_o = np.abs(got - ref_b).max()
        err_a = np.abs(got - alloc_b).max()
        assert err_o <= TOL, "call %d: max |diff| vs oracle %.3e" % (call, err_o)
        assert err_a <= TOL, "call %d: max |diff| vs fb_dassemble %.3e" % (call, err_a)
    ctx.close()


def test_noalloc_call_leaves_free_memory_unchanged(fdata_root):
    torch = pytest.importorskip("torch")
    ctx, st, s, norb = _setup("si64", fdata_root)
    rho, cape = symmetric_denmat(s, norb, 99)
    d_rho = torch.from_numpy(rho).cuda()
    d_cape = torch.from_numpy(cape).cuda()
    d_f = torch.zeros(3 * st.natoms, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert _call(ctx, d_rho, d_cape, d_f) == 0
    free0 = torch.cuda.mem_get_info()[0]
    assert _call(ctx, d_rho, d_cape, d_f) == 0
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, "free device memory changed by %d bytes across a call" % (free1 - free0)
    ctx.close()


def test_noalloc_without_cape_drops_pulay(fdata_root):
    torch = pytest.importorskip("torch")
    ctx, st, s, norb = _setup("si64", fdata_root)
    rho, cape = symmetric_denmat(s, norb, 1234)
    ref = s.dassemble(rho, np.zeros_like(cape))["ftot"]
    d_rho = torch.from_numpy(rho).cuda()
    d_f = torch.zeros(3 * st.natoms, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert _call(ctx, d_rho, None, d_f) == 0
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
    code = _call(ctx, d_rho, None, d_f)
    assert code == 12  # FB_ERR_CAPACITY
    assert b"at most" in ctx.L.fb_last_error(ctx.h)
    ctx.close()
