"""fb_step_forces: one value + force step through host buffers with the
copies overlapped with the kernels, against the oracle (1e-10 eV per block
element and eV/Angstrom per force component) and against the separate calls,
in both precisions, twice in a row, with and without cape.  By default the
two-center kernels run on a second stream beside the common-neighbor stage;
with per-kernel timing on, the step runs in the serial order: both orders
are checked."""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("serial", [False, True])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name", ["si64", "cho_small"])
def test_step_forces_matches_oracle(fdata_root, name, prec, serial):
    torch = pytest.importorskip("torch")
    import fbgpu
    path, nZ, st = workload(name, fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    blocks = s.assemble()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 21)
    fref = s.dassemble(rho, cape)["ftot"]
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_precision(prec)
    ctx.set_timing(serial)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    nb = s.nblock
    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    outs = [pin(nb) for _ in range(4)] + [pin(3 * st.natoms)]
    for call in range(2):
        for o in outs:
            o[:] = np.nan
        ctx.step_forces(st.ratom, rho, cape, *outs)
        for key, got, ref in zip(("S", "T", "vna", "vnao"), outs[:4], blocks):
            err = np.abs(got - ref).max()
            assert err <= 1e-10, (call, key, err)
        assert np.abs(outs[4] - fref).max() <= 1e-10, call
    # without cape: no Pulay term, as fb_set_denmat(rho, NULL)
    ctx.step_forces(None, rho, None, None, None, None, None, outs[4])
    f0 = s.dassemble(rho, np.zeros_like(cape))["ftot"]
    assert np.abs(outs[4] - f0).max() <= 1e-10
    ctx.close()


@pytest.mark.parametrize("name", ["si64", "cho_small"])
def test_step_orders_agree(fdata_root, name):
    """The overlapped and the serial step give the same blocks (bit for bit:
    the value blocks are written, not accumulated, by the two-center kernel)
    and the same forces to 1e-12 eV/Angstrom (atomic adds in either order)."""
    torch = pytest.importorskip("torch")
    import fbgpu
    path, nZ, st = workload(name, fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 22)
    nb = s.nblock
    pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    got = []
    for serial in (False, True):
        ctx = fbgpu.Context(0)
        ctx.read_Fdata(path, nZ)
        ctx.set_timing(serial)
        ctx.set_structure(st.ratom, st.imass, st.lattice)
        outs = [pin(nb) for _ in range(4)] + [pin(3 * st.natoms)]
        ctx.step_forces(st.ratom, rho, cape, *outs)
        got.append([o.copy() for o in outs])
        ctx.close()
    for k in (0, 1, 3):
        assert np.array_equal(got[0][k], got[1][k]), k
    assert np.abs(got[0][2] - got[1][2]).max() <= 1e-12
    assert np.abs(got[0][4] - got[1][4]).max() <= 1e-12
