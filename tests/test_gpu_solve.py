"""The k-point Lowdin solver on the GPU (fb_solve_k) against the oracle's
numpy restatement of kspace_Lowdin / diagonalize_S / diagonalize_H_Lowdin
(oracle/lowdin.py) on the oracle's own Bloch sums: the band energies, the
number of overlap eigenvalues dropped by the linear-dependence rule, and the
eigenvectors c up to a phase per well-separated level.  The synthetic
overlap tables give an indefinite S(k), so the drop-and-shift path of
diagonalize_S is exercised at every k-point."""
import numpy as np
import pytest

from conftest import workload
from oracle import lowdin
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

KPTS = np.array([[0.0, 0.0, 0.0], [0.11, -0.23, 0.31], [0.4, 0.1, -0.2]])


@pytest.mark.parametrize("name", ["si64"])
def test_solve_k_matches_oracle(fdata_root, name):
    torch = pytest.importorskip("torch")
    import fbgpu
    path, nZ, st = workload(name, fdata_root)
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors()
    S, T, vb, vbo = s.assemble()
    Hk = s.bloch(KPTS, T + vb + vbo)
    Sk = s.bloch(KPTS, S)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.assemble()
    n = int(ctx.L.fb_norbitals(ctx.h))
    c = torch.zeros((len(KPTS), n, n, 2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    eig, dropped = ctx.solve_k(KPTS, c_ptr=c.data_ptr())
    cg = c.cpu().numpy()
    cg = np.transpose(cg[..., 0] + 1j * cg[..., 1], (0, 2, 1))  # column-major storage
    for k in range(len(KPTS)):
        eps, cl, cref, S12, m = lowdin.solve_k(Hk[k], Sk[k])
        assert dropped[k] == m
        scale = max(1.0, np.abs(eps).max())
        assert np.abs(eig[k] - eps).max() <= 1e-8 * scale, (name, k, np.abs(eig[k] - eps).max())
        gap = np.minimum(np.diff(eps, prepend=-np.inf), np.diff(eps, append=np.inf))
        for j in np.nonzero(gap > 1e-4 * scale)[0]:
            a, b = cg[k][:, j], cref[:, j]
            ov = abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b))
            assert ov > 1.0 - 1e-8, (name, k, j, ov)
    assert dropped.max() > 0  # the drop-and-shift path ran
    ctx.close()


def test_solve_k_reports_an_undefined_lowdin_transform(fdata_root):
    """On the SiC64 cell the synthetic S(k) has 147 of 256 eigenvalues below
    1e-4: the reference's column shift then keeps negative eigenvalues in
    S^-1/2 (the oracle's restatement gives NaN); the GPU solver returns
    FB_ERR_SOLVER and stays usable."""
    import fbgpu
    path, nZ, st = workload("sic_small", fdata_root)
    s = orc.System(orc.Fdata(path, nZ), st.ratom, st.imass, st.lattice).neighbors()
    S, T, vb, vbo = s.assemble()
    with np.errstate(invalid="ignore"):
        S12, m = lowdin.s12_of(s.bloch(KPTS[:1], S)[0])
    assert 2 * m > S12.shape[0] and np.isnan(S12).any()
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.assemble()
    with pytest.raises(fbgpu.FBError) as e:
        ctx.solve_k(KPTS[:1])
    assert e.value.code == 14  # FB_ERR_SOLVER
    assert b"below 1e-4" in ctx.L.fb_last_error(ctx.h)
    path2, nZ2, st2 = workload("si64", fdata_root)
    ctx.read_Fdata(path2, nZ2)
    ctx.set_structure(st2.ratom, st2.imass, st2.lattice)
    ctx.driver_neighbors()
    ctx.assemble()
    eig, dropped = ctx.solve_k(KPTS[:1])
    assert np.isfinite(eig).all()
    ctx.close()


def test_solve_k_needs_assembled_blocks(fdata_root):
    import fbgpu
    path, nZ, st = workload("si64", fdata_root)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    with pytest.raises(fbgpu.FBError) as e:
        ctx.solve_k(KPTS[:1])
    assert e.value.code == 11  # FB_ERR_STATE
    ctx.close()
