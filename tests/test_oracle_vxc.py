"""The oracle's restatement of the McWEDA exchange-correlation value pass
(j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90,
j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90,
g.XC_FUNCTIONALS/lda_ceperley_alder.f90).

The Ceperley-Alder functional is pinned to the published Perdew-Zunger
parameterisation (an independent restatement below) and to its own
derivative identities by central differences; the assembled densities and
vxc blocks are checked for the symmetries the synthetic tables carry
(Hermitian across neigh_back), for the structure of the formulas (rho_bond
is rho_in without the three-center and the neighbors' atom terms; vxc =
vxc_bond + vxc_SN - vxc_SN_bond), and for both branches of the functional
being reached on the test systems."""
import numpy as np
import pytest

from conftest import workload
from oracle import oracle as orc

P_ABOHR = 0.529177
P_HARTREE = 14.39975 / P_ABOHR


def pz81_exc(rs):
    """Exchange + correlation energy per electron (Hartree) of the
    Perdew-Zunger fit to Ceperley-Alder (PRB 23, 5048 (1981), Table XII)."""
    ex = -0.4581652 / rs
    if rs >= 1.0:
        ec = -0.1423 / (1.0 + 1.0529 * np.sqrt(rs) + 0.3334 * rs)
    else:
        ec = -0.0480 + 0.0311 * np.log(rs) - 0.0116 * rs + 0.0020 * rs * np.log(rs)
    return ex + ec


def _rh_of_rs(rs):
    """Density in 1/A^3 whose smoothed value sqrt(rh^2 + 1e-6) has radius rs."""
    rho_au = 3.0 / (4.0 * np.pi * rs ** 3)
    rhx = rho_au / P_ABOHR ** 3
    return np.sqrt(rhx * rhx - 1.0e-6)


@pytest.mark.parametrize("rs", [0.4, 0.8, 1.5, 3.0, 6.0])
def test_lda_matches_published_fit(rs):
    exc = orc.lda_ceperley_alder(_rh_of_rs(rs))[0]
    assert abs(exc - pz81_exc(rs) * P_HARTREE) < 2e-6 * abs(exc)


@pytest.mark.parametrize("rh", [0.02, 0.3, 1.2, 2.5, 8.0])
def test_lda_derivative_identities(rh):
    h = 1e-5 * rh
    f = orc.lda_ceperley_alder
    exc, muxc, dexc, d2exc, dmuxc, d2muxc = f(rh)
    rhx = np.sqrt(rh * rh + 1e-6)
    # muxc = d(rho exc)/d rho and dmuxc = d muxc / d rho, rho = sqrt(rh^2 + 1e-6)
    drhx = np.sqrt((rh + h) ** 2 + 1e-6) - np.sqrt((rh - h) ** 2 + 1e-6)
    fp, fm = f(rh + h), f(rh - h)
    n_p, n_m = np.sqrt((rh + h) ** 2 + 1e-6), np.sqrt((rh - h) ** 2 + 1e-6)
    # the fit's constants are rounded (0.15273333 for 0.4581652 / 3), so the
    # identities hold to about 2e-5 (muxc) and 1e-4 (dmuxc, d2muxc)
    assert abs((n_p * fp[0] - n_m * fm[0]) / drhx - muxc) < 5e-5 * abs(muxc)
    assert abs((fp[1] - fm[1]) / drhx - dmuxc) < 2e-4 * abs(dmuxc)
    assert abs(dexc - (muxc - exc) / rhx) < 1e-12 * abs(dexc)
    # d2muxc = d dmuxc / d rho holds in the high-density branch; in the low
    # density one the reference's d2dec carries (dden*3) where the
    # derivative has dden**3, which the restatement keeps
    fd2 = (fp[4] - fm[4]) / drhx
    rho_au = rhx * P_ABOHR ** 3
    if rho_au >= 0.23873241:
        assert abs(fd2 - d2muxc) < 3e-4 * abs(d2muxc)
    else:
        assert abs(fd2 - d2muxc) > 1e-2 * abs(d2muxc)


def _system(fdata_root, name):
    path, nZ, st = workload(name, fdata_root, vxc=True)
    fd = orc.Fdata(path, nZ)
    return st, orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()


@pytest.fixture(scope="module", params=["si64", "sic_small", "cho_small"])
def vxc_case(request, fdata_root):
    st, s = _system(fdata_root, request.param)
    r3 = s.assemble_vxc(with3c=True, parts=True)
    r2 = s.assemble_vxc(with3c=False)
    return request.param, st, s, r3, r2


def _norb(s, st):
    return [s.fd.norb(int(k)) for k in st.imass]


def _nssh(st, name):
    # shells per species of the synthetic sets: Si, C, O sp; H s
    return [1 if (name == "cho_small" and k == 2) else 2 for k in st.imass]


def test_blocks_are_hermitian(vxc_case):
    name, st, s, r, _ = vxc_case
    norb, nsh = _norb(s, st), _nssh(st, name)
    for key in ("S", "rho_in", "rho_bond", "vxc"):
        x = r[key]
        worst = 0.0
        for i in range(len(st.imass)):
            for p in range(s.pair_off[i], s.pair_off[i + 1]):
                j = s.neigh_j[p]
                q = s.pair_off[j] + s.neigh_back[p]
                a = x[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
                b = x[s.blk_off[q]:s.blk_off[q + 1]].reshape(norb[i], norb[j]).T
                worst = max(worst, np.abs(a - b.T).max())
        assert worst < 1e-12 * max(1.0, np.abs(x).max()), key
    for key in ("wrho_in", "wrho_bond"):
        w = r[key]
        for i in range(len(st.imass)):
            for p in range(s.pair_off[i], s.pair_off[i + 1]):
                j = s.neigh_j[p]
                q = s.pair_off[j] + s.neigh_back[p]
                a = w[p][:nsh[i] * nsh[j]].reshape(nsh[j], nsh[i]).T
                b = w[q][:nsh[i] * nsh[j]].reshape(nsh[i], nsh[j]).T
                assert np.abs(a - b.T).max() < 1e-13
                assert np.all(w[p][nsh[i] * nsh[j]:] == 0.0)


def test_density_structure(vxc_case):
    """rho_bond equals rho_in off site without the three-center part; on the
    self block it holds only the atom's own term; the weighted densities
    are positive with the synthetic tables."""
    name, st, s, r3, r2 = vxc_case
    N = len(st.imass)
    self_p = s.pair_off[:-1] + s.neigh_self
    off = np.ones(s.npairs, bool)
    off[self_p] = False
    for p in np.nonzero(off)[0][:400]:
        sl = slice(s.blk_off[p], s.blk_off[p + 1])
        assert np.array_equal(r2["rho_in"][sl], r2["rho_bond"][sl])
        assert np.array_equal(r2["wrho_in"][p], r2["wrho_bond"][p])
        assert np.array_equal(r3["rho_bond"][sl], r2["rho_bond"][sl])
    assert np.all(r3["wrho_in"][:, 0] > 0.0)
    # the three-center part reaches the pairs with common neighbours
    assert np.abs(r3["rho_in"] - r2["rho_in"]).max() > 1e-6
    assert np.abs(r3["wrho_in"] - r2["wrho_in"]).max() > 1e-6
    # self block of rho_bond: only the self pair's atom term, so smaller
    for i in range(min(N, 8)):
        ps = self_p[i]
        assert r3["wrho_bond"][ps][0] < r3["wrho_in"][ps][0]


def test_vxc_is_the_sum_of_its_parts(vxc_case):
    _, _, _, r, _ = vxc_case
    assert np.array_equal(r["vxc"], r["vxc_bond"] + r["vxc_SN"] - r["vxc_SN_bond"])


def test_both_lda_branches_are_reached(fdata_root):
    """The on-site weighted densities of Si64 are above the density where
    the Ceperley-Alder fit changes form (rs = 1, 1.61 / A^3), the off-site
    ones below, so both branches feed the vxc blocks."""
    st, s = _system(fdata_root, "si64")
    r = s.assemble_vxc()
    w = r["wrho_in"]
    self_p = s.pair_off[:-1] + s.neigh_self
    rho_rs1 = 0.23873241 / P_ABOHR ** 3
    assert w[self_p, 0].max() > rho_rs1
    off = np.setdiff1d(np.arange(s.npairs), self_p)
    assert w[off, 0].max() < rho_rs1


def test_translation_invariance(fdata_root):
    path, nZ, st = workload("sic_small", fdata_root, vxc=True)
    fd = orc.Fdata(path, nZ)
    a = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors().assemble_vxc()
    b = orc.System(fd, st.ratom + np.array([0.31, -0.17, 0.05]), st.imass, st.lattice).neighbors().assemble_vxc()
    assert np.abs(a["vxc"] - b["vxc"]).max() < 1e-9


# ---------------------------------------------------------------------------
# force pass (Dassemble_vxc, k.DASSEMBLERS/M_Dassemble_vxc_McWEDA_Harris.f90
# and M_Dassemble_vxc_3c_McWEDA_Harris.f90)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def cluster(fdata_root):
    from conftest import symmetric_denmat
    from fbgpu import synth
    path, nZ, _ = workload("sic_small", fdata_root, vxc=True)
    st = synth.diamond((1, 1, 1), 4.36, 0.1, 41, sp_a=1, sp_b=2, name="SiC8cluster")
    fd = orc.Fdata(path, nZ)

    def at(r):
        return orc.System(fd, r, st.imass, st.lattice, icluster=1).neighbors()

    s = at(st.ratom)
    rho, _ = symmetric_denmat(s, [fd.norb(int(k)) for k in st.imass], 5)
    return st, at, s, rho


def _offsite_energy_gradient(st, at, s, rho, atoms):
    """-d/dR of sum over the off-site pairs of rho . vxc, by central
    differences (the same neighbor maps at every displacement)."""
    self_p = s.pair_off[:-1] + s.neigh_self
    mask = np.ones(s.nblock, bool)
    for p in self_p:
        mask[s.blk_off[p]:s.blk_off[p + 1]] = False

    def E(r):
        t = at(r)
        assert t.npairs == s.npairs
        v = t.assemble_vxc()["vxc"]
        return float(np.sum(rho[mask] * v[mask]))

    h = 1e-5
    out = np.zeros((len(atoms), 3))
    for n, k in enumerate(atoms):
        for c in range(3):
            rp, rm = st.ratom.copy(), st.ratom.copy()
            rp[k, c] += h
            rm[k, c] -= h
            out[n, c] = -(E(rp) - E(rm)) / (2 * h)
    return out


def _offsite_force(s, d, N):
    P = s.npairs
    off = d["vxc_off_site"].reshape(P, 3)
    F = np.zeros((N, 3))
    for i in range(N):
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            F[i] += off[p]
            F[s.neigh_j[p]] -= off[p]
    return F + (d["f3xca"] + d["f3xcb"] + d["f3xcc"]).reshape(N, 3)


def test_vxc_forces_are_gradients_with_exact_derivatives(cluster):
    """With the reference's two non-derivative forms replaced by exact ones
    (or_set_exact_derivatives), the off-site pair forces plus the
    three-center forces are minus the gradient of sum rho . vxc over the
    off-site blocks, to the 1e-4 the fit's rounded constants allow.  The
    on-site forces are not compared: the reference takes the shell-density
    derivative of the diagonal terms from the self pair's never-assembled
    Dblocko (zero) and reuses rho_in's for rho_bond's off-diagonal ones."""
    st, at, s, rho = cluster
    L = orc.lib()
    L.or_set_exact_derivatives(1)
    try:
        d = s.dassemble_vxc(rho)
        F = _offsite_force(s, d, len(st.imass))
        fd = _offsite_energy_gradient(st, at, s, rho, [0, 1, 5])
    finally:
        L.or_set_exact_derivatives(0)
    an = F[[0, 1, 5]]
    assert np.all(np.abs(fd - an) <= 1e-3 + 1e-3 * np.abs(an))
    assert np.abs(an).max() > 0.5


def test_reference_forms_are_kept(cluster):
    """With the reference's forms the same comparison is off by percents:
    the restatement keeps them (d2muxc of the low-density branch enters the
    shell-density terms, the linear 3c branch the three-center ones)."""
    st, at, s, rho = cluster
    d = s.dassemble_vxc(rho)
    F = _offsite_force(s, d, len(st.imass))
    fd = _offsite_energy_gradient(st, at, s, rho, [0])
    assert np.abs(fd - F[[0]]).max() > 1e-2


def test_vxc_forces_conserve_momentum(cluster):
    st, at, s, rho = cluster
    d = s.dassemble_vxc(rho)
    assert np.abs(d["ftot_add"].reshape(-1, 3).sum(0)).max() < 1e-11


@pytest.mark.parametrize("kind", ["atom", "dimer", "isolated"])
def test_sparse_clusters(fdata_root, kind):
    """Ragged lists under McWEDA: a lone Si atom (its self pair only: the
    density and vxc come from the atom term and vxc_1c), a Si dimer, and a
    Si8 cluster with one atom far away.  Blocks finite and Hermitian, the
    lone atom's density block the same with and without three-center terms,
    and the vxc forces summing to zero."""
    from conftest import symmetric_denmat
    from fbgpu import synth
    path, nZ, _ = workload("sic_small", fdata_root, vxc=True)
    if kind == "atom":
        r = np.zeros((1, 3))
    elif kind == "dimer":
        r = np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 2.3]])
    else:
        r = np.vstack([synth.diamond((1, 1, 1), 5.43, 0.1, 21).ratom, [[30.0, 30.0, 30.0]]])
    imass = np.ones(len(r), np.int32)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, r, imass, 20.0 * np.eye(3), icluster=1).neighbors()
    v3 = s.assemble_vxc()
    v2 = s.assemble_vxc(with3c=False)
    norb = [fd.norb(1)] * len(r)
    for key in ("rho_in", "rho_bond", "vxc"):
        x = v3[key]
        assert np.all(np.isfinite(x)), key
        for i in range(len(r)):
            for p in range(s.pair_off[i], s.pair_off[i + 1]):
                j = s.neigh_j[p]
                q = s.pair_off[j] + s.neigh_back[p]
                a = x[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
                b = x[s.blk_off[q]:s.blk_off[q + 1]].reshape(norb[i], norb[j]).T
                assert np.abs(a - b.T).max() < 1e-12 * max(1.0, np.abs(x).max()), key
    if kind in ("atom", "dimer"):  # no triplets: the three-center terms add nothing
        assert s.ntrip == 0
        for key in ("rho_in", "vxc"):
            assert np.array_equal(v3[key], v2[key]), key
    rho, _ = symmetric_denmat(s, norb, 5)
    d = s.dassemble_vxc(rho)
    f = d["ftot_add"].reshape(-1, 3)
    assert np.all(np.isfinite(f))
    assert np.abs(f.sum(0)).max() < 1e-11 * max(1.0, np.abs(f).max())
