"""System-level property tests of the oracle (CPU only): neighbor maps
against a numpy brute force in the reference order, Hermiticity of the
assembled blocks, forces against finite differences of the band energy,
invariance under rigid motions, and the reference's error stops."""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from fbgpu import synth
from oracle import oracle as orc


def _system(name, root, threads=1, st=None):
    path, nZ, st0 = workload(name, root)
    st = st or st0
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, threads=threads).neighbors()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    return fd, s, st, norb


def _xl(lattice):
    out = [np.zeros(3)]
    for iz in range(-4, 5):
        for iy in range(-4, 5):
            for ix in range(-4, 5):
                if ix or iy or iz:
                    out.append(ix * lattice[0] + iy * lattice[1] + iz * lattice[2])
    return np.array(out)


@pytest.mark.parametrize("name", ["si64", "cho_small", "sic_vac"])
def test_neighbors_match_brute_force(fdata_root, name):
    fd, s, st, norb = _system(name, fdata_root)
    xl = _xl(st.lattice)
    path, nZ, _ = workload(name, fdata_root)
    sp = synth.species_for({"si64": "si64", "cho_small": "cho1536", "sic_vac": "sic4096"}[name])
    rc = np.array([max(r * 0.529177 for r in x.rcutoff) for x in sp])[st.imass - 1]
    N = st.natoms
    for i in range(N):
        want = []
        for mb in range(len(xl)):
            d = np.linalg.norm(st.ratom + xl[mb] - st.ratom[i], axis=1)
            for j in np.nonzero(d < rc[i] + rc - 0.01)[0]:
                want.append((j, mb))
        got = list(zip(s.neigh_j[s.pair_off[i]:s.pair_off[i + 1]], s.neigh_b[s.pair_off[i]:s.pair_off[i + 1]]))
        assert got == want
    # neigh_self and neigh_back
    for i in range(N):
        p = s.pair_off[i] + s.neigh_self[i]
        assert s.neigh_j[p] == i and s.neigh_b[p] == 0
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            j, q = s.neigh_j[p], s.pair_off[s.neigh_j[p]] + s.neigh_back[p]
            assert s.neigh_j[q] == i
            assert np.allclose(xl[s.neigh_b[p]] + xl[s.neigh_b[q]], 0.0, atol=1e-9)


def _rc(name, st):
    sp = synth.species_for(name)
    return np.array([max(r * 0.529177 for r in x.rcutoff) for x in sp])[st.imass - 1]


def _common_brute(s, st, xl, rc):
    """find_common_neighbors (c.SYSTEM/M_neighbors.f90:548-812) as plain
    loops: for each ialpha, ineigh then jneigh over its non-self neighbors,
    i != j index, kept when |r1 - r2| < rc_i + rc_j - 0.01 and j is found in
    i's list by the vector match (first kneigh, 1e-4 per component)."""
    out = []
    for a in range(st.natoms):
        p0, p1 = s.pair_off[a], s.pair_off[a + 1]
        pself = p0 + s.neigh_self[a]
        for pi in range(p0, p1):
            if pi == pself:
                continue
            i, ib = s.neigh_j[pi], s.neigh_b[pi]
            r1 = st.ratom[i] + xl[ib]
            q0, q1 = s.pair_off[i], s.pair_off[i + 1]
            r3 = st.ratom[s.neigh_j[q0:q1]] + xl[s.neigh_b[q0:q1]] - st.ratom[i]
            for pj in range(p0, p1):
                if pj == pself or pj == pi:
                    continue
                j, jb = s.neigh_j[pj], s.neigh_b[pj]
                r2 = st.ratom[j] + xl[jb]
                if not np.linalg.norm(r2 - r1) < rc[i] + rc[j] - 0.01:
                    continue
                hit = np.nonzero(np.all(np.abs(r3 - r2 + r1) < 1e-4, axis=1))[0]
                if len(hit):
                    out.append((a, i, ib, j, jb, int(hit[0])))
    return out


def _common_got(s):
    return [(a, s.ci_j[t], s.ci_b[t], s.cj_j[t], s.cj_b[t], s.cneigh[t])
            for a in range(len(s.trip_off) - 1) for t in range(s.trip_off[a], s.trip_off[a + 1])]


@pytest.mark.parametrize("name", ["si_vac", "sic_vac"])
def test_common_neighbors_match_brute_force(fdata_root, name):
    """Every triplet of the reference loops, in their order, and no other."""
    fd, s, st, norb = _system(name, fdata_root)
    rc = _rc({"si_vac": "si64", "sic_vac": "sic4096"}[name], st)
    want = _common_brute(s, st, _xl(st.lattice), rc)
    assert s.ntrip == len(want) > 0
    assert _common_got(s) == want


def _cluster(ratom):
    ratom = np.asarray(ratom, float)
    return synth.Structure(ratom=ratom, imass=np.ones(len(ratom), np.int32), lattice=20.0 * np.eye(3),
                           icluster=1, name="cluster")


@pytest.mark.parametrize("kind", ["atom", "dimer", "isolated"])
def test_sparse_clusters(fdata_root, kind):
    """Ragged neighbor lists: one atom (only its self pair, no triplets), a
    dimer (rows without a partner, no triplets) and a cluster with one atom
    far from the rest (a self-only list among full ones).  Neighbors and
    triplets as the brute force gives them; blocks Hermitian; the total
    force on the cluster vanishes (zero on a lone atom)."""
    path, nZ, base = workload("sic_vac", fdata_root)
    if kind == "atom":
        st = _cluster([[0.0, 0.0, 0.0]])
    elif kind == "dimer":
        st = _cluster([[0.0, 0.0, 0.0], [0.3, -0.2, 2.3]])
    else:
        si8 = synth.diamond((1, 1, 1), 5.43, 0.1, 21, name="Si8")
        st = _cluster(np.vstack([si8.ratom, [[30.0, 30.0, 30.0]]]))
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice, icluster=1).neighbors()
    rc = _rc("sic4096", st)
    xl = np.zeros((1, 3))
    N = st.natoms
    for i in range(N):
        d = np.linalg.norm(st.ratom - st.ratom[i], axis=1)
        want = [(j, 0) for j in np.nonzero(d < rc[i] + rc - 0.01)[0]]
        got = list(zip(s.neigh_j[s.pair_off[i]:s.pair_off[i + 1]], s.neigh_b[s.pair_off[i]:s.pair_off[i + 1]]))
        assert got == want
    assert _common_got(s) == _common_brute(s, st, xl, rc)
    if kind == "atom":
        assert (s.npairs, s.ntrip) == (1, 0)
    elif kind == "dimer":
        assert (s.npairs, s.ntrip) == (4, 0)
    else:
        assert np.diff(s.pair_off)[-1] == 1 and s.ntrip > 0
    S, T, vb, vbo = s.assemble()
    assert np.all(np.isfinite(S)) and np.all(np.isfinite(T + vb + vbo))
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    for i in range(N):
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            j = s.neigh_j[p]
            q = s.pair_off[j] + s.neigh_back[p]
            a = S[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
            b = S[s.blk_off[q]:s.blk_off[q + 1]].reshape(norb[i], norb[j]).T
            assert np.abs(a - b.T).max() < 1e-13
    rho, cape = symmetric_denmat(s, norb, 3)
    f = s.dassemble(rho, cape)["ftot"].reshape(N, 3)
    assert np.all(np.isfinite(f))
    if kind == "atom":
        assert np.abs(f).max() < 1e-12
    else:
        assert np.abs(f.sum(axis=0)).max() < 1e-9 * max(1.0, np.abs(f).max())


def test_common_neighbors_are_pairs_within_cutoff(fdata_root):
    fd, s, st, norb = _system("si64", fdata_root)
    xl = _xl(st.lattice)
    for a in range(st.natoms):
        for t in range(s.trip_off[a], s.trip_off[a + 1]):
            i, j = s.ci_j[t], s.cj_j[t]
            r1 = st.ratom[i] + xl[s.ci_b[t]]
            r2 = st.ratom[j] + xl[s.cj_b[t]]
            q = s.pair_off[i] + s.cneigh[t]
            assert s.neigh_j[q] == j
            assert np.allclose(st.ratom[j] + xl[s.neigh_b[q]] - st.ratom[i], r2 - r1, atol=1e-9)


@pytest.mark.parametrize("name", ["si64", "cho_small", "sic_small"])
def test_blocks_hermitian(fdata_root, name):
    fd, s, st, norb = _system(name, fdata_root)
    S, T, vb, vbo = s.assemble()
    H = T + vb + vbo
    for B, tol in ((S, 1e-13), (T, 1e-12), (H, 1e-11)):
        for i in range(st.natoms):
            for p in range(s.pair_off[i], s.pair_off[i + 1]):
                j = s.neigh_j[p]
                q = s.pair_off[j] + s.neigh_back[p]
                a = B[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
                b = B[s.blk_off[q]:s.blk_off[q + 1]].reshape(norb[i], norb[j]).T
                assert np.abs(a - b.T).max() < tol


def _band_energy(fd, st, ratom, rho, cape, layout):
    s = orc.System(fd, ratom, st.imass, st.lattice).neighbors()
    assert s.npairs == layout.npairs and np.array_equal(s.neigh_j[:s.npairs], layout.neigh_j[:s.npairs])
    S, T, vb, vbo = s.assemble()
    return float(rho @ (T + vb + vbo) - cape @ S)


@pytest.mark.parametrize("name", ["si_vac", "cho_small"])
def test_forces_are_minus_gradient_of_band_energy(fdata_root, name):
    """ftot = -dE/dR for E = sum rho.(T + vna + vnao) - sum cape.S at fixed
    density matrices: checks the whole derivative chain of the oracle."""
    fd, s, st, norb = _system(name, fdata_root)
    rho, cape = symmetric_denmat(s, norb, 11)
    f = s.dassemble(rho, cape)["ftot"].reshape(-1, 3)
    h = 1e-5
    rng = np.random.default_rng(3)
    for i in rng.choice(st.natoms, 4, replace=False):
        for k in range(3):
            rp, rm = st.ratom.copy(), st.ratom.copy()
            rp[i, k] += h
            rm[i, k] -= h
            g = (_band_energy(fd, st, rp, rho, cape, s) - _band_energy(fd, st, rm, rho, cape, s)) / (2 * h)
            assert abs(-g - f[i, k]) < 1e-5 * max(1.0, abs(g)), (i, k, -g, f[i, k])


def test_rigid_motion_invariance(fdata_root):
    fd, s, st, norb = _system("si64", fdata_root)
    S, T, vb, vbo = s.assemble()
    Q, _ = np.linalg.qr(np.random.default_rng(5).normal(size=(3, 3)))
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    st2 = synth.Structure(st.ratom @ Q.T + np.array([0.3, -1.1, 2.0]), st.imass, st.lattice @ Q.T)
    s2 = orc.System(fd, st2.ratom, st2.imass, st2.lattice).neighbors()
    assert np.array_equal(s.neigh_j, s2.neigh_j) and np.array_equal(s.neigh_b, s2.neigh_b)
    S2, T2, vb2, vbo2 = s2.assemble()
    for A, B in ((S, S2), (T, T2), (vb, vb2), (vbo, vbo2)):
        for p in range(s.npairs):
            a = A[s.blk_off[p]:s.blk_off[p + 1]]
            b = B[s.blk_off[p]:s.blk_off[p + 1]]
            assert abs(np.linalg.norm(a) - np.linalg.norm(b)) < 1e-10 * max(1.0, np.linalg.norm(a))


def test_atoms_too_close_is_an_error(fdata_root):
    path, nZ, st = workload("si64", fdata_root)
    r = st.ratom.copy()
    r[1] = r[0] + np.array([0.3, 0.0, 0.0])
    fd = orc.Fdata(path, nZ)
    with pytest.raises(orc.OracleError) as ei:
        orc.System(fd, r, st.imass, st.lattice).neighbors()
    assert ei.value.code == 6


def test_parallel_oracle_matches_serial(fdata_root):
    fd, s1, st, norb = _system("cho_small", fdata_root, threads=1)
    _, s4, _, _ = _system("cho_small", fdata_root, threads=4)
    assert np.array_equal(s1.neigh_j, s4.neigh_j) and np.array_equal(s1.cneigh, s4.cneigh)
    a1, a4 = s1.assemble(), s4.assemble()
    for x, y in zip(a1, a4):
        assert np.abs(x - y).max() < 1e-12
    rho, cape = symmetric_denmat(s1, norb, 5)
    f1 = s1.dassemble(rho, cape)["ftot"]
    f4 = s4.dassemble(rho, cape)["ftot"]
    assert np.abs(f1 - f4).max() < 1e-11


def test_cluster_forces_are_minus_gradient(fdata_root):
    """The same derivative check on a cluster (icluster = 1: no images),
    placed off the origin, with one isolated atom: ftot = -dE/dR."""
    path, nZ, _ = workload("sic_vac", fdata_root)
    fd = orc.Fdata(path, nZ)
    r = np.vstack([synth.diamond((1, 1, 1), 5.43, 0.1, 21).ratom, [[30.0, 30.0, 30.0]]]) + [1.1, 0.7, -0.4]
    imass = np.ones(len(r), np.int32)
    lat = 20.0 * np.eye(3)
    s = orc.System(fd, r, imass, lat, icluster=1).neighbors()
    norb = np.array([fd.norb(1)] * len(r))
    rho, cape = symmetric_denmat(s, norb, 12)
    f = s.dassemble(rho, cape)["ftot"].reshape(-1, 3)
    assert np.abs(f[-1]).max() == 0.0  # the isolated atom feels nothing

    def energy(x):
        t = orc.System(fd, x, imass, lat, icluster=1).neighbors()
        assert t.npairs == s.npairs and t.ntrip == s.ntrip
        S, T, vb, vbo = t.assemble()
        return float(rho @ (T + vb + vbo) - cape @ S)

    h = 1e-5
    for i in (0, 3, 6):
        for k in range(3):
            rp, rm = r.copy(), r.copy()
            rp[i, k] += h
            rm[i, k] -= h
            g = (energy(rp) - energy(rm)) / (2 * h)
            assert abs(-g - f[i, k]) < 1e-5 * max(1.0, abs(g)), (i, k, -g, f[i, k])


def test_synthetic_denmat_symmetric_across_neigh_back(fdata_root):
    """The vectorised density-matrix generator the benchmark and the
    full-size tests use: rho_ij(mu, nu) = rho_ji(nu, mu) for every pair of
    mixed-size blocks, self blocks symmetric."""
    fd, s, st, norb = _system("cho_small", fdata_root)
    rho, cape = synth.symmetric_denmat(np.diff(s.pair_off), s.neigh_j[:s.npairs], s.neigh_back[:s.npairs],
                                       s.blk_off, norb, seed=3)
    for i in range(len(norb)):
        for p in range(s.pair_off[i], s.pair_off[i + 1]):
            j = s.neigh_j[p]
            q = s.pair_off[j] + s.neigh_back[p]
            for m in (rho, cape):
                a = m[s.blk_off[p]:s.blk_off[p + 1]].reshape(norb[j], norb[i]).T
                b = m[s.blk_off[q]:s.blk_off[q + 1]].reshape(norb[i], norb[j]).T
                assert np.array_equal(a, b.T)
