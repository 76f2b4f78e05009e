"""Property tests of the oracle's pointwise routines (CPU only).

The reference ships no golden data, so the restatement is checked against
mathematics: the 7-point Lagrange and the 16-point bicubic interpolators
reproduce polynomials of their degree exactly, every derivative routine
agrees with finite differences, and the local frames are orthonormal.
"""
import os
import shutil

import numpy as np
import pytest

from fbgpu import synth
from oracle import oracle as orc

P_OVERLAP = 1


@pytest.fixture(scope="module")
def si_fdata(tmp_path_factory):
    path = str(tmp_path_factory.mktemp("fdata_si"))
    synth.write_fdata(path, [synth.si(5.0)])
    return path


def _poly_fdata(src, dst):
    """Copy an Fdata set and replace the Si-Si overlap table by degree-6
    polynomials and the bcna tables by bicubic polynomials."""
    shutil.copytree(src, dst)
    xmax = 2 * 5.0 * 0.529177
    x = np.linspace(0.0, xmax, 200)
    coef = np.random.default_rng(3).normal(size=(6, 7))
    data = np.stack([np.polyval(c, x / xmax) for c in coef], axis=1)
    with open(os.path.join(dst, "overlap.14.14.dat"), "w") as f:
        for row in data:
            f.write(" ".join("%24.16E" % v for v in row) + "\n")
    n = 31
    u = np.linspace(0.0, 1.0, n)
    rng = np.random.default_rng(5)
    cubic = {}
    for th in range(1, 6):
        cx = rng.normal(size=(10, 4))
        cy = rng.normal(size=(10, 4))
        cubic[th] = (cx, cy)
        with open(os.path.join(dst, "bcna_%02d_00.14.14.14.dat" % th), "w") as f:
            for iy in range(n):
                for ix in range(n):
                    # large linear terms keep the gradient switch on the bicubic branch
                    vals = [np.polyval(cx[e], u[ix]) * np.polyval(cy[e], u[iy]) + 3.0 * u[ix] + 2.0 * u[iy]
                            for e in range(10)]
                    f.write(" ".join("%24.16E" % v for v in vals) + "\n")
    return coef, cubic, xmax


def test_lagrange_exact_on_degree6(si_fdata, tmp_path):
    coef, cubic, xmax = _poly_fdata(si_fdata, str(tmp_path / "poly"))
    fd = orc.Fdata(str(tmp_path / "poly"), [14])
    mu, nu, _ = synth.make_munu([0, 1], [0, 1])
    for x in np.random.default_rng(1).uniform(0.0, xmax, 50):
        h = orc.getMEs_2c(fd, 1, 1, P_OVERLAP, x, 4, 4)
        for e in range(6):
            want = np.polyval(coef[e], x / xmax)
            assert abs(h[mu[e] - 1, nu[e] - 1] - want) < 1e-10 * max(1.0, abs(want))


def test_bicubic_exact_on_bicubic(si_fdata, tmp_path):
    coef, cubic, xmax = _poly_fdata(si_fdata, str(tmp_path / "poly"))
    fd = orc.Fdata(str(tmp_path / "poly"), [14])
    mu, nu, mv = synth.make_munu_3c([0, 1], [0, 1])
    X = 10.0 * 0.529177  # both axes span 10 bohr
    rng = np.random.default_rng(2)
    for _ in range(40):
        x, y, c = rng.uniform(0.05 * X, 0.95 * X), rng.uniform(0.05 * X, 0.95 * X), rng.uniform(-0.95, 0.95)
        h = orc.getMEs_3c(fd, 1, 1, 1, x, y, c, 4, 4)
        P = [1.0, c, 0.5 * (3 * c * c - 1), 0.5 * c * (5 * c * c - 3), 0.125 * (3 - c * c * (30 - 35 * c * c))]
        s = np.sqrt(max(1e-5, 1 - c * c))
        for e in range(10):
            want = sum(P[th - 1] * (np.polyval(cubic[th][0][e], x / X) * np.polyval(cubic[th][1][e], y / X)
                                    + 3.0 * x / X + 2.0 * y / X) for th in range(1, 6))
            if mv[e] == 1:
                want *= s
            assert abs(h[mu[e] - 1, nu[e] - 1] - want) < 1e-9 * max(1.0, abs(want))


def test_getDMEs_2c_matches_finite_difference(si_fdata):
    fd = orc.Fdata(si_fdata, [14])
    for it in (1, 2, 3, 4, 5):
        for x in (0.7, 1.9, 2.35, 4.1, 5.2):
            hv, d = orc.getDMEs_2c(fd, 1, 1, it, x, 4, 4)
            hp = orc.getMEs_2c(fd, 1, 1, it, x + 1e-5, 4, 4)
            hm = orc.getMEs_2c(fd, 1, 1, it, x - 1e-5, 4, 4)
            assert np.allclose(hv, orc.getMEs_2c(fd, 1, 1, it, x, 4, 4), atol=1e-13)
            assert np.allclose(d, (hp - hm) / 2e-5, atol=1e-6, rtol=1e-6)


def test_getDMEs_2c_small_x_returns_table_origin(si_fdata):
    fd = orc.Fdata(si_fdata, [14])
    h, d = orc.getDMEs_2c(fd, 1, 1, 1, 0.0, 4, 4)
    assert np.all(d == 0.0)
    h0 = orc.getMEs_2c(fd, 1, 1, 1, 0.0, 4, 4)
    assert np.allclose(h, h0, atol=1e-12)


def test_getDMEs_3c_matches_finite_difference(si_fdata):
    fd = orc.Fdata(si_fdata, [14])
    rng = np.random.default_rng(4)
    checked = 0
    for _ in range(60):
        x, y, c = rng.uniform(0.3, 4.5), rng.uniform(1.0, 4.8), rng.uniform(-0.9, 0.9)
        h, dp, dx, dy = orc.getDMEs_3c(fd, 1, 1, 1, x, y, c, 4, 4)
        e = 1e-6
        # stay inside one grid cell so the interpolation branch is fixed
        dxg = 10 * 0.529177 / 30
        if min(x / dxg % 1, 1 - x / dxg % 1, y / dxg % 1, 1 - y / dxg % 1) < 1e-3:
            continue
        fx = (orc.getMEs_3c(fd, 1, 1, 1, x + e, y, c, 4, 4) - orc.getMEs_3c(fd, 1, 1, 1, x - e, y, c, 4, 4)) / (2 * e)
        fy = (orc.getMEs_3c(fd, 1, 1, 1, x, y + e, c, 4, 4) - orc.getMEs_3c(fd, 1, 1, 1, x, y - e, c, 4, 4)) / (2 * e)
        fc = (orc.getMEs_3c(fd, 1, 1, 1, x, y, c + e, 4, 4) - orc.getMEs_3c(fd, 1, 1, 1, x, y, c - e, 4, 4)) / (2 * e)
        assert np.allclose(h, orc.getMEs_3c(fd, 1, 1, 1, x, y, c, 4, 4), atol=1e-13)
        assert np.allclose(dp, fc, atol=2e-6)
        lin = np.abs(dx - fx).max() > 1e-4  # the linear branch uses one scalar gradient for all MEs
        if not lin:
            assert np.allclose(dx, fx, atol=2e-6)
            assert np.allclose(dy, fy, atol=2e-6)
        checked += 1
    assert checked > 30


def test_epsilon_orthonormal_right_handed():
    rng = np.random.default_rng(7)
    for _ in range(100):
        r1, r2 = rng.normal(size=3), rng.normal(size=3)
        e = orc.epsilon(r1, r2)
        assert np.allclose(e.T @ e, np.eye(3), atol=1e-13)
        assert np.isclose(np.linalg.det(e), 1.0)
        assert np.allclose(e[:, 2], r2 / np.linalg.norm(r2))
    # colinear fallback and zero r2 (identity)
    assert np.allclose(orc.epsilon(np.array([0, 0, 1.0]), np.array([0, 0, 2.0])).T @
                       orc.epsilon(np.array([0, 0, 1.0]), np.array([0, 0, 2.0])), np.eye(3))
    assert np.allclose(orc.epsilon(np.ones(3), np.zeros(3)), np.eye(3))


def _eps2c(r1, r2):
    z = np.linalg.norm(r2 - r1)
    return orc.epsilon(r2, (r2 - r1) / z)


def test_depsilon_2c_matches_finite_difference():
    lib = orc.lib()
    rng = np.random.default_rng(8)
    for _ in range(20):
        r1, r2 = rng.normal(size=3) * 2, rng.normal(size=3) * 2 + 3
        z = np.linalg.norm(r2 - r1)
        e = _eps2c(r1, r2)
        d = np.zeros(27)
        lib.or_depsilon_2c(r1, r2, z, np.ascontiguousarray(e.T.ravel()), d)
        d = d.reshape(3, 3, 3).transpose(2, 1, 0)  # deps(ix, imu, k)
        for ix in range(3):
            h = np.zeros(3)
            h[ix] = 1e-6
            fd = (_eps2c(r1 + h, r2) - _eps2c(r1 - h, r2)) / 2e-6
            assert np.allclose(d[ix], fd, atol=1e-6)


def _eps3c(r1, r2, ra):
    r21 = r2 - r1
    sig = r21 / np.linalg.norm(r21)
    rn = ra - (r1 + r21 / 2)
    return orc.epsilon(rn / np.linalg.norm(rn), sig)


def test_depsilon_3c_matches_finite_difference():
    lib = orc.lib()
    rng = np.random.default_rng(9)
    for _ in range(20):
        r1, r2, ra = rng.normal(size=3) * 2, rng.normal(size=3) * 2 + 2, rng.normal(size=3) * 2 - 1
        r21 = r2 - r1
        z = np.linalg.norm(r21)
        rn = ra - (r1 + r21 / 2)
        e = _eps3c(r1, r2, ra)
        dA, dB = np.zeros(27), np.zeros(27)
        lib.or_depsilon_3c(r1, r2, r21, z, ra, rn, np.ascontiguousarray(e.T.ravel()), dA, dB)
        dA = dA.reshape(3, 3, 3).transpose(2, 1, 0)
        dB = dB.reshape(3, 3, 3).transpose(2, 1, 0)
        for ix in range(3):
            h = np.zeros(3)
            h[ix] = 1e-6
            fa = (_eps3c(r1, r2, ra + h) - _eps3c(r1, r2, ra - h)) / 2e-6
            fb = (_eps3c(r1 + h, r2, ra) - _eps3c(r1 - h, r2, ra)) / 2e-6
            assert np.allclose(dA[ix], fa, atol=1e-6)
            assert np.allclose(dB[ix], fb, atol=1e-6)


def test_rotate_is_L_M_Rt(si_fdata):
    fd = orc.Fdata(si_fdata, [14])
    rng = np.random.default_rng(10)
    for _ in range(20):
        e = orc.epsilon(rng.normal(size=3), rng.normal(size=3))
        M = rng.normal(size=(4, 4))
        X = orc.rotate(fd, 1, 1, e, M)
        perm = [1, 2, 0]
        P = e[np.ix_(perm, perm)]
        L = np.eye(4)
        L[1:, 1:] = P
        assert np.allclose(X, L @ M @ L.T, atol=1e-13)


def test_rotation_reproduces_slater_koster_table(si_fdata):
    """Known answer: the rotation of the molecular-frame sigma / pi elements
    into the crystal frame, in the frame the 2c assemblers build
    (epsilon(r2, sighat), M_assemble_2c_Harris.f90:177), gives the s, p
    entries of the Slater-Koster table (Phys. Rev. 94, 1498 (1954), Table I)
    for the bond direction cosines (l, m, n).  Orbital order s, py, pz, px."""
    fd = orc.Fdata(si_fdata, [14])
    rng = np.random.default_rng(21)
    for _ in range(20):
        r1, r2 = rng.normal(size=3) * 2.0, rng.normal(size=3) * 2.0
        d = r2 - r1
        l, m, n = d / np.linalg.norm(d)
        e = orc.epsilon(r2, d / np.linalg.norm(d))
        ss, sp, ps, pps, ppp = rng.normal(size=5)
        M = np.zeros((4, 4))
        M[0, 0], M[0, 2], M[2, 0] = ss, sp, ps
        M[1, 1], M[2, 2], M[3, 3] = ppp, pps, ppp
        X = orc.rotate(fd, 1, 1, e, M)
        c = {1: m, 2: n, 3: l}   # the direction cosine of each p orbital
        want = np.zeros((4, 4))
        want[0, 0] = ss
        for a in (1, 2, 3):
            want[0, a] = c[a] * sp
            want[a, 0] = c[a] * ps
            for b in (1, 2, 3):
                want[a, b] = c[a] * c[b] * (pps - ppp) + (ppp if a == b else 0.0)
        assert np.abs(X - want).max() < 1e-13


def test_d_rotation_reproduces_slater_koster_sigma_entries(tmp_path):
    """The same known answer for d orbitals (order xy, yz, 3z^2 - r^2, xz,
    x^2 - y^2): a molecular-frame s-d sigma element gives the Table I
    entries sqrt(3) lm, sqrt(3) mn, n^2 - (l^2 + m^2)/2, sqrt(3) ln,
    sqrt(3)/2 (l^2 - m^2) times V_sd sigma, and a p-d sigma element the same
    factors times the direction cosine of the p orbital."""
    path = str(tmp_path / "fdata_ti")
    synth.write_fdata(path, [synth.ti()])
    fd = orc.Fdata(path, [22])
    rng = np.random.default_rng(22)
    s3 = np.sqrt(3.0)
    for _ in range(10):
        r1, r2 = rng.normal(size=3) * 2.0, rng.normal(size=3) * 2.0
        d = r2 - r1
        l, m, n = d / np.linalg.norm(d)
        e = orc.epsilon(r2, d / np.linalg.norm(d))
        sd, pd = rng.normal(size=2)
        M = np.zeros((9, 9))
        M[0, 6] = sd          # <s | d_z2>
        M[2, 6] = pd          # <p_z | d_z2>
        X = orc.rotate(fd, 1, 1, e, M)
        f = np.array([s3 * l * m, s3 * m * n, n * n - 0.5 * (l * l + m * m), s3 * l * n, 0.5 * s3 * (l * l - m * m)])
        assert np.abs(X[0, 4:9] - sd * f).max() < 1e-13
        for a, ca in ((1, m), (2, n), (3, l)):
            assert np.abs(X[a, 4:9] - pd * ca * f).max() < 1e-13


def test_x_beyond_table_is_an_error(si_fdata):
    fd = orc.Fdata(si_fdata, [14])
    with pytest.raises(orc.OracleError) as ei:
        orc.getMEs_2c(fd, 1, 1, 1, 6.0, 4, 4)
    assert ei.value.code == 5


def test_missing_fdata_file_is_an_error(si_fdata, tmp_path):
    dst = str(tmp_path / "broken")
    shutil.copytree(si_fdata, dst)
    os.remove(os.path.join(dst, "3c.14.14.14.dir"))
    with pytest.raises(orc.OracleError) as ei:
        orc.Fdata(dst, [14])
    assert ei.value.code == 2
