"""The three-center force kernels contract the frame derivative of the
rotation with the density through the rotation rates of the frame instead of
Dtwister's dL (M_Drotations.f90:456-471) and Depsilon_3c's full derivative
(b.FUNCTIONS/Depsilon_3c.f90:49-189).  This checks that identity on the
oracle's epsilon and Depsilon_3c: for X = L M L^T,

    sum rho (dL M L^T + L M dL^T) = sum_ij Omega_ij kappa_ij,
    Omega = L^T dL,  kappa_ij = sum_e M_e ([a = p_j] G(p_i, b) + [b = p_j] G(a, p_i)),

with the rates in the closed forms the kernels use (frame_rates_3c,
frame_extra_3c), for the standard frame and for epsilon's collinear fallback
frame.  The numpy here restates the kernels' formulas; the literal side is
the oracle's Depsilon_3c."""
import numpy as np
import pytest

from oracle import oracle as O

PPERM = [1, 2, 0]          # p order (y, z, x): orbital slot -> frame axis
P_OF_AXIS = {0: 3, 1: 1, 2: 2}  # frame axis x, y, z -> orbital of an s+p block
# ME positions of an sp x sp three-center block (make_munu_3c)
ME = [(0, 0), (0, 2), (2, 0), (2, 2), (3, 3), (1, 1), (0, 3), (3, 0), (3, 2), (2, 3)]


def _frame(r1, r2, ratm):
    r21 = r2 - r1
    z = np.linalg.norm(r21)
    sig = r21 / z
    rnabc = ratm - (r1 + 0.5 * r21)
    x = np.linalg.norm(rnabc)
    rhat = rnabc / x
    e = O.epsilon(rhat, sig)  # e[imu][k]: component imu of frame axis k
    dA, dB = np.zeros(27), np.zeros(27)
    O.lib().or_depsilon_3c(np.ascontiguousarray(r1), np.ascontiguousarray(r2), np.ascontiguousarray(r21), float(z),
                           np.ascontiguousarray(ratm), np.ascontiguousarray(rnabc),
                           np.ascontiguousarray(e.T.ravel()), dA, dB)
    dA = dA.reshape(3, 3, 3, order="F")  # [ix][imu][k]
    dB = dB.reshape(3, 3, 3, order="F")
    ypm = np.linalg.norm(np.cross(sig, rhat))
    return e, dA, dB, r21, z, rnabc, ypm >= 1.0e-4


def _L(e):
    L = np.zeros((4, 4))
    L[0, 0] = 1.0
    for a in range(3):
        for b in range(3):
            L[1 + a, 1 + b] = e[PPERM[a], PPERM[b]]
    return L


def _literal(e, d, M, rho):
    L = _L(e)
    out = np.zeros(3)
    for c in range(3):
        dL = np.zeros((4, 4))
        for a in range(3):
            for b in range(3):
                dL[1 + a, 1 + b] = d[c, PPERM[a], PPERM[b]]
        out[c] = np.sum(rho * (dL @ M @ L.T + L @ M @ dL.T))
    return out


def _kappa(G, M, i, j):
    Pi, Pj = P_OF_AXIS[i], P_OF_AXIS[j]
    return sum(M[a, b] * ((a == Pj) * G[Pi, b] + (b == Pj) * G[a, Pi]) for a, b in ME)


def _rates(e, r1, r2, ratm, r21, z, rnabc, std, M, rho):
    L = _L(e)
    G = L.T @ rho @ L
    tau = [_kappa(G, M, 0, 1) - _kappa(G, M, 1, 0), _kappa(G, M, 1, 2) - _kappa(G, M, 2, 1),
           _kappa(G, M, 0, 2) - _kappa(G, M, 2, 0)]
    cm = np.linalg.norm(np.cross(r21, rnabc))
    if cm < 1.0e-3:
        return np.zeros(3), np.zeros(3)
    ic, iz = 1.0 / cm, 1.0 / z
    ex, ey, ez = e[:, 0], e[:, 1], e[:, 2]
    byz = -iz * ey
    hA = ic * np.cross(ex, r21) * tau[0]
    hB = ic * np.cross(ex, ratm - r2) * tau[0] + byz * tau[1] - iz * ex * tau[2]
    if not std:
        r1m2, r2m2, ram2 = r1 @ r1, r2 @ r2, ratm @ ratm
        r12, r2a, r1a = r1 @ r2, r2 @ ratm, r1 @ ratm
        A1, A2, A3 = r1m2 + r2m2 - 2 * r12, r12 - r1m2 - r2a + r1a, r12 - r2m2 + r2a - r1a
        B1, B2, B3 = r2a - r1a + r12 - r2m2, r2a + r1a - r12 - ram2, ram2 - 2 * r2a + r2m2
        V = A1 * ratm + A2 * r2 + A3 * r1
        Vb = B1 * ratm + B2 * r2 + B3 * r1
        s = ratm - r2
        psiA = ic * (np.cross(ey, r21) - ic * V)
        psiB = ic * (np.cross(ey, s) - ic * Vb)
        chiB = ic * np.cross(ez, s)
        kd = _kappa(G, M, 0, 0) + _kappa(G, M, 1, 1)
        kzy = _kappa(G, M, 2, 1)
        hA = hA + psiA * kd
        hB = hB + psiB * kd + (chiB + byz) * kzy
    return hA, hB


def _block(rng):
    M = np.zeros((4, 4))
    for a, b in ME:
        M[a, b] = rng.normal()
    return M, rng.normal(size=(4, 4))


def test_rates_match_literal_standard_frame():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(300):
        r1 = rng.normal(size=3) * 3.0
        r2 = r1 + rng.normal(size=3) * 2.0
        ratm = rng.normal(size=3) * 3.0
        e, dA, dB, r21, z, rnabc, std = _frame(r1, r2, ratm)
        assert std
        M, rho = _block(rng)
        hA, hB = _rates(e, r1, r2, ratm, r21, z, rnabc, std, M, rho)
        ref = np.concatenate([_literal(e, dA, M, rho), _literal(e, dB, M, rho)])
        err = np.abs(np.concatenate([hA, hB]) - ref).max() / (1.0 + np.abs(ref).max())
        worst = max(worst, err)
    assert worst < 1e-12, worst


def test_rates_match_literal_fallback_frame():
    """epsilon's collinear fallback frame with |r21 x rnabc| >= 1e-3: the
    literal derivatives are then not a rotation of that frame, and the
    kernels add the psi / chi terms of frame_extra_3c."""
    rng = np.random.default_rng(7)
    n, worst, uncorrected = 0, 0.0, 0.0
    while n < 12:
        r1 = rng.normal(size=3) * 3.0
        r2 = r1 + rng.normal(size=3) * 3.0
        ax = (r2 - r1) / np.linalg.norm(r2 - r1)
        perp = np.cross(ax, rng.normal(size=3))
        perp /= np.linalg.norm(perp)
        d, s = rng.uniform(4.0, 8.0), rng.uniform(2e-5, 9e-5)
        ratm = r1 + 0.5 * (r2 - r1) + d * ax + d * s * perp
        e, dA, dB, r21, z, rnabc, std = _frame(r1, r2, ratm)
        if std or np.linalg.norm(np.cross(r21, rnabc)) < 1.0e-3:
            continue
        n += 1
        M, rho = _block(rng)
        ref = np.concatenate([_literal(e, dA, M, rho), _literal(e, dB, M, rho)])
        got = np.concatenate(_rates(e, r1, r2, ratm, r21, z, rnabc, False, M, rho))
        plain = np.concatenate(_rates(e, r1, r2, ratm, r21, z, rnabc, True, M, rho))
        scale = np.abs(ref).max()
        worst = max(worst, np.abs(got - ref).max() / scale)
        uncorrected = max(uncorrected, np.abs(plain - ref).max() / scale)
    # the fallback geometry is ill-conditioned (ic ~ 1e3, ic^2 V cancels):
    # rounding differences of ~1e-11 of the largest term remain
    assert worst < 1e-9, worst
    assert uncorrected > 1e-2


@pytest.mark.parametrize("seed", [0, 1])
def test_degenerate_triplet_has_no_frame_terms(seed):
    """|r21 x rnabc| < 1e-3: Depsilon_3c returns zeros and so do the rates."""
    rng = np.random.default_rng(seed)
    r1 = rng.normal(size=3)
    r2 = r1 + np.array([0.0, 0.0, 2.5])
    ratm = r1 + 0.5 * (r2 - r1) + np.array([0.0, 0.0, 3.0]) + 1e-5 * rng.normal(size=3)
    e, dA, dB, r21, z, rnabc, std = _frame(r1, r2, ratm)
    M, rho = _block(rng)
    hA, hB = _rates(e, r1, r2, ratm, r21, z, rnabc, std, M, rho)
    assert np.all(hA == 0.0) and np.all(hB == 0.0)
    assert np.abs(_literal(e, dA, M, rho)).max() == 0.0
    assert np.abs(_literal(e, dB, M, rho)).max() == 0.0


def _frame2(r1, r2):
    z = np.linalg.norm(r2 - r1)
    sig = (r2 - r1) / z
    e = O.epsilon(r2, sig)
    d = np.zeros(27)
    O.lib().or_depsilon_2c(np.ascontiguousarray(r1), np.ascontiguousarray(r2), float(z),
                           np.ascontiguousarray(e.T.ravel()), d)
    return e, d.reshape(3, 3, 3, order="F"), z


def test_two_center_rates_match_depsilon_2c():
    """The two-center force kernel's rates (frame_rates_2c) against the
    oracle's Depsilon_2c in the standard frame: e^T de is skew with
    W^xy = (e_x x r2)_q / |r2 x r1|, W^yz = -e_y,q / z, W^xz = -e_x,q / z."""
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(200):
        r1 = rng.normal(size=3) * 20.0
        r2 = r1 + rng.normal(size=3) * 2.0
        e, d, z = _frame2(r1, r2)
        ic, iz = 1.0 / np.linalg.norm(np.cross(r2, r1)), 1.0 / z
        ex, ey = e[:, 0], e[:, 1]
        wxy = ic * np.cross(ex, r2)
        for q in range(3):
            W = np.array([[0.0, wxy[q], -iz * ex[q]], [-wxy[q], 0.0, -iz * ey[q]], [iz * ex[q], iz * ey[q], 0.0]])
            Om = e.T @ d[q]
            worst = max(worst, np.abs(Om - W).max() / (1.0 + np.abs(Om).max()))
    assert worst < 1e-12, worst
