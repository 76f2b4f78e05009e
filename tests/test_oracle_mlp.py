"""CPU checks of the MLP-3c oracle itself: its back-propagation against
finite differences (float64, no BF16 rounding), and the BF16 rounding rule."""
import numpy as np

from oracle import mlp_oracle as mo


def _random_params(ntrip, seed):
    rng = np.random.default_rng(seed)
    sizes = [ntrip * 16, 128 * 32, 128, 128 * 128, 128, 128 * 128, 128, 64 * 128, 64]
    off = np.concatenate([[0], np.cumsum(sizes)])
    p = rng.normal(0.0, 0.1, off[-1])
    P = mo.unpack(p, off)
    P["W1"][:, 19:] = 0.0
    P["W4"][50:] = 0.0
    P["b4"][50:] = 0.0
    return mo.pack(P, off), off


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-3], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                 # halfway: ties to the even neighbor
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5
    assert abs(r[4] - 1e-3) <= 1e-3 * 2 ** -8


def test_oracle_gradient_finite_differences():
    ntrip, n = 8, 16
    p, off = _random_params(ntrip, 1)
    rng = np.random.default_rng(2)
    feat = rng.uniform(-1, 1, (n, 3))
    trip = rng.integers(0, ntrip, n)
    nme = np.array([10, 4, 4, 10, 10, 4, 4, 10])
    target = rng.normal(0, 1, (n, 64))
    loss, g = mo.loss_and_grad(mo.unpack(p, off), feat, trip, target, nme, exact=True)
    gv = mo.pack(g, off)
    # central differences on a sample of coordinates of every block
    idx = np.concatenate([rng.integers(off[k], off[k + 1], 6) for k in range(9)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = mo.loss_and_grad(mo.unpack(pp, off), feat, trip, target, nme, exact=True)
        lm, _ = mo.loss_and_grad(mo.unpack(pm, off), feat, trip, target, nme, exact=True)
        fd = (lp - lm) / (2 * h)
        in_pad = (off[1] <= i < off[2] and (i - off[1]) % 32 >= 19) or (off[7] + 50 * 128 <= i < off[8]) or \
            (off[8] + 50 <= i < off[9])
        if in_pad:
            assert gv[i] == 0.0
        else:
            assert abs(fd - gv[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, gv[i])
