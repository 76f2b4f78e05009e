"""CPU oracle of the MLP-3c surrogate (test infrastructure only).

The MLP has no reference counterpart: it stands in for the table walk of
getMEs_Fdata_3c (e.FDATA/M_Fdata_3c.f90:293-517), whose per-Legendre-term
values are its training targets.  This module restates, in numpy, the
network the GPU library trains and evaluates, with the same BF16 roundings
at the same points (weights, the input row, every hidden activation and
every back-propagated pre-activation gradient are rounded to BF16 before
they enter a product; products accumulate in float64 here and FP32 on the
GPU), so that the library's forward pass and gradients can be checked
against it.  ``exact=True`` drops the roundings (float64 throughout) for
finite-difference checks of the back-propagation itself.

The three coordinates enter as a BF16 pair: their rounding in columns 0..2
and the rounding of the remainder in columns 19..21, which share W1's
columns 0..2.

Parameter vector layout (float32): the 10 offsets of fb_mlp_layout --
embedding [ntriple][16], W1 [128][32], b1 [128], W2 [128][128], b2,
W3 [128][128], b3, W4 [64][128], b4 [64], end.
"""
from __future__ import annotations

import numpy as np

N_IN, N_EMB, N_H, N_OUT, N_ME, N_THETA = 32, 16, 128, 64, 10, 5
N_USED = N_THETA * N_ME
N_LO = 3 + N_EMB  # columns of the coordinates' low parts (weights tied to columns 0..2)


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(p, offsets):
    o = [int(v) for v in offsets]
    p = np.asarray(p, dtype=np.float64)
    return {
        "emb": p[o[0]:o[1]].reshape(-1, N_EMB),
        "W1": p[o[1]:o[2]].reshape(N_H, N_IN), "b1": p[o[2]:o[3]],
        "W2": p[o[3]:o[4]].reshape(N_H, N_H), "b2": p[o[4]:o[5]],
        "W3": p[o[5]:o[6]].reshape(N_H, N_H), "b3": p[o[6]:o[7]],
        "W4": p[o[7]:o[8]].reshape(N_OUT, N_H), "b4": p[o[8]:o[9]],
    }


def pack(d, offsets):
    out = np.zeros(int(offsets[-1]))
    for k, a, b in (("emb", 0, 1), ("W1", 1, 2), ("b1", 2, 3), ("W2", 3, 4), ("b2", 4, 5), ("W3", 5, 6),
                    ("b3", 6, 7), ("W4", 7, 8), ("b4", 8, 9)):
        out[int(offsets[a]):int(offsets[b])] = np.asarray(d[k]).ravel()
    return out


def used_mask(trip, nme):
    """[n][64] mask of the outputs a row's triple has (ime < nME, 50 used)."""
    o = np.arange(N_OUT)
    return (o[None, :] < N_USED) & ((o % N_ME)[None, :] < np.asarray(nme)[np.asarray(trip)][:, None])


def forward(P, feat3, trip, exact=False):
    """Normalized outputs [n][64] and the intermediates back-propagation needs."""
    r = (lambda v: np.asarray(v, dtype=np.float64)) if exact else bf16
    n = len(trip)
    X = np.zeros((n, N_IN))
    X[:, :3] = feat3
    X[:, 3:3 + N_EMB] = P["emb"][trip]
    X = r(X)
    if not exact:
        X[:, N_LO:N_LO + 3] = bf16(np.asarray(feat3, np.float32) - X[:, :3].astype(np.float32))
    cache = {"X": X, "Z": [], "H": []}
    h = X
    for l in (1, 2, 3):
        W = np.array(P["W%d" % l], dtype=np.float64)
        if l == 1:
            W[:, N_LO:N_LO + 3] = W[:, :3]
        z = h @ r(W).T + P["b%d" % l]
        h = r(silu(z))
        cache["Z"].append(z)
        cache["H"].append(h)
    out = h @ r(P["W4"]).T + P["b4"]
    return out, cache


def loss_and_grad(P, feat3, trip, target, nme, exact=False):
    """loss = sum over used outputs of (out - target)^2 / (50 n) and its
    gradient with respect to every parameter block."""
    r = (lambda v: np.asarray(v, dtype=np.float64)) if exact else bf16
    n = len(trip)
    out, c = forward(P, feat3, trip, exact)
    mask = used_mask(trip, nme)
    d = np.where(mask, out - target, 0.0)
    loss = float((d * d).sum() / (N_USED * n))
    g = {}
    dO = r(2.0 * d / (N_USED * n))
    H = c["H"]
    g["W4"] = dO.T @ H[2]
    g["W4"][N_USED:] = 0.0
    g["b4"] = dO.sum(0)
    g["b4"][N_USED:] = 0.0
    gin, Win = dO, r(P["W4"])
    for l in (3, 2, 1):
        dz = r((gin @ Win) * dsilu(c["Z"][l - 1]))
        hin = c["X"] if l == 1 else H[l - 2]
        g["W%d" % l] = dz.T @ hin
        g["b%d" % l] = dz.sum(0)
        W = np.array(P["W%d" % l], dtype=np.float64)
        if l == 1:
            W[:, N_LO:N_LO + 3] = W[:, :3]
        gin, Win = dz, r(W)
    g["W1"][:, :3] += g["W1"][:, N_LO:N_LO + 3]
    g["W1"][:, 3 + N_EMB:] = 0.0
    dX = gin @ Win
    gemb = np.zeros_like(P["emb"])
    np.add.at(gemb, np.asarray(trip), dX[:, 3:3 + N_EMB])
    g["emb"] = gemb
    return loss, g
