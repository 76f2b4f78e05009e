"""Closed-form matrix elements of a three-atom Si cluster on polynomial Fdata.

Used by the known-answer tests of the oracle and of the GPU path.  The Fdata
set is a seeded synthetic Si set whose Si-Si overlap table holds degree-6
polynomials of x (the 7-point Lagrange interpolation of getMEs_Fdata_2c,
e.FDATA/M_Fdata_2c.f90:302-415, reproduces them exactly) and whose bcna
tables hold products of cubics in x and y plus a plane (the 16-point
bicubic branch of getMEs_Fdata_3c, e.FDATA/M_Fdata_3c.f90:423-482,
reproduces them exactly).  The blocks are then known without any
interpolation code:

* the molecular-frame elements are the polynomials, summed over the
  Legendre terms P_0..P_4(cos theta) and multiplied by sin(theta) on the
  mvalue = 1 channels (M_Fdata_3c.f90:348-354, :497-507);
* the crystal-frame block is U M U^T, with U = diag(1, Q) for an sp3 atom:
  an s orbital is invariant and the p orbitals (ordered y, z, x) turn like
  the vector components, Q[a][c] = c-th molecular axis . a-th crystal axis
  (the Slater-Koster transformation, Phys. Rev. 94, 1498 (1954));
* the molecular axes are those of epsilon (b.FUNCTIONS/epsilon.f90:73-202):
  z' along the second vector, y' = z' x (first vector), x' = y' x z';
  the two-center assemblers pass the absolute position of atom j as the
  first vector (j.ASSEMBLERS/M_assemble_2c_Harris.f90:177), the
  three-center one the unit vector from the bond center to the neutral
  atom (j.ASSEMBLERS/M_assemble_3c_Harris.f90:189);
* the three-center term of the vna block (i, j) from the neutral atom k is
  P_eq2 U M(x, y, cos theta) U^T with y = |r_j - r_i|, x = |r_k - (r_i +
  r_j) / 2| and cos theta = sighat . rhat (M_assemble_3c_Harris.f90:82-227).
"""
import os
import shutil

import numpy as np

from fbgpu import synth

P_EQ2 = 14.39975
XMAX2 = 2 * 5.0 * 0.529177   # 2c overlap table range (A)
X3 = 10.0 * 0.529177         # both 3c axes span 10 bohr


def write_poly_fdata(dst):
    """A synthetic Si Fdata set with polynomial overlap and bcna tables;
    returns the polynomial coefficients."""
    src = dst + "_base"
    synth.write_fdata(src, [synth.si(5.0)])
    shutil.copytree(src, dst)
    x = np.linspace(0.0, XMAX2, 200)
    coef2 = np.random.default_rng(3).normal(size=(6, 7))
    data = np.stack([np.polyval(c, x / XMAX2) for c in coef2], axis=1)
    with open(os.path.join(dst, "overlap.14.14.dat"), "w") as f:
        for row in data:
            f.write(" ".join("%24.16E" % v for v in row) + "\n")
    n = 31
    u = np.linspace(0.0, 1.0, n)
    rng = np.random.default_rng(5)
    coef3 = {}
    for th in range(1, 6):
        cx = rng.normal(size=(10, 4))
        cy = rng.normal(size=(10, 4))
        coef3[th] = (cx, cy)
        with open(os.path.join(dst, "bcna_%02d_00.14.14.14.dat" % th), "w") as f:
            for iy in range(n):
                for ix in range(n):
                    # the plane keeps the gradient switch on the bicubic branch
                    vals = [np.polyval(cx[e], u[ix]) * np.polyval(cy[e], u[iy]) + 3.0 * u[ix] + 2.0 * u[iy]
                            for e in range(10)]
                    f.write(" ".join("%24.16E" % v for v in vals) + "\n")
    return coef2, coef3


def cluster():
    """Three Si atoms off the origin, pairwise 2.1-2.6 A apart, in a
    40 A box used as a cluster (no periodic images)."""
    r = np.array([[1.30, 0.70, -0.40], [3.35, 1.05, 0.20], [2.05, 2.85, 0.55]])
    return r, np.ones(3, np.int32), 40.0 * np.eye(3)


def _frame(v1, v2):
    z = v2 / np.linalg.norm(v2)
    y = np.cross(z, v1 / np.linalg.norm(v1))
    y /= np.linalg.norm(y)
    xx = np.cross(y, z)
    return xx, y, z


def _U(frame):
    xx, y, z = frame
    mol = [y, z, xx]           # p orbitals in (y, z, x) order
    Q = np.array([[mol[c][a] for c in range(3)] for a in (1, 2, 0)])
    U = np.eye(4)
    U[1:, 1:] = Q
    return U


def overlap_block(coef2, ri, rj):
    """S block (i, j), j != i: 4 x 4, rows on atom i."""
    r21 = rj - ri
    d = np.linalg.norm(r21)
    mu, nu, _ = synth.make_munu([0, 1], [0, 1])
    M = np.zeros((4, 4))
    for e in range(6):
        M[mu[e] - 1, nu[e] - 1] = np.polyval(coef2[e], d / XMAX2)
    U = _U(_frame(rj, r21))
    return U @ M @ U.T


def bcna_block(coef3, ri, rj, rk):
    """Three-center vna term of block (i, j) from the neutral atom k."""
    r21 = rj - ri
    y = np.linalg.norm(r21)
    sighat = r21 / y
    rnabc = rk - (ri + 0.5 * r21)
    x = np.linalg.norm(rnabc)
    rhat = rnabc / x
    c = float(sighat @ rhat)
    P = [1.0, c, 0.5 * (3 * c * c - 1), 0.5 * c * (5 * c * c - 3), 0.125 * (3 - c * c * (30 - 35 * c * c))]
    s = np.sqrt(max(1e-5, 1 - c * c))
    mu, nu, mv = synth.make_munu_3c([0, 1], [0, 1])
    M = np.zeros((4, 4))
    for e in range(10):
        v = sum(P[th - 1] * (np.polyval(coef3[th][0][e], x / X3) * np.polyval(coef3[th][1][e], y / X3)
                             + 3.0 * x / X3 + 2.0 * y / X3) for th in range(1, 6))
        M[mu[e] - 1, nu[e] - 1] = v * s if mv[e] == 1 else v
    U = _U(_frame(rhat, sighat))
    return P_EQ2 * (U @ M @ U.T)


def block_of(flat, blk_off, pair_off, neigh_j0, i, j):
    """Block (i, j) of a flat pair-major array (column-major 4 x 4)."""
    for p in range(pair_off[i], pair_off[i + 1]):
        if neigh_j0[p] == j:
            return flat[blk_off[p]:blk_off[p + 1]].reshape(4, 4).T
    raise KeyError((i, j))
