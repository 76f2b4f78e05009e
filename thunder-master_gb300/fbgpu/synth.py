"""Seeded synthetic Fdata and structures in FIREBALL's own on-disk formats.

The reference ships no Fdata and no example inputs, so every workload is
generated here, deterministically from a seed, and written in exactly the text
formats the reference readers parse:

* ``info.dat``          -- read by ``read_info`` (c.SYSTEM/M_species.f90:1057-1251)
* ``2c.ZZ.ZZ.dat/.dir`` -- read by ``read_Fdata_2c`` (e.FDATA/M_Fdata_2c.f90:149-272)
* ``NN_munu_2c.ZZ.ZZ.dat`` (mu, nu, mvalue lines, M_Fdata_2c.f90:236-245)
* ``clPP.ZZ.dat``       -- opened unconditionally by read_Fdata_2c (:252-258)
* ``3c.ZZ.ZZ.ZZ.dat/.dir`` and the data files, iy outer / ix inner
  (e.FDATA/M_Fdata_3c.f90:192-231)
* ``03_munu_3c.ZZ.ZZ.ZZ.dat`` holding one (mu, nu, mvalue) triple of lines per
  theta cell, because the create step appends it once per theta
  (p.THEORY/M_bcna_Harris.f90:258-273) and the reader re-opens the unit
  without rewinding (M_Fdata_3c.f90:239-245).

Matrix-element index maps follow ``make_munu`` / ``make_munu_atom``
(c.SYSTEM/M_integrals_2c.f90:232-488) and ``make_munu_3c``
(c.SYSTEM/M_integrals_3c.f90:230-587).

Table values: every channel is a sum of three Gaussians times cubic
polynomials with seeded coefficients.  The two pi channels (m = -1, +1) of a
two-center table share coefficients so the physics is rotation invariant; the
three-center channels are independent.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

P_ABOHR = 0.529177  # include/constants.h:2

# interaction ids (include/interactions_2c.h:5-9, interactions_3c.h:8)
P_OVERLAP, P_KINETIC, P_VNA_ONTOPL, P_VNA_ONTOPR, P_VNA_ATOM = 1, 2, 3, 4, 5
P_VNL = 6           # include/interactions_2c.h:10
P_DIPOLE_Z = 10     # include/interactions_2c.h:14
P_BCNA = 3
P_NTHETA = 5
# McWEDA exchange-correlation (include/interactions_2c.h:11,20-26,
# interactions_3c.h:6-7)
P_VXC_ONTOP = 7
P_RHO_ONTOPL, P_RHO_ONTOPR, P_RHO_ATOM = 15, 16, 17
P_RHOS_ONTOPL, P_RHOS_ONTOPR, P_RHOS_ATOM = 19, 20, 21
P_RHO_3C, P_RHOS_3C = 1, 2


@dataclass
class Species:
    symbol: str
    nZ: int
    xmass: float
    lssh: list            # angular momentum per shell
    rcutoff: list         # bohr, per shell
    qneutral: list
    lssh_pp: list = field(default_factory=lambda: [0, 1])
    rcutoff_pp: float = 1.5

    @property
    def norb(self) -> int:
        return sum(2 * l + 1 for l in self.lssh)

    @property
    def rcA(self) -> float:
        """Largest shell cutoff in Angstrom (M_species.f90:1180-1183)."""
        return max(r * P_ABOHR for r in self.rcutoff)


def si(rc=5.0):
    return Species("Si", 14, 28.0855, [0, 1], [rc, rc], [2.0, 2.0])


def c(rc=5.0):
    return Species("C", 6, 12.011, [0, 1], [rc, rc], [2.0, 2.0])


def o(rc=4.0):
    return Species("O", 8, 15.999, [0, 1], [rc, rc], [2.0, 4.0])


def h(rc=4.0):
    return Species("H", 1, 1.008, [0], [rc], [1.0], lssh_pp=[0])


def ti(rc=5.0):
    """A transition-metal-like species with an s, p, d basis (9 orbitals),
    used only to exercise the d-orbital rotation paths."""
    return Species("Ti", 22, 47.867, [0, 1, 2], [rc, rc, rc], [2.0, 0.0, 2.0],
                   lssh_pp=[0, 1, 2])


# ---------------------------------------------------------------------------
# matrix-element maps
# ---------------------------------------------------------------------------
def make_munu(ls_i, ls_j):
    """(mu, nu, mvalue) lists of the 2c sigma/pi/delta map.

    Follows make_munu (c.SYSTEM/M_integrals_2c.f90:232-340): for every shell
    pair the channels m = -min(l1,l2)..min(l1,l2) sit at n1 + m, n2 + m where
    n1, n2 are the m=0 positions of the two shells.
    """
    mu, nu, mv = [], [], []
    n1 = 0
    for l1 in ls_i:
        n1 += l1 + 1
        n2 = 0
        for l2 in ls_j:
            n2 += l2 + 1
            for m in range(-min(l1, l2), min(l1, l2) + 1):
                mu.append(n1 + m)
                nu.append(n2 + m)
                mv.append(0)
            n2 += l2
        n1 += l1
    return mu, nu, mv


def make_munu_3c(ls_i, ls_j):
    """(mu, nu, mvalue) lists of the 3c map (c.SYSTEM/M_integrals_3c.f90:230-587):
    the 2c map with mvalue 0, then the mvalue 1 and mvalue 2 channels."""
    mu, nu, mv = make_munu(ls_i, ls_j)
    n1 = 0
    for l1 in ls_i:
        n1 += l1 + 1
        n2 = 0
        for l2 in ls_j:
            n2 += l2 + 1
            if l1 == 0 and l2 != 0:
                mu.append(n1); nu.append(n2 + 1); mv.append(1)
            if l1 == 1:
                mu.append(n1 + 1); nu.append(n2); mv.append(1)
                if l2 != 0:
                    mu.append(n1); nu.append(n2 + 1); mv.append(1)
                if l2 == 2:
                    mu.append(n1 + 1); nu.append(n2 + 2); mv.append(1)
                    mu.append(n1 - 1); nu.append(n2 - 2); mv.append(1)
            if l1 == 2:
                mu.append(n1 + 1); nu.append(n2); mv.append(1)
                if l2 != 0:
                    mu.append(n1); nu.append(n2 + 1); mv.append(1)
                    mu.append(n1 - 2); nu.append(n2 - 1); mv.append(1)
                    mu.append(n1 + 2); nu.append(n2 + 1); mv.append(1)
                if l2 == 2:
                    mu.append(n1 + 1); nu.append(n2 + 2); mv.append(1)
                    mu.append(n1 - 1); nu.append(n2 - 2); mv.append(1)
            n2 += l2
        n1 += l1
    n1 = 0
    for l1 in ls_i:
        n1 += l1 + 1
        n2 = 0
        for l2 in ls_j:
            n2 += l2 + 1
            if l1 == 2:
                mu.append(n1 + 2); nu.append(n2); mv.append(2)
            if l2 == 2:
                mu.append(n1); nu.append(n2 + 2); mv.append(2)
            n2 += l2
        n1 += l1
    return mu, nu, mv


def make_munu_s(ls_i, ls_j):
    """Shell-level map of make_munuS / make_munuS_atom / make_munuS_3c
    (c.SYSTEM/M_integrals_2c.f90:521-755, M_integrals_3c.f90:623-753): one
    channel per shell pair (issh outer, jssh inner), mvalue 0."""
    mu, nu, mv = [], [], []
    for a in range(len(ls_i)):
        for b in range(len(ls_j)):
            mu.append(a + 1)
            nu.append(b + 1)
            mv.append(0)
    return mu, nu, mv


def _orbital_lm(ls):
    """(shell index, l, m) for each orbital of a species, m = -l..l."""
    out = []
    for issh, l in enumerate(ls):
        for m in range(-l, l + 1):
            out.append((issh, l, m))
    return out


# ---------------------------------------------------------------------------
# table functions
# ---------------------------------------------------------------------------
_ALPHA = (3.0, 7.0, 16.0)

# Sign of each real orbital under a rotation by pi about the molecular x
# axis (x -> x, y -> -y, z -> -z); this maps the frame of pair (A, B) onto
# the frame of the reversed pair (B, A).  Orbital order in a shell is
# m = -l..l: p = (y, z, x), d = (xy, yz, z^2, xz, x^2-y^2).
_FLIP = {0: (1,), 1: (-1, -1, 1), 2: (-1, 1, 1, -1, 1)}


def _flip_sign(orb):
    _, l, m = orb
    return _FLIP[l][m + l]


def _f1d(coef, t, odd):
    """Sum of three Gaussians times cubics in t in [0, 1]."""
    val = np.zeros_like(t)
    for g, a in enumerate(_ALPHA):
        c0, c1, c2, c3 = coef[4 * g: 4 * g + 4]
        val += (c0 + c1 * t + c2 * t * t + c3 * t ** 3) * np.exp(-a * t * t)
    if odd:
        val = val * t
    return val


def _f2d(coef, u, v, scale):
    val = np.zeros(np.broadcast(u, v).shape)
    for g in range(3):
        cc = coef[10 * g: 10 * g + 10]
        poly = (cc[0] + cc[1] * u + cc[2] * v + cc[3] * u * u + cc[4] * u * v
                + cc[5] * v * v + cc[6] * u ** 3 + cc[7] * u * u * v
                + cc[8] * u * v * v + cc[9] * v ** 3)
        val = val + poly * np.exp(-_ALPHA[g] * u * u - 0.6 * _ALPHA[g] * v * v)
    return scale * val


def _seed_of(*keys):
    h = 1469598103934665603
    for k in keys:
        for ch in str(k).encode():
            h = ((h ^ ch) * 1099511628211) & ((1 << 63) - 1)
        h = ((h ^ 0x2C) * 1099511628211) & ((1 << 63) - 1)
    return h


_AMP2 = {P_OVERLAP: 0.6, P_KINETIC: 3.0, P_VNA_ONTOPL: 0.4, P_VNA_ONTOPR: 0.4, P_VNA_ATOM: 0.3,
         P_DIPOLE_Z: 0.5, P_VNL: 0.5, P_VXC_ONTOP: 0.8, P_RHO_ONTOPL: 0.25, P_RHO_ONTOPR: 0.25,
         P_RHO_ATOM: 0.1}
# ontop left / right pairs: <A|O_A|B> of (A, B) is <B|O_A|A> of (B, A)
_SWAP_LR = {P_VNA_ONTOPL: P_VNA_ONTOPR, P_VNA_ONTOPR: P_VNA_ONTOPL,
            P_RHO_ONTOPL: P_RHO_ONTOPR, P_RHO_ONTOPR: P_RHO_ONTOPL,
            P_RHOS_ONTOPL: P_RHOS_ONTOPR, P_RHOS_ONTOPR: P_RHOS_ONTOPL}
_RIGHT = (P_VNA_ONTOPR, P_RHO_ONTOPR, P_RHOS_ONTOPR)


def _base2c(seed, itype, zA, zB, oa, ob, t, asym_pi, isub=0):
    """Seeded channel function of the canonical orientation.  The m != 0
    channels equal the m = 0 channel plus t^2 times their own function, so
    all channels of a shell pair agree at zero separation (on-site blocks are
    then rotation invariant, as a physical table's are).  isub > 0: the
    charged-shell sub-cell isorp = isub (smaller amplitude)."""
    sa, la, ma = oa
    sb, lb, mb = ob
    sub = () if isub == 0 else ("isorp", isub)
    amp = _AMP2[itype] * (1.0 if isub == 0 else 0.4)
    rng = np.random.default_rng(_seed_of(seed, "2c", itype, zA, zB, sa, la, sb, lb, 0, *sub))
    val = amp * _f1d(rng.normal(0.0, 1.0, 12), t, (la + lb) % 2 == 1)
    mkey = ma if asym_pi else abs(ma)
    if mkey != 0:
        rng = np.random.default_rng(_seed_of(seed, "2c", itype, zA, zB, sa, la, sb, lb, mkey, *sub))
        val = val + t * t * amp * _f1d(rng.normal(0.0, 1.0, 12), t, False)
    return val


def table2c_vnl(seed, A, B, oa, ob, t):
    """<A oa | projector B ob> (interaction 6): a basis orbital of A against
    a pseudopotential projector of B.  No transpose symmetry relates it to
    <B ob | projector A oa>, so every (A, B) pair has its own channels; the
    m != 0 channels follow the m = 0 one as in _base2c (rotation invariant)."""
    sa, la, ma = oa
    sb, lb, mb = ob
    amp = _AMP2[P_VNL]
    rng = np.random.default_rng(_seed_of(seed, "vnl", A.nZ, B.nZ, sa, la, sb, lb, 0))
    val = amp * _f1d(rng.normal(0.0, 1.0, 12), t, (la + lb) % 2 == 1)
    if ma != 0:
        rng = np.random.default_rng(_seed_of(seed, "vnl", A.nZ, B.nZ, sa, la, sb, lb, abs(ma)))
        val = val + t * t * amp * _f1d(rng.normal(0.0, 1.0, 12), t, False)
    return val


def _canonical(zA, oa, zB, ob):
    return (zA, oa[0], oa[1]) <= (zB, ob[0], ob[1])


def table2c(seed, itype, A, B, oa, ob, t, asym_pi=False, isub=0):
    """Values of one 2c channel <A oa| O |B ob> on the grid t.

    Channels of the reversed pair are generated from the canonical ones with
    f^{BA}[nu, mu] = s(mu) s(nu) f^{AB}[mu, nu] (s = _flip_sign), so that
    S, T and the ontop potentials are Hermitian across neigh_back, and
    vna_ontopL of (B, A) is the transpose of vna_ontopR of (A, B)."""
    if itype in (P_VNA_ATOM, P_RHO_ATOM):   # both orbitals on A: symmetric in (mu, nu)
        if (oa[0], oa[1]) > (ob[0], ob[1]):
            oa, ob = ob, oa
        return _base2c(seed, itype, A.nZ, B.nZ, oa, ob, t, asym_pi, isub)
    if _canonical(A.nZ, oa, B.nZ, ob):
        if itype in _RIGHT and A.nZ == B.nZ and oa == ob:
            itype = _SWAP_LR[itype]
        return _base2c(seed, itype, A.nZ, B.nZ, oa, ob, t, asym_pi, isub)
    sign = _flip_sign(oa) * _flip_sign(ob)
    rtype = _SWAP_LR.get(itype, itype)
    if rtype in _RIGHT and A.nZ == B.nZ and oa == ob:
        rtype = _SWAP_LR[rtype]
    return sign * _base2c(seed, rtype, B.nZ, A.nZ, ob, oa, t, asym_pi, isub)


def _pos2c(seed, itype, zA, zB, sa, sb, t, isub):
    """A positive shell-level density channel a exp(-c t^2) (1 + 0.2 sin(...))."""
    rng = np.random.default_rng(_seed_of(seed, "2cS", itype, zA, zB, sa, sb, isub))
    a = 0.02 + 0.04 * rng.random()
    cc = 1.0 + 3.0 * rng.random()
    k, ph = 2.0 + 3.0 * rng.random(), 6.2832 * rng.random()
    return a * np.exp(-cc * t * t) * (1.0 + 0.2 * np.sin(k * t + ph))


def table2c_shell(seed, itype, A, B, sa, sb, t, isub):
    """Values of one shell-level density channel (rhoS ontop L / R, atom;
    interactions 19-21) between shell sa of A and shell sb of B (of A for
    the atom case).  Positive, and the ontop channels of the reversed pair
    are the transposed ones (the weighted densities are then symmetric
    across neigh_back)."""
    if itype == P_RHOS_ATOM:
        if sa > sb:
            sa, sb = sb, sa
        return _pos2c(seed, itype, A.nZ, B.nZ, sa, sb, t, isub)
    if (A.nZ, sa) <= (B.nZ, sb):
        if itype in _RIGHT and A.nZ == B.nZ and sa == sb:
            itype = _SWAP_LR[itype]
        return _pos2c(seed, itype, A.nZ, B.nZ, sa, sb, t, isub)
    rtype = _SWAP_LR[itype]
    if rtype in _RIGHT and A.nZ == B.nZ and sa == sb:
        rtype = _SWAP_LR[rtype]
    return _pos2c(seed, rtype, B.nZ, A.nZ, sb, sa, t, isub)


def table3c(seed, A, B, K, oa, ob, mval, itheta, u, v, theta_decay=1.0, isub=0, itype=P_BCNA):
    """Legendre coefficient itheta of the bcna channel <A oa| V_K |B ob>.

    c^{BAK}_l[nu, mu] = (-1)^l s(mu) s(nu) c^{ABK}_l[mu, nu] with l = itheta-1
    (reversing the bond flips cos(theta)), so the three-center blocks are
    Hermitian across neigh_back as well."""
    l = itheta - 1
    if (A.nZ, oa) == (B.nZ, ob):
        if l % 2 == 1:
            return np.zeros(np.broadcast(u, v).shape)
        key = (A.nZ, B.nZ, oa, ob)
        sign = 1.0
    elif (A.nZ, oa) < (B.nZ, ob):
        key = (A.nZ, B.nZ, oa, ob)
        sign = 1.0
    else:
        key = (B.nZ, A.nZ, ob, oa)
        sign = (-1.0) ** l * _flip_sign(oa) * _flip_sign(ob)
    sub = () if isub == 0 else ("isorp", isub)
    tag = () if itype == P_BCNA else ("itype", itype)
    rng = np.random.default_rng(_seed_of(seed, "3c", key, K.nZ, mval, itheta, *sub, *tag))
    coef = rng.normal(0.0, 1.0, 30)
    amp = 0.5 / (itheta ** theta_decay) * (1.0 if isub == 0 else 0.4)
    if itype == P_RHO_3C:
        amp *= 0.1
    return sign * _f2d(coef, u, v, amp)


def table3c_shell(seed, A, B, K, sa, sb, itheta, u, v, isub):
    """Legendre coefficient itheta of the shell-level three-center density
    (rhoS_3c, interaction 2) between shell sa of A and shell sb of B, the
    density of shell isub of K.  The isotropic term is positive; reversing
    the bond transposes the shells and flips the odd terms."""
    l = itheta - 1
    if (A.nZ, sa) == (B.nZ, sb):
        if l % 2 == 1:
            return np.zeros(np.broadcast(u, v).shape)
        key, sign = (A.nZ, B.nZ, sa, sb), 1.0
    elif (A.nZ, sa) < (B.nZ, sb):
        key, sign = (A.nZ, B.nZ, sa, sb), 1.0
    else:
        key, sign = (B.nZ, A.nZ, sb, sa), (-1.0) ** l
    rng = np.random.default_rng(_seed_of(seed, "3cS", key, K.nZ, itheta, isub))
    a = 0.004 + 0.008 * rng.random()
    cu, cv = 1.0 + 2.0 * rng.random(), 0.5 + rng.random()
    base = a * np.exp(-cu * u * u - cv * v * v)
    if l == 0:
        return base * (1.0 + 0.2 * np.sin(3.0 * u + 2.0 * v))
    return sign * 0.15 / itheta * base * np.sin((2.0 + l) * u + v + rng.random())


# ---------------------------------------------------------------------------
# writers
# ---------------------------------------------------------------------------
def _fmt(vals):
    return " ".join("%24.16E" % v for v in vals)


def write_fdata(path, species, seed=20261203, nx2c=200, n3c=31,
                asym_pi=False, theta_decay=1.0, dogs=False, vxc=False):
    """Write a complete Harris Fdata set for ``species`` into ``path``.

    nx2c: 2c grid points on [0, rcA_i + rcA_j] (200 points over 10 bohr for
    the rc = 5 bohr species).  n3c: 3c grid points on both axes.
    asym_pi: give the two pi channels of 2c tables different coefficients
    (breaks rotation invariance; used only to sharpen frame tests).
    dogs: also the charged-shell sub-cells isorp = 1..nssh of vna_ontopL
    (shells of the first atom), vna_ontopR and vna_atom (shells of the
    second atom) and bcna (shells of the neutral atom), and the z-dipole
    table, which the DOGS assemblers read.  Cells of one interaction are
    consecutive and its munu file holds one record triple per cell (the
    reference re-opens the open unit, which keeps its position).
    vxc: also the McWEDA exchange-correlation tables: vxc_ontop, the
    density sub-cells isorp = 1..nssh of den_ontopl / den_ontopr / den_atom
    and of their shell-level (spherical) forms, the three-center densities
    den3 and denS3 (shells of the third atom), and vxc_1c.ZZ.dat.
    """
    os.makedirs(path, exist_ok=True)
    ns = len(species)
    # Fdata.inp (M_species.f90:227-233)
    with open(os.path.join(path, "Fdata.inp"), "w") as f:
        f.write("%d\n" % ns)
        for s in species:
            f.write("%d\n" % s.nZ)
        f.write("%s\n" % path)
    # info.dat (M_species.f90:1094-1160): signature, count, 16 lines/species
    with open(os.path.join(path, "info.dat"), "w") as f:
        f.write("  synthetic seeded Fdata (gaussian-polynomial tables)\n")
        f.write("%12d\n" % ns)
        for isp, s in enumerate(species):
            f.write("  " + "=" * 70 + "\n")
            f.write("%12d  - Information for this species \n" % (isp + 1))
            f.write("  %-2s          - Element \n" % s.symbol)
            f.write("%12d  - Nuclear Z \n" % s.nZ)
            f.write("%12.4f  - Atomic Mass \n" % s.xmass)
            f.write("%12d  - Number of shells; L for each shell \n" % len(s.lssh))
            f.write("  " + " ".join("%d" % l for l in s.lssh) + "\n")
            f.write("  " + " ".join("%5.2f" % q for q in s.qneutral) + "\n")
            f.write("  " + " ".join("%7.4f" % r for r in s.rcutoff) + "\n")
            f.write("%12d  - Number of shells (PP) \n" % len(s.lssh_pp))
            f.write("  " + " ".join("%d" % l for l in s.lssh_pp) + "\n")
            f.write("%12.4f  - Radial cutoffs (PP) \n" % s.rcutoff_pp)
            f.write("  " + "  ".join("%-20s" % ("%03d_%02d.wf%d" % (s.nZ, int(10 * s.rcutoff[k]) % 100, k + 1))
                                       for k in range(len(s.lssh))) + "\n")
            f.write("  " + "  ".join("%-20s" % ("%03d_%02d.na%d" % (s.nZ, int(10 * s.rcutoff[0]) % 100, k))
                                       for k in range(len(s.lssh) + 1)) + "\n")
            f.write("%12.4f  - Atomic energy \n" % (-100.0 - s.nZ))
            f.write("  " + "=" * 70 + "\n")
    for s in species:
        with open(os.path.join(path, "clPP.%02d.dat" % s.nZ), "w") as f:
            for k in range(len(s.lssh_pp)):
                f.write("%22.14E\n" % (0.5 + 0.1 * k))

    # two-center tables
    for si_ in species:
        for sj in species:
            zz = "%02d.%02d" % (si_.nZ, sj.nZ)
            xmax = si_.rcA + sj.rcA
            x = np.linspace(0.0, xmax, nx2c)
            t = x / xmax
            mm = make_munu(si_.lssh, sj.lssh)
            ma = make_munu(si_.lssh, si_.lssh)
            nsub = {P_VNA_ONTOPL: len(si_.lssh), P_VNA_ONTOPR: len(sj.lssh), P_VNA_ATOM: len(sj.lssh)}
            stems = {P_VNA_ONTOPL: "vna_ontopl", P_VNA_ONTOPR: "vna_ontopr", P_VNA_ATOM: "vna_atom"}
            cells = [(P_OVERLAP, 0, "overlap", mm), (P_KINETIC, 0, "kinetic", mm)]
            for itype in (P_VNA_ONTOPL, P_VNA_ONTOPR, P_VNA_ATOM):
                for isub in range(0, (nsub[itype] if dogs else 0) + 1):
                    cells.append((itype, isub, "%s_%02d" % (stems[itype], isub),
                                  ma if itype == P_VNA_ATOM else mm))
            if dogs:
                cells.append((P_DIPOLE_Z, 0, "dipole_z", mm))
            if vxc:
                ms_ = make_munu_s(si_.lssh, sj.lssh)
                mas = make_munu_s(si_.lssh, si_.lssh)
                ni, nj = len(si_.lssh), len(sj.lssh)
                cells.append((P_VXC_ONTOP, 0, "vxc_ontop", mm))
                for itype, n, stem, mp in ((P_RHO_ONTOPL, ni, "den_ontopl", mm), (P_RHO_ONTOPR, nj, "den_ontopr", mm),
                                           (P_RHO_ATOM, nj, "den_atom", ma), (P_RHOS_ONTOPL, ni, "denS_ontopl", ms_),
                                           (P_RHOS_ONTOPR, nj, "denS_ontopr", ms_), (P_RHOS_ATOM, nj, "denS_atom", mas)):
                    for isub in range(1, n + 1):
                        cells.append((itype, isub, "%s_%02d" % (stem, isub), mp))
            # non-local pseudopotential <basis i | projector j> (every Fdata set)
            cells.append((P_VNL, 0, "vnl", make_munu(si_.lssh, sj.lssh_pp)))
            with open(os.path.join(path, "2c.%s.dat" % zz), "w") as f:
                f.write("%d\n" % len(cells))
            munu_records = {}
            with open(os.path.join(path, "2c.%s.dir" % zz), "w") as fd:
                for icell, (itype, isub, stem, (mu, nu, mv)) in enumerate(cells, start=1):
                    fname = "%s.%s.dat" % (stem, zz)
                    atom_like = itype in (P_VNA_ATOM, P_RHO_ATOM, P_RHOS_ATOM)
                    ls_b = si_.lssh if atom_like else sj.lssh_pp if itype == P_VNL else sj.lssh
                    orb_a, orb_b = _orbital_lm(si_.lssh), _orbital_lm(ls_b)
                    xm = si_.rcA + sj.rcutoff_pp if itype == P_VNL else xmax
                    tt = np.linspace(0.0, xm, nx2c) / xm
                    data = np.zeros((nx2c, len(mu)))
                    for ime in range(len(mu)):
                        if itype == P_VNL:
                            data[:, ime] = table2c_vnl(seed, si_, sj, orb_a[mu[ime] - 1], orb_b[nu[ime] - 1], tt)
                        elif itype in (P_RHOS_ONTOPL, P_RHOS_ONTOPR, P_RHOS_ATOM):
                            data[:, ime] = table2c_shell(seed, itype, si_, sj, mu[ime] - 1, nu[ime] - 1, t, isub)
                        else:
                            data[:, ime] = table2c(seed, itype, si_, sj, orb_a[mu[ime] - 1],
                                                   orb_b[nu[ime] - 1], t, asym_pi, isub)
                    with open(os.path.join(path, fname), "w") as f:
                        for ix in range(nx2c):
                            f.write(_fmt(data[ix]) + "\n")
                        f.write("\n")
                    fd.write("  %3d %3d %3d %-29s %3d %4d %9.6f\n"
                             % (icell, itype, isub, fname, len(mu), nx2c, xm))
                    munu_records.setdefault(itype, []).append((mu, nu, mv))
            for itype, recs in munu_records.items():
                with open(os.path.join(path, "%02d_munu_2c.%s.dat" % (itype, zz)), "w") as f:
                    for mu, nu, mv in recs:
                        f.write(" ".join("%d" % v for v in mu) + "\n")
                        f.write(" ".join("%d" % v for v in nu) + "\n")
                        f.write(" ".join("%d" % v for v in mv) + "\n")

    # three-center tables (bcna, theta = 1..5; isorp = 0, and with dogs the
    # neutral atom's shells isorp = 1..nssh)
    for si_ in species:
        for sj in species:
            for sk in species:
                zzz = "%02d.%02d.%02d" % (si_.nZ, sj.nZ, sk.nZ)
                ymax = si_.rcA + sj.rcA                       # dbc
                xmax = sk.rcA + max(si_.rcA, sj.rcA)          # dna
                m3 = make_munu_3c(si_.lssh, sj.lssh)
                orb_a, orb_b = _orbital_lm(si_.lssh), _orbital_lm(sj.lssh)
                u = np.linspace(0.0, 1.0, n3c)[None, :]       # x fastest
                v = np.linspace(0.0, 1.0, n3c)[:, None]
                nk = len(sk.lssh)
                # (itype, isub, stem, map), cells of one interaction consecutive
                cells = [(P_BCNA, isub, "bcna", m3) for isub in range(0, (nk if dogs else 0) + 1)]
                if vxc:
                    cells += [(P_RHO_3C, isub, "den3", m3) for isub in range(1, nk + 1)]
                    cells += [(P_RHOS_3C, isub, "denS3", make_munu_s(si_.lssh, sj.lssh)) for isub in range(1, nk + 1)]
                with open(os.path.join(path, "3c.%s.dat" % zzz), "w") as f:
                    f.write("%d\n" % (P_NTHETA * len(cells)))
                munu3 = {}
                icell = 0
                with open(os.path.join(path, "3c.%s.dir" % zzz), "w") as fd:
                    for itype, isub, stem, (mu, nu, mv) in cells:
                        for itheta in range(1, P_NTHETA + 1):
                            icell += 1
                            fname = "%s_%02d_%02d.%s.dat" % (stem, itheta, isub, zzz)
                            data = np.zeros((n3c, n3c, len(mu)))
                            for ime in range(len(mu)):
                                if itype == P_RHOS_3C:
                                    data[:, :, ime] = table3c_shell(seed, si_, sj, sk, mu[ime] - 1, nu[ime] - 1,
                                                                    itheta, u, v, isub)
                                else:
                                    data[:, :, ime] = table3c(seed, si_, sj, sk, orb_a[mu[ime] - 1],
                                                              orb_b[nu[ime] - 1], mv[ime], itheta, u, v,
                                                              theta_decay, isub, itype)
                            with open(os.path.join(path, fname), "w") as f:
                                for iy in range(n3c):
                                    for ix in range(n3c):
                                        f.write(_fmt(data[iy, ix]) + "\n")
                            fd.write("  %2d %2d %2d %3d %-29s %3d %4d %9.6f %4d %9.6f\n"
                                     % (icell, itype, isub, itheta, fname, len(mu), n3c, xmax, n3c, ymax))
                            munu3.setdefault(itype, []).append((mu, nu, mv))
                for itype, recs in munu3.items():
                    with open(os.path.join(path, "%02d_munu_3c.%s.dat" % (itype, zzz)), "w") as fm:
                        for mu, nu, mv in recs:
                            fm.write(" " + " ".join("%d" % q for q in mu) + "\n")
                            fm.write(" " + " ".join("%d" % q for q in nu) + "\n")
                            fm.write(" " + " ".join("%d" % q for q in mv) + "\n")
    if vxc:
        # one-center xc (read_Fdata_1c, e.FDATA/M_Fdata_1c_McWEDA_Harris.f90:118-136):
        # nssh rows of E, then nssh rows of V
        for s in species:
            n = len(s.lssh)
            rng = np.random.default_rng(_seed_of(seed, "1c", s.nZ))
            E = rng.normal(0.0, 0.3, (n, n))
            V = rng.normal(0.0, 0.3, (n, n))
            E = 0.5 * (E + E.T) - 8.0 * np.eye(n)
            V = 0.5 * (V + V.T) - 6.0 * np.eye(n)
            with open(os.path.join(path, "vxc_1c.%02d.dat" % s.nZ), "w") as f:
                for M in (E, V):
                    for r in M:
                        f.write(_fmt(r) + "\n")
    return path


# ---------------------------------------------------------------------------
# structures
# ---------------------------------------------------------------------------
@dataclass
class Structure:
    ratom: np.ndarray          # (N, 3) Angstrom
    imass: np.ndarray          # (N,) 1-based species index
    lattice: np.ndarray        # (3, 3) rows a1, a2, a3
    icluster: int = 0
    name: str = ""

    @property
    def natoms(self):
        return len(self.imass)


_DIAMOND_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                           [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])


def diamond(n, a, sigma, seed, sp_a=1, sp_b=1, vacancy=0.0, name=""):
    """n = (n1, n2, n3) conventional cells of diamond (sp_a == sp_b) or
    zincblende; Gaussian jitter sigma (Angstrom); random vacancy fraction."""
    rng = np.random.default_rng(seed)
    n1, n2, n3 = n
    pos, sp = [], []
    for i in range(n1):
        for j in range(n2):
            for k in range(n3):
                for b, fr in enumerate(_DIAMOND_BASIS):
                    pos.append((np.array([i, j, k]) + fr) * a)
                    sp.append(sp_a if b < 4 else sp_b)
    pos = np.array(pos, dtype=np.float64)
    sp = np.array(sp, dtype=np.int32)
    pos += rng.normal(0.0, sigma, pos.shape)
    if vacancy > 0:
        nvac = int(round(vacancy * len(sp)))
        keep = np.sort(rng.permutation(len(sp))[nvac:])
        pos, sp = pos[keep], sp[keep]
    lat = np.diag([n1 * a, n2 * a, n3 * a]).astype(np.float64)
    return Structure(pos, sp, lat, 0, name)


def random_box(counts, box, dmin, seed, name=""):
    """Uniform random positions in a cubic periodic box with a minimum image
    distance dmin (random sequential addition); counts = list of atoms per
    species (1-based species order)."""
    rng = np.random.default_rng(seed)
    total = sum(counts)
    sp = np.concatenate([np.full(cnt, isp + 1, np.int32) for isp, cnt in enumerate(counts)])
    sp = sp[rng.permutation(total)]
    pos = np.zeros((total, 3))
    ncell = max(1, int(box // dmin))
    grid = {}
    placed = 0
    while placed < total:
        trial = rng.uniform(0.0, box, 3)
        cidx = tuple((trial / box * ncell).astype(int) % ncell)
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    key = ((cidx[0] + dx) % ncell, (cidx[1] + dy) % ncell, (cidx[2] + dz) % ncell)
                    for q in grid.get(key, ()):
                        d = trial - pos[q]
                        d -= box * np.round(d / box)
                        if d @ d < dmin * dmin:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pos[placed] = trial
            grid.setdefault(cidx, []).append(placed)
            placed += 1
    return Structure(pos, sp, np.diag([box] * 3).astype(np.float64), 0, name)


# Workload definitions (synthetic, seeded)
SEED_SI64, SEED_SI512, SEED_CHO, SEED_BATCH, SEED_SIC = 1001, 1002, 1003, 1004, 1005


def species_for(workload):
    if workload in ("si64", "si512"):
        return [si(5.0)]
    if workload == "cho1536":
        return [c(4.5), h(4.0), o(4.0)]
    if workload in ("sic4096", "batch256"):
        return [si(5.0), c(5.0)]
    raise ValueError(workload)


def structure_for(workload):
    if workload == "si64":
        return diamond((2, 2, 2), 5.43, 0.05, SEED_SI64, name="Si64")
    if workload == "si512":
        return diamond((4, 4, 4), 5.43, 0.15, SEED_SI512, name="Si512")
    if workload == "cho1536":
        return random_box([384, 768, 384], 24.0, 1.0, SEED_CHO, name="CHO1536")
    if workload == "sic4096":
        return diamond((8, 8, 8), 4.36, 0.1, SEED_SIC, sp_a=1, sp_b=2, name="SiC4096")
    raise ValueError(workload)


def batch_structures(nstruct=256, seed=SEED_BATCH):
    """Independent Si / SiC structures of 32..512 atoms with 0-5 % vacancies."""
    rng = np.random.default_rng(seed)
    dims = [(a, b, cc) for a in range(1, 5) for b in range(1, 5) for cc in range(1, 5)
            if 32 <= 8 * a * b * cc <= 512]
    out = []
    for k in range(nstruct):
        target = int(rng.integers(32, 513))
        best = min(dims, key=lambda d: abs(8 * d[0] * d[1] * d[2] - target))
        zinc = bool(rng.integers(0, 2))
        a = 4.36 if zinc else 5.43
        vac = float(rng.uniform(0.0, 0.05))
        out.append(diamond(best, a, 0.1, int(rng.integers(1 << 30)), sp_a=1,
                           sp_b=2 if zinc else 1, vacancy=vac, name="batch%03d" % k))
    return out


def fdata_dir_for(workload, root=None, dogs=False, vxc=False):
    """Generate (once) and return the Fdata directory of a workload (with
    the DOGS sub-cells and dipole table when dogs is set, the McWEDA
    exchange-correlation tables when vxc is set)."""
    root = root or os.environ.get("FBGPU_FDATA_ROOT") or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "_fdata")
    key = {"si64": "Si_rc50", "si512": "Si_rc50", "cho1536": "CHO_rc45_40_40",
           "sic4096": "SiC_rc50", "batch256": "SiC_rc50"}[workload]
    path = os.path.join(root, key + ("_DOGS" if dogs else "") + ("_VXC" if vxc else ""))
    stamp = os.path.join(path, ".complete_vnl")
    if not os.path.exists(stamp):
        write_fdata(path, species_for(workload), dogs=dogs, vxc=vxc)
        with open(stamp, "w") as f:
            f.write("ok\n")
    return path


def symmetric_denmat(neighn, neigh_j0, neigh_back0, blk_off, norb_of, seed=42):
    """Seeded stand-ins for the density matrices rho and cape that the
    solver supplies, symmetric across neigh_back as the solver's are:
    rho_ji(nu, mu) = rho_ij(mu, nu).  neigh_j0 and neigh_back0 are 0-based
    (global atom index, position in j's list); blocks are column-major
    norb_i x norb_j at blk_off."""
    rng = np.random.default_rng(seed)
    NB = int(blk_off[-1])
    raw_r = rng.normal(0.0, 0.1, NB)
    raw_c = rng.normal(0.0, 0.05, NB)
    neigh_j0 = np.asarray(neigh_j0, np.int64)
    neigh_back0 = np.asarray(neigh_back0, np.int64)
    blk_off = np.asarray(blk_off, np.int64)
    norb_of = np.asarray(norb_of, np.int64)
    P = len(neigh_j0)
    pair_off = np.concatenate([[0], np.cumsum(neighn)]).astype(np.int64)
    owner = np.repeat(np.arange(len(neighn)), neighn)
    ni = norb_of[owner]
    nj = norb_of[neigh_j0]
    q = pair_off[neigh_j0] + neigh_back0
    # every element e of pair p: (mu, nu) column-major, mu fastest
    size = ni * nj
    pe = np.repeat(np.arange(P), size)
    loc = np.arange(NB) - np.repeat(blk_off[:P], size)
    mu = loc % np.repeat(ni, size)
    nu = loc // np.repeat(ni, size)
    # the mirrored element (nu, mu) of pair q (an nj x ni block)
    mirror = np.repeat(blk_off[q], size) + nu + np.repeat(nj, size) * mu
    lead = pe <= np.repeat(q, size)  # the pair with the smaller index supplies the values
    rho = np.where(lead, raw_r, raw_r[mirror])
    cape = np.where(lead, raw_c, raw_c[mirror])
    selfp = pe == np.repeat(q, size)
    rho[selfp] = 0.5 * (raw_r[selfp] + raw_r[mirror[selfp]])
    cape[selfp] = 0.5 * (raw_c[selfp] + raw_c[mirror[selfp]])
    return rho, cape
