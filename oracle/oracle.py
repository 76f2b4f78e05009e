"""ctypes wrapper of the C oracle (oracle/fb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, by the smoke check and by
the CPU-baseline leg of the benchmark, always as the checker or the timed CPU
baseline, never as part of the GPU product path.  Parity status: unpinned
(the reference has no golden data and its Fortran cannot be built here).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "fb_oracle.c")):
            build()
        L = C.CDLL(LIB)
        L.or_load_fdata.restype = C.c_void_p
        L.or_load_fdata.argtypes = [C.c_char_p, C.c_int, _ip, C.c_char_p, C.c_int]
        L.or_free_fdata.argtypes = [C.c_void_p]
        L.or_species_norb.argtypes = [C.c_void_p, C.c_int]
        L.or_create_system.restype = C.c_void_p
        L.or_create_system.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _dp, C.c_int]
        L.or_free_system.argtypes = [C.c_void_p]
        L.or_neighbors.argtypes = [C.c_void_p]
        L.or_npairs.argtypes = [C.c_void_p]
        L.or_ntriplets.argtypes = [C.c_void_p]
        L.or_nblock.argtypes = [C.c_void_p]
        L.or_nblock.restype = C.c_longlong
        L.or_get_pairs.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _ip, _lp]
        L.or_get_triplets.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _ip, _ip]
        L.or_assemble_2c.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.or_assemble_3c.argtypes = [C.c_void_p, _dp]
        L.or_dassemble_2c.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.or_dassemble_3c.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.or_build_forces.argtypes = [C.c_void_p] + [_dp] * 13
        L.or_bloch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.or_set_charges.argtypes = [C.c_void_p, _dp, C.c_int]
        L.or_assemble_dipole_z.argtypes = [C.c_void_p, _dp]
        L.or_assemble_vna_2c_dogs.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.or_assemble_vna_3c_dogs.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.or_dassemble_dipole_z.argtypes = [C.c_void_p, _dp]
        L.or_neighbors_pp.argtypes = [C.c_void_p]
        L.or_assemble_ewald.argtypes = [C.c_void_p, _dp]
        L.or_dassemble_ewald.argtypes = [C.c_void_p, _dp, _dp]
        L.or_dassemble_ewaldsr.argtypes = [C.c_void_p] + [_dp] * 9
        L.or_dassemble_ewaldlr.argtypes = [C.c_void_p] + [_dp] * 8
        L.or_assemble_ewaldsr.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.or_assemble_ewaldlr.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.or_pp_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 4 + [C.POINTER(C.c_longlong)] * 2
        L.or_pp_sizes.restype = None
        L.or_get_pp.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, C.c_void_p, C.c_void_p]
        L.or_get_pp.restype = None
        L.or_get_pp_common.argtypes = [C.c_void_p] + [_ip] * 8
        L.or_get_pp_common.restype = None
        L.or_assemble_svnl.argtypes = [C.c_void_p, _dp]
        L.or_assemble_vnl_2c.argtypes = [C.c_void_p, _dp, _dp]
        L.or_assemble_vnl_3c.argtypes = [C.c_void_p, _dp, _dp]
        L.or_dassemble_svnl.argtypes = [C.c_void_p, _dp]
        L.or_dassemble_vnl_2c.argtypes = [C.c_void_p] + [_dp] * 5
        L.or_dassemble_vnl_3c.argtypes = [C.c_void_p] + [_dp] * 6
        L.or_build_forces_vnl.argtypes = [C.c_void_p] + [_dp] * 7
        L.or_dassemble_vna_2c_dogs.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.or_dassemble_vna_3c_dogs.argtypes = [C.c_void_p] + [_dp] * 8
        L.or_lda_ceperley_alder.argtypes = [C.c_double, _dp]
        L.or_assemble_rho_2c.argtypes = [C.c_void_p] + [_dp] * 4
        L.or_assemble_rho_3c.argtypes = [C.c_void_p] + [_dp] * 2
        L.or_dassemble_vxc.argtypes = [C.c_void_p] + [_dp] * 12
        L.or_assemble_vxc.argtypes = [C.c_void_p] + [_dp] * 6 + [C.c_void_p] * 3
        L.or_getMEs_2c.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _dp]
        L.or_getDMEs_2c.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                    _dp, _dp]
        L.or_getMEs_3c.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_int, C.c_int, C.c_double, _dp]
        L.or_getDMEs_3c.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.c_double, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _dp]
        L.or_epsilon.argtypes = [_dp, _dp, _dp]
        L.or_depsilon_2c.argtypes = [_dp, _dp, C.c_double, _dp, _dp]
        L.or_depsilon_3c.argtypes = [_dp, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp]
        L.or_rotate.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, C.c_int, _dp, _dp]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_set_exact_derivatives.argtypes = [C.c_int]
        L.or_last_error.restype = C.c_char_p
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("oracle status %d: %s" % (code, msg))
        self.code = code


def _check(st):
    if st != 0:
        raise OracleError(st, lib().or_last_error().decode())


class Fdata:
    def __init__(self, path, nZ):
        L = lib()
        err = C.create_string_buffer(512)
        nz = np.ascontiguousarray(nZ, dtype=np.int32)
        self.h = L.or_load_fdata(path.encode(), len(nz), nz, err, 512)
        if not self.h:
            raise OracleError(2, err.value.decode())
        self.nZ = list(nZ)

    def norb(self, isp):
        return lib().or_species_norb(self.h, isp)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_free_fdata(self.h)
            self.h = None


class System:
    """One structure with its neighbor maps, mirroring T_structure."""

    def __init__(self, fd: Fdata, ratom, imass, lattice, icluster=0, threads=1):
        L = lib()
        self.fd = fd
        self.ratom = np.ascontiguousarray(ratom, dtype=np.float64).reshape(-1, 3)
        self.imass = np.ascontiguousarray(imass, dtype=np.int32)
        self.lattice = np.ascontiguousarray(lattice, dtype=np.float64).reshape(3, 3)
        self.h = L.or_create_system(fd.h, len(self.imass), self.ratom.ravel(), self.imass,
                                    self.lattice.ravel(), icluster)
        if not self.h:
            raise OracleError(1, "bad system")
        self.threads = threads

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_free_system(self.h)
            self.h = None

    def neighbors(self):
        L = lib()
        L.or_set_threads(self.threads)
        _check(L.or_neighbors(self.h))
        N = len(self.imass)
        P = L.or_npairs(self.h)
        T = L.or_ntriplets(self.h)
        self.npairs, self.ntrip, self.nblock = P, T, L.or_nblock(self.h)
        self.pair_off = np.zeros(N + 1, np.int32)
        self.neigh_j = np.zeros(max(P, 1), np.int32)
        self.neigh_b = np.zeros(max(P, 1), np.int32)
        self.neigh_back = np.zeros(max(P, 1), np.int32)
        self.neigh_self = np.zeros(N, np.int32)
        self.blk_off = np.zeros(P + 1, np.int64)
        L.or_get_pairs(self.h, self.pair_off, self.neigh_j, self.neigh_b, self.neigh_back, self.neigh_self,
                       self.blk_off)
        self.trip_off = np.zeros(N + 1, np.int32)
        self.ci_j = np.zeros(max(T, 1), np.int32)
        self.ci_b = np.zeros(max(T, 1), np.int32)
        self.cj_j = np.zeros(max(T, 1), np.int32)
        self.cj_b = np.zeros(max(T, 1), np.int32)
        self.cneigh = np.zeros(max(T, 1), np.int32)
        L.or_get_triplets(self.h, self.trip_off, self.ci_j, self.ci_b, self.cj_j, self.cj_b, self.cneigh)
        return self

    def assemble(self, with3c=True):
        L = lib()
        L.or_set_threads(self.threads)
        nb = self.nblock
        S, T, vb, vbo = (np.zeros(nb) for _ in range(4))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        if with3c:
            _check(L.or_assemble_3c(self.h, vb))
        return S, T, vb, vbo

    def assemble_dogs(self, dQ, with3c=True):
        """DOGS value pass: S, T, vna (atom + 3c), vnao (ontop) and the
        z-dipole blocks, with shell charges dQ (natoms, nssh_max)."""
        L = lib()
        L.or_set_threads(self.threads)
        nb = self.nblock
        d = np.ascontiguousarray(dQ, np.float64)
        d = d.reshape(len(self.imass), -1)
        _check(L.or_set_charges(self.h, np.ascontiguousarray(d.ravel()), d.shape[1]))
        S, T, vb, vbo, dip = (np.zeros(nb) for _ in range(5))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        _check(L.or_assemble_dipole_z(self.h, dip))
        _check(L.or_assemble_vna_2c_dogs(self.h, S, vb, vbo))
        if with3c:
            _check(L.or_assemble_vna_3c_dogs(self.h, S, dip, vb))
        return S, T, vb, vbo, dip

    def assemble_3c_only(self):
        L = lib()
        L.or_set_threads(self.threads)
        vb = np.zeros(self.nblock)
        _check(L.or_assemble_3c(self.h, vb))
        return vb

    def bloch(self, kpts, blocks):
        """Dense complex matrices sum_pairs phase(k . vec) block over the
        k-points (nk, n, n), the reference's Hmatrix / Smatrix."""
        L = lib()
        k = np.ascontiguousarray(kpts, np.float64).reshape(-1, 3)
        n = int(sum(self.fd.norb(int(q)) for q in self.imass))
        out = np.zeros(len(k) * 2 * n * n)
        _check(L.or_bloch(self.h, len(k), k.ravel(), np.ascontiguousarray(blocks, np.float64), out))
        m = out.reshape(len(k), n, n, 2)   # [k][jnu][jmu][re/im] (column-major)
        return np.transpose(m[..., 0] + 1j * m[..., 1], (0, 2, 1))

    def dassemble(self, rho, cape):
        L = lib()
        L.or_set_threads(self.threads)
        nb, P, N = self.nblock, self.npairs, len(self.imass)
        rho = np.ascontiguousarray(rho, np.float64)
        cape = np.ascontiguousarray(cape, np.float64)
        dS, dT = np.zeros(3 * nb), np.zeros(3 * nb)
        ontop, atom = np.zeros(3 * P), np.zeros(3 * P)
        _check(L.or_dassemble_2c(self.h, rho, dS, dT, ontop, atom))
        fa, fb, fc = np.zeros(3 * N), np.zeros(3 * N), np.zeros(3 * N)
        _check(L.or_dassemble_3c(self.h, rho, fa, fb, fc))
        kin, vna, pul, ftot = (np.zeros(3 * N) for _ in range(4))
        _check(L.or_build_forces(self.h, rho, cape, dS, dT, ontop, atom, fa, fb, fc, kin, vna, pul, ftot))
        return dict(dS=dS, dT=dT, vna_ontop=ontop, vna_atom=atom, f3naa=fa, f3nab=fb, f3nac=fc,
                    kinetic=kin, vna=vna, pulay=pul, ftot=ftot)

    def dassemble_dogs(self, rho, cape, dQ):
        """DOGS force pass: the Harris S, T, Pulay and kinetic terms, the DOGS
        vna ontop / atom and f3na terms, and build_forces, with shell
        charges dQ (natoms, nssh_max)."""
        L = lib()
        L.or_set_threads(self.threads)
        nb, P, N = self.nblock, self.npairs, len(self.imass)
        d = np.ascontiguousarray(dQ, np.float64).reshape(N, -1)
        _check(L.or_set_charges(self.h, np.ascontiguousarray(d.ravel()), d.shape[1]))
        rho = np.ascontiguousarray(rho, np.float64)
        cape = np.ascontiguousarray(cape, np.float64)
        S, T, vb, vbo, dip = (np.zeros(nb) for _ in range(5))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        _check(L.or_assemble_dipole_z(self.h, dip))
        dS, dT, ddip = np.zeros(3 * nb), np.zeros(3 * nb), np.zeros(3 * nb)
        ontop, atom = np.zeros(3 * P), np.zeros(3 * P)
        _check(L.or_dassemble_2c(self.h, rho, dS, dT, ontop, atom))
        _check(L.or_dassemble_dipole_z(self.h, ddip))
        _check(L.or_dassemble_vna_2c_dogs(self.h, rho, S, ontop, atom))
        fa, fb, fc = np.zeros(3 * N), np.zeros(3 * N), np.zeros(3 * N)
        _check(L.or_dassemble_vna_3c_dogs(self.h, rho, S, dS, dip, ddip, fa, fb, fc))
        kin, vna, pul, ftot = (np.zeros(3 * N) for _ in range(4))
        _check(L.or_build_forces(self.h, rho, cape, dS, dT, ontop, atom, fa, fb, fc, kin, vna, pul, ftot))
        return dict(dS=dS, dT=dT, ddip=ddip, vna_ontop=ontop, vna_atom=atom, f3naa=fa, f3nab=fb, f3nac=fc,
                    kinetic=kin, vna=vna, pulay=pul, ftot=ftot)

    def assemble_ewald(self, dQ):
        """DOGS Ewald: the N x N matrix ewald(i, j) and the ewaldsr and
        ewaldlr block sets, with shell charges dQ (natoms, nssh_max)."""
        L = lib()
        N, nb = len(self.imass), self.nblock
        d = np.ascontiguousarray(dQ, np.float64).reshape(N, -1)
        _check(L.or_set_charges(self.h, np.ascontiguousarray(d.ravel()), d.shape[1]))
        S, T, vb, vbo, dip = (np.zeros(nb) for _ in range(5))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        _check(L.or_assemble_dipole_z(self.h, dip))
        ew = np.zeros(N * N)
        _check(L.or_assemble_ewald(self.h, ew))
        sr, lr = np.zeros(nb), np.zeros(nb)
        _check(L.or_assemble_ewaldsr(self.h, S, dip, sr))
        _check(L.or_assemble_ewaldlr(self.h, ew, S, dip, lr))
        return ew.reshape(N, N), sr, lr

    def dassemble_ewald(self, rho, dQ):
        """DOGS Ewald force pass: dewald (N, N, 3), the Ewald energy force,
        the ewaldsr pair forces (3 per pair) with their three-center part
        (f3naa/b/c), the ewaldlr atom forces, and their build_forces
        addition to ftot (-ewaldsr on i, + on j, + ewaldlr, + the f3na part)."""
        L = lib()
        N, nb, P = len(self.imass), self.nblock, self.npairs
        ew, _, _ = self.assemble_ewald(dQ)
        S, T, vb, vbo, dip = (np.zeros(nb) for _ in range(5))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        _check(L.or_assemble_dipole_z(self.h, dip))
        rho = np.ascontiguousarray(rho, np.float64)
        dS, dT, ddip = np.zeros(3 * nb), np.zeros(3 * nb), np.zeros(3 * nb)
        _check(L.or_dassemble_2c(self.h, rho, dS, dT, np.zeros(3 * P), np.zeros(3 * P)))
        _check(L.or_dassemble_dipole_z(self.h, ddip))
        dew, few = np.zeros(3 * N * N), np.zeros(3 * N)
        _check(L.or_dassemble_ewald(self.h, dew, few))
        fsr = np.zeros(3 * P)
        fa, fb, fc = np.zeros(3 * N), np.zeros(3 * N), np.zeros(3 * N)
        _check(L.or_dassemble_ewaldsr(self.h, rho, S, dS, dip, ddip, fsr, fa, fb, fc))
        flr = np.zeros(3 * N)
        _check(L.or_dassemble_ewaldlr(self.h, rho, np.ascontiguousarray(ew.ravel()), dew, S, dS, dip, ddip, flr))
        add = (flr + fa + fb + fc).reshape(N, 3)
        fs = fsr.reshape(P, 3)
        for i in range(N):
            for p in range(self.pair_off[i], self.pair_off[i + 1]):
                add[i] -= fs[p]
                add[self.neigh_j[p]] += fs[p]
        return dict(ewald=ew, dewald=dew.reshape(N, N, 3), fewald=few, ewaldsr=fsr, f3na_add=(fa, fb, fc),
                    ewaldlr=flr, ftot_add=add.ravel())

    # ---- McWEDA exchange-correlation (Harris) ---------------------------
    def assemble_vxc(self, with3c=True, parts=False):
        """McWEDA value pass: returns dict(S, rho_in, rho_bond, wrho_in,
        wrho_bond, vxc) and with parts also vxc_SN, vxc_SN_bond, vxc_bond.
        Weighted densities: (npairs, 9), element (issh, jssh) at
        issh + nssh_i * jssh."""
        L = lib()
        L.or_set_threads(self.threads)
        nb, P = self.nblock, self.npairs
        S, T, vb, vbo = (np.zeros(nb) for _ in range(4))
        _check(L.or_assemble_2c(self.h, S, T, vb, vbo))
        ri, rb, wi, wb = np.zeros(nb), np.zeros(nb), np.zeros(9 * max(P, 1)), np.zeros(9 * max(P, 1))
        _check(L.or_assemble_rho_2c(self.h, ri, rb, wi, wb))
        if with3c:
            _check(L.or_assemble_rho_3c(self.h, ri, wi))
        vxc = np.zeros(nb)
        out = dict(S=S, rho_in=ri, rho_bond=rb, wrho_in=wi.reshape(-1, 9)[:P], wrho_bond=wb.reshape(-1, 9)[:P],
                   vxc=vxc)
        if parts:
            sn, snb, bond = np.zeros(nb), np.zeros(nb), np.zeros(nb)
            _check(L.or_assemble_vxc(self.h, S, ri, rb, wi, wb, vxc, sn.ctypes.data, snb.ctypes.data,
                                     bond.ctypes.data))
            out.update(vxc_SN=sn, vxc_SN_bond=snb, vxc_bond=bond)
        else:
            _check(L.or_assemble_vxc(self.h, S, ri, rb, wi, wb, vxc, None, None, None))
        return out

    def dassemble_vxc(self, rho):
        """McWEDA force pass: dict(vxc_off_site, vxc_on_site (3 per pair),
        f3xca, f3xcb, f3xcc, and vxc, the pair sums build_forces makes of
        them (off + on site on i, minus on j), and ftot_add = vxc + f3xc)."""
        L = lib()
        N, nb, P = len(self.imass), self.nblock, self.npairs
        r = self.assemble_vxc()
        rho = np.ascontiguousarray(rho, np.float64)
        dS, dT = np.zeros(3 * nb), np.zeros(3 * nb)
        _check(L.or_dassemble_2c(self.h, rho, dS, dT, np.zeros(3 * P), np.zeros(3 * P)))
        off, on = np.zeros(3 * P), np.zeros(3 * P)
        fa, fb, fc = np.zeros(3 * N), np.zeros(3 * N), np.zeros(3 * N)
        wi = np.ascontiguousarray(r["wrho_in"].ravel())
        wb = np.ascontiguousarray(r["wrho_bond"].ravel())
        _check(L.or_dassemble_vxc(self.h, rho, r["S"], dS, r["rho_in"], r["rho_bond"], wi, wb, off, on, fa, fb, fc))
        pair = (off + on).reshape(P, 3)
        vxc = np.zeros((N, 3))
        for i in range(N):
            for p in range(self.pair_off[i], self.pair_off[i + 1]):
                vxc[i] += pair[p]
                vxc[self.neigh_j[p]] -= pair[p]
        return dict(vxc_off_site=off, vxc_on_site=on, f3xca=fa, f3xcb=fb, f3xcc=fc, vxc=vxc.ravel(),
                    ftot_add=vxc.ravel() + fa + fb + fc, values=r)

    # ---- non-local pseudopotential (vnl) --------------------------------
    def neighbors_pp(self):
        """driver_neighbors_PP: PP, PPx and PPp maps (0-based) and the PP
        common-neighbor triplets."""
        L = lib()
        _check(L.or_neighbors_pp(self.h))
        n = [C.c_int() for _ in range(4)]
        b = [C.c_longlong() for _ in range(2)]
        L.or_pp_sizes(self.h, *[C.byref(x) for x in n], *[C.byref(x) for x in b])
        self.npp, self.nppx, self.nppp, self.ntrip_pp = (x.value for x in n)
        self.nsvnl, self.nvnl = (x.value for x in b)
        N = len(self.imass)
        self.pp = {}
        for which, name, cnt in ((0, "PP", self.npp), (1, "PPx", self.nppx), (2, "PPp", self.nppp)):
            off = np.zeros(N + 1, np.int32)
            jj, bb = np.zeros(max(cnt, 1), np.int32), np.zeros(max(cnt, 1), np.int32)
            self_ = np.zeros(N, np.int32)
            mp, pt = np.zeros(max(cnt, 1), np.int32), np.zeros(max(cnt, 1), np.int32)
            L.or_get_pp(self.h, which, off, jj, bb, self_, mp.ctypes.data_as(C.c_void_p) if which < 2 else None,
                        pt.ctypes.data_as(C.c_void_p) if which == 1 else None)
            d = dict(off=off, j=jj[:cnt], b=bb[:cnt], self=self_)
            if which < 2:
                d["map"] = mp[:cnt]
            if which == 1:
                d["point"] = pt[:cnt]
            self.pp[name] = d
        T = self.ntrip_pp
        arrs = [np.zeros(N + 1, np.int32)] + [np.zeros(max(T, 1), np.int32) for _ in range(7)]
        L.or_get_pp_common(self.h, *arrs)
        self.pp["common"] = dict(off=arrs[0], i=arrs[1][:T], ib=arrs[2][:T], j=arrs[3][:T], jb=arrs[4][:T],
                                 m=arrs[5][:T], m31=arrs[6][:T], m32=arrs[7][:T])
        return self

    def assemble_pp(self, with3c=True):
        """svnl blocks (PP pairs) and vnl blocks (PPp pairs)."""
        L = lib()
        svnl, vnl = np.zeros(max(self.nsvnl, 1)), np.zeros(max(self.nvnl, 1))
        _check(L.or_assemble_svnl(self.h, svnl))
        _check(L.or_assemble_vnl_2c(self.h, svnl, vnl))
        if with3c:
            _check(L.or_assemble_vnl_3c(self.h, svnl, vnl))
        return svnl[:self.nsvnl], vnl[:self.nvnl]

    def dassemble_pp(self, rho_pp):
        """vnl force pass with the density over PPp: dsvnl, vnl_atom (per PP
        pair), vnl_ontop (per PPx pair), f3nl{a,b,c}, the vnl force and the
        build_forces addition to ftot."""
        L = lib()
        N = len(self.imass)
        svnl = np.zeros(max(self.nsvnl, 1))
        _check(L.or_assemble_svnl(self.h, svnl))
        dsvnl = np.zeros(max(3 * self.nsvnl, 1))
        _check(L.or_dassemble_svnl(self.h, dsvnl))
        rho = np.ascontiguousarray(rho_pp, np.float64)
        va, vo = np.zeros(max(3 * self.npp, 1)), np.zeros(max(3 * self.nppx, 1))
        _check(L.or_dassemble_vnl_2c(self.h, rho, svnl, dsvnl, va, vo))
        fa, fb, fc = np.zeros(3 * N), np.zeros(3 * N), np.zeros(3 * N)
        _check(L.or_dassemble_vnl_3c(self.h, rho, svnl, dsvnl, fa, fb, fc))
        vnl, add = np.zeros(3 * N), np.zeros(3 * N)
        _check(L.or_build_forces_vnl(self.h, va, vo, fa, fb, fc, vnl, add))
        return dict(dsvnl=dsvnl[:3 * self.nsvnl], vnl_atom=va[:3 * self.npp], vnl_ontop=vo[:3 * self.nppx],
                    f3nla=fa, f3nlb=fb, f3nlc=fc, vnl=vnl, ftot_vnl=add)


def getMEs_2c(fd, isp, jsp, iint, x, nmu, nnu, isub=0):
    out = np.zeros(nmu * nnu)
    _check(lib().or_getMEs_2c(fd.h, isp, jsp, iint, isub, float(x), nmu, nnu, out))
    return out.reshape(nnu, nmu).T


def getDMEs_2c(fd, isp, jsp, iint, x, nmu, nnu, isub=0):
    h, d = np.zeros(nmu * nnu), np.zeros(nmu * nnu)
    _check(lib().or_getDMEs_2c(fd.h, isp, jsp, iint, isub, float(x), nmu, nnu, h, d))
    return h.reshape(nnu, nmu).T, d.reshape(nnu, nmu).T


def getMEs_3c(fd, isp, jsp, ksp, x, y, cost, nmu, nnu, iint=3, isub=0):
    out = np.zeros(nmu * nnu)
    _check(lib().or_getMEs_3c(fd.h, isp, jsp, ksp, iint, isub, float(x), float(y), nmu, nnu, float(cost), out))
    return out.reshape(nnu, nmu).T


def getDMEs_3c(fd, isp, jsp, ksp, x, y, cost, nmu, nnu, iint=3, isub=0):
    h, dp, dx, dy = (np.zeros(nmu * nnu) for _ in range(4))
    _check(lib().or_getDMEs_3c(fd.h, isp, jsp, ksp, iint, isub, float(x), float(y), nmu, nnu, float(cost),
                               h, dp, dx, dy))
    return tuple(a.reshape(nnu, nmu).T for a in (h, dp, dx, dy))


def lda_ceperley_alder(rh):
    """(exc, muxc, dexc, d2exc, dmuxc, d2muxc) of lda_ceperley_alder."""
    out = np.zeros(6)
    lib().or_lda_ceperley_alder(float(rh), out)
    return out


def epsilon(r1, r2):
    out = np.zeros(9)
    lib().or_epsilon(np.ascontiguousarray(r1, np.float64), np.ascontiguousarray(r2, np.float64), out)
    return out.reshape(3, 3).T  # spe(i, j)


def rotate(fd, in1, in3, eps, mm):
    nmu, nnu = mm.shape
    out = np.zeros(nmu * nnu)
    e = np.ascontiguousarray(np.asarray(eps).T.ravel())
    lib().or_rotate(fd.h, in1, in3, e, nmu, nnu, np.ascontiguousarray(mm.T.ravel()), out)
    return out.reshape(nnu, nmu).T
