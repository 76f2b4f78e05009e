"""fbgpu -- GB300 (sm_103a) FIREBALL Harris matrix-element assembly.

Python host mirror of the reference's assembler interfaces over the C ABI of
``libfbgpu.so`` (include/fbgpu.h).  The procedure names follow the Fortran
modules they replace:

=====================  =============================================  ====================================
this module            reference procedure                            reference file
=====================  =============================================  ====================================
Context.read_Fdata     read_info + read_Fdata_2c + read_Fdata_3c      c.SYSTEM/M_species.f90:1057,
                                                                      e.FDATA/M_Fdata_2c.f90:149,
                                                                      e.FDATA/M_Fdata_3c.f90:143
Context.set_structure  read_positions + make_cells                    c.SYSTEM/make_cells.f90:51
Context.set_batch      (no counterpart) many structures, one system   --
Context.driver_neighbors  driver_neighbors                            c.SYSTEM/M_neighbors.f90:93
Context.assemble_S     assemble_S                                     j.ASSEMBLERS/M_assemble_2c_Harris.f90:89
Context.assemble_T     assemble_T                                     j.ASSEMBLERS/M_assemble_2c_Harris.f90:233
Context.assemble_vna_2c  assemble_vna_2c                              j.ASSEMBLERS/M_assemble_2c_Harris.f90:435
Context.assemble_vna_3c  assemble_vna_3c                              j.ASSEMBLERS/M_assemble_3c_Harris.f90:82
Context.Dassemble_*    Dassemble_S / _T / _vna_2c / _vna_3c           k.DASSEMBLERS/M_Dassemble_{2c,3c}_Harris.f90
Context.build_forces   build_forces (assembly terms)                  c.SYSTEM/M_build_forces.f90:172
Context.set_theory     DOGS instead of Harris vna 2c / 3c             j.ASSEMBLERS/M_assemble_2c_DOGS.f90:640,
                                                                      j.ASSEMBLERS/M_assemble_3c_DOGS.f90:158
Context.assemble_dipole_z  assemble_dipole_z                          j.ASSEMBLERS/M_assemble_2c_DOGS.f90:376
Context.bloch          Bloch sums into H(k), S(k)                     h.SOLVESH/M_kspace_Lowdin.f90:680
Context.assemble(FB_EWALD)  assemble_ewald / ewaldsr / ewaldlr (DOGS)  j.ASSEMBLERS/M_assemble_ewald_DOGS.f90
Context.driver_neighbors_PP  driver_neighbors_PP                      c.SYSTEM/M_neighbors_PP.f90:98
Context.assemble(FB_VNL)  assemble_svnl / vnl_2c / vnl_3c             j.ASSEMBLERS/M_assemble_PP_{2c,3c}.f90
Context.Dassemble(FB_VNL2C | FB_VNL3C)  Dassemble_svnl / vnl_2c / vnl_3c  k.DASSEMBLERS/M_Dassemble_PP_{2c,3c}.f90
Context.assemble(FB_VXC)  assemble_vxc (McWEDA, Harris)               j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90:102,
                                                                      j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90
Context.Dassemble(FB_VXC)  Dassemble_vxc (McWEDA, Harris)             k.DASSEMBLERS/M_Dassemble_vxc_McWEDA_Harris.f90:102,
                                                                      k.DASSEMBLERS/M_Dassemble_vxc_3c_McWEDA_Harris.f90:97
=====================  =============================================  ====================================

There is no CPU fallback: every call runs on the GPU through the native
library, and a missing library or GPU raises FBError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "_lib", "libfbgpu.so")

FB_S, FB_T, FB_VNA2C, FB_VNA3C, FB_ALL, FB_KEEP_DBLOCKS, FB_FORCES = 1, 2, 4, 8, 15, 16, 32
FB_DIPOLE = 64
FB_EWALD = 1024
FB_VXC = 2048
FB_SVNL, FB_VNL2C, FB_VNL3C = 128, 256, 512
FB_VNL = FB_SVNL | FB_VNL2C | FB_VNL3C
FB_PP_MAP, FB_PPX_MAP, FB_PPP_MAP = 0, 1, 2
FB_THEORY_HARRIS, FB_THEORY_DOGS = 0, 1
FB_MLP_OFF, FB_MLP_GATED, FB_MLP_ALL = 0, 1, 2
FB_MLP_ENGINE_MMA, FB_MLP_ENGINE_TC = 0, 1
TUNABLE = ("assemble_2c", "assemble_3c", "dassemble_2c", "dassemble_3c")
BLOCK = {"S": 0, "T": 1, "vna": 2, "vnao": 3, "dS": 4, "dT": 5, "rho": 6, "cape": 7, "dip": 8,
         "svnl": 9, "vnl": 10, "dsvnl": 11, "rho_pp": 12, "ewaldsr": 13, "ewaldlr": 14,
         "vxc": 15, "rho_in": 16, "rho_bond": 17, "wrho_in": 18, "wrho_bond": 19}
FORCE = {"ftot": 0, "kinetic": 1, "vna": 2, "pulay": 3, "f3naa": 4, "f3nab": 5, "f3nac": 6,
         "vna_ontop": 7, "vna_atom": 8,
         "vnl": 9, "f3nla": 10, "f3nlb": 11, "f3nlc": 12, "vnl_atom": 13, "vnl_ontop": 14,
         "ewaldsr": 15, "ewaldlr": 16, "ewald": 17,
         "vxc": 18, "f3xca": 19, "f3xcb": 20, "f3xcc": 21, "vxc_off_site": 22, "vxc_on_site": 23}
STATUS = {0: "OK", 1: "ARG", 2: "IO", 3: "TABLE", 4: "X_NEGATIVE", 5: "X_TOO_LARGE",
          6: "ATOMS_CLOSE", 7: "NEIGH_SELF", 8: "NEIGH_BACK", 9: "CUDA", 10: "WATCHDOG",
          11: "STATE", 12: "CAPACITY", 13: "UNSUPPORTED", 14: "SOLVER"}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")

# every symbol include/fbgpu.h declares, with its ctypes signature
_SIGS = {
    "fb_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "fb_destroy": (None, [C.c_void_p]),
    "fb_last_error": (C.c_char_p, [C.c_void_p]),
    "fb_version": (C.c_char_p, []),
    "fb_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fb_load_fdata": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, _ip]),
    "fb_species_norb": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_set_structure": (C.c_int, [C.c_void_p, C.c_int, _dp, _ip, _dp, C.c_int]),
    "fb_set_batch": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _ip, C.c_void_p, C.c_void_p]),
    "fb_get_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_update_positions": (C.c_int, [C.c_void_p, _dp]),
    "fb_mlp_init": (C.c_int, [C.c_void_p, C.c_ulonglong]),
    "fb_norbitals": (C.c_longlong, [C.c_void_p]),
    "fb_bloch": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_void_p]),
    "fb_bloch_device": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_solve_k": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_void_p, _dp, C.c_void_p, C.c_void_p]),
    "fb_step_forces": (C.c_int, [C.c_void_p] + [C.c_void_p] * 8),
    "fb_mlp_nparams": (C.c_longlong, [C.c_void_p]),
    "fb_mlp_layout": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fb_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fb_mlp_scales": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fb_mlp_train": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_double, C.c_ulonglong,
                               C.c_void_p]),
    "fb_mlp_samples": (C.c_int, [C.c_void_p, C.c_int, C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_mlp_grad": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p]),
    "fb_mlp_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_mlp_validate": (C.c_int, [C.c_void_p, C.c_int, C.c_ulonglong, C.c_void_p]),
    "fb_mlp_bin_errors": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_mlp_gate": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "fb_mlp_set_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_mlp_routed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_mlp_set_engine": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_mlp_eval_points": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "fb_assemble_graph": (C.c_int, [C.c_void_p, C.c_uint]),
    "fb_set_launch": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int]),
    "fb_get_launch": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_autotune": (C.c_int, [C.c_void_p, C.c_uint, C.c_int, C.c_void_p]),
    "fb_neighbors": (C.c_int, [C.c_void_p]),
    "fb_set_neighbors": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "fb_get_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "fb_get_neighbors": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "fb_get_common": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6),
    "fb_neighbors_pp": (C.c_int, [C.c_void_p]),
    "fb_get_pp_sizes": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6),
    "fb_get_pp_neighbors": (C.c_int, [C.c_void_p, C.c_int] + [C.c_void_p] * 6),
    "fb_get_pp_common": (C.c_int, [C.c_void_p] + [C.c_void_p] * 8),
    "fb_set_denmat_pp": (C.c_int, [C.c_void_p, _dp]),
    "fb_get_ewald": (C.c_int, [C.c_void_p, _dp]),
    "fb_set_denmat_pp_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fb_assemble": (C.c_int, [C.c_void_p, C.c_uint]),
    "fb_get_blocks": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "fb_device_blocks": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "fb_set_denmat": (C.c_int, [C.c_void_p, _dp, C.c_void_p]),
    "fb_dassemble": (C.c_int, [C.c_void_p, C.c_uint]),
    "fb_get_forces": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "fb_assemble_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "fb_set_denmat_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_get_timing": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "fb_probe_fp64": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fb_probe_fp32": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fb_dassemble_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fb_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_set_theory": (C.c_int, [C.c_void_p, C.c_int]),
    "fb_set_charges": (C.c_int, [C.c_void_p, _dp, C.c_int]),
}

FB_PREC_FP64, FB_PREC_DF = 0, 1

KERNELS = ("neigh_count", "neigh_fill", "neigh_back", "common_count", "common_fill", "assemble_2c",
           "assemble_3c", "dassemble_2c", "dassemble_3c", "build_forces", "trip_bins", "split_rho",
           "mlp_eval", "assemble_3c_mlp", "dassemble_3c_mlp", "bloch", "pp_pairs", "ppp", "pp_common", "svnl",
           "vnl_2c", "vnl_3c", "dsvnl", "dvnl_2c", "dvnl_3c", "vnl_forces", "ewald", "ewald_blocks",
           "rho_2c", "rho_3c", "vxc", "dvxc_2c", "dvxc_3c", "vxc_forces")


class FBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("fbgpu status %d (%s): %s" % (code, STATUS.get(code, "?"), msg))
        self.code = code


_lib = None


def load_library(path=LIBPATH):
    """Load libfbgpu.so (raises FBError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FBError(9, "native library %s is missing: build it with fbgpu.build.build()" % path)
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One GPU assembly context: Fdata, one structure, its neighbor maps and
    block sets (the parts of T_structure the assembly path owns)."""

    def __init__(self, device=0):
        L = load_library()
        h = C.c_void_p()
        st = L.fb_create(device, C.byref(h))
        if st != 0:
            raise FBError(st, "fb_create(device=%d) failed (no usable GPU?)" % device)
        self.h = h
        self.L = L
        self.nspecies = 0
        self.natoms = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.fb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise FBError(st, self.L.fb_last_error(self.h).decode())

    # ---- setup -------------------------------------------------------------
    def set_precision(self, mode):
        """FB_PREC_DF (default): three-center contractions in double-float
        on the FP32 pipe; FB_PREC_FP64: everything in FP64."""
        self._check(self.L.fb_set_precision(self.h, int(mode)))

    def set_theory(self, theory):
        """FB_THEORY_HARRIS (default) or FB_THEORY_DOGS: the charge-weighted
        neutral-atom terms of M_assemble_2c_DOGS.f90 / M_assemble_3c_DOGS.f90
        (value pass, FP64 kernels)."""
        self._check(self.L.fb_set_theory(self.h, int(theory)))

    def set_charges(self, dq):
        """DOGS shell charges Qin - Qneutral, one row per atom (natoms, nssh_max)."""
        d = np.ascontiguousarray(dq, np.float64)
        if d.ndim == 1:
            d = d.reshape(-1, 1)
        self._check(self.L.fb_set_charges(self.h, np.ascontiguousarray(d.reshape(-1)), int(d.shape[1])))

    def assemble_dipole_z(self):
        """z-dipole blocks (assemble_dipole_z, M_assemble_2c_DOGS.f90:376-499)."""
        self._check(self.L.fb_assemble(self.h, FB_DIPOLE))

    def set_stream(self, stream_ptr):
        self._check(self.L.fb_set_stream(self.h, C.c_void_p(stream_ptr)))

    def read_Fdata(self, fdata_dir, nZ):
        nz = np.ascontiguousarray(nZ, np.int32)
        self._check(self.L.fb_load_fdata(self.h, fdata_dir.encode(), len(nz), nz))
        self.nspecies = len(nz)
        self.norb_species = [self.L.fb_species_norb(self.h, k + 1) for k in range(len(nz))]

    def set_structure(self, ratom, imass, lattice, icluster=0):
        r = np.ascontiguousarray(ratom, np.float64).reshape(-1)
        im = np.ascontiguousarray(imass, np.int32)
        lat = np.ascontiguousarray(lattice if lattice is not None else np.eye(3), np.float64).reshape(-1)
        self._check(self.L.fb_set_structure(self.h, len(im), r, im, lat, int(icluster)))
        self.natoms = len(im)
        self.imass = im.copy()
        self.nstruct = 1

    def set_batch(self, structures):
        """Many independent structures assembled together.  ``structures`` is
        a list of (ratom (n, 3), imass (n,), lattice (3, 3) or None,
        icluster) tuples; later calls act on the whole batch and
        ``batch_offsets`` slices their results per structure."""
        nat = np.array([len(st[1]) for st in structures], np.int32)
        r = np.ascontiguousarray(np.concatenate([np.asarray(st[0], np.float64).reshape(-1, 3)
                                                 for st in structures]).reshape(-1))
        im = np.ascontiguousarray(np.concatenate([np.asarray(st[1], np.int32) for st in structures]))
        lat = np.ascontiguousarray(np.concatenate([
            np.asarray(st[2] if st[2] is not None else np.eye(3), np.float64).reshape(-1)
            for st in structures]))
        icl = np.array([int(st[3]) if len(st) > 3 else 0 for st in structures], np.int32)
        self._check(self.L.fb_set_batch(self.h, len(nat), nat, r, im, _ptr(lat), _ptr(icl)))
        self.natoms = len(im)
        self.imass = im.copy()
        self.nstruct = len(nat)

    def batch_offsets(self):
        """Per-structure offsets (nstruct + 1 each): atoms, pairs, triplets,
        block elements."""
        n = getattr(self, "nstruct", 1) + 1
        a, p, t = (np.zeros(n, np.int32) for _ in range(3))
        b = np.zeros(n, np.int64)
        self._check(self.L.fb_get_batch(self.h, _ptr(a), _ptr(p), _ptr(t), _ptr(b)))
        return dict(atom=a, pair=p, trip=t, block=b)

    def update_positions(self, ratom):
        self._check(self.L.fb_update_positions(self.h, np.ascontiguousarray(ratom, np.float64).reshape(-1)))

    def driver_neighbors(self):
        self._check(self.L.fb_neighbors(self.h))
        return self.sizes()

    def set_neighbors(self, neighn, neigh_j, neigh_b):
        self._check(self.L.fb_set_neighbors(self.h, np.ascontiguousarray(neighn, np.int32),
                                            np.ascontiguousarray(neigh_j, np.int32),
                                            np.ascontiguousarray(neigh_b, np.int32)))
        return self.sizes()

    def sizes(self):
        p, t, n = C.c_int(), C.c_int(), C.c_longlong()
        self._check(self.L.fb_get_sizes(self.h, C.byref(p), C.byref(t), C.byref(n)))
        self.npairs, self.ntrip, self.nblock = p.value, t.value, n.value
        return self.npairs, self.ntrip, self.nblock

    def neighbors(self):
        """Neighbor maps with the reference's 1-based indices."""
        N, P = self.natoms, self.npairs
        neighn = np.zeros(N, np.int32)
        nj, nb, nback = (np.zeros(max(P, 1), np.int32) for _ in range(3))
        nself = np.zeros(N, np.int32)
        blk = np.zeros(P + 1, np.int64)
        self._check(self.L.fb_get_neighbors(self.h, _ptr(neighn), _ptr(nj), _ptr(nb), _ptr(nback), _ptr(nself),
                                            _ptr(blk)))
        return dict(neighn=neighn, neigh_j=nj[:P], neigh_b=nb[:P], neigh_back=nback[:P], neigh_self=nself,
                    blk_off=blk)

    # ---- non-local pseudopotential (vnl) ----------------------------------
    def driver_neighbors_PP(self):
        """driver_neighbors_PP: PP, PPx, PPp maps and the PP common triplets."""
        self._check(self.L.fb_neighbors_pp(self.h))
        return self.pp_sizes()

    def pp_sizes(self):
        n = [C.c_int() for _ in range(4)]
        b = [C.c_longlong() for _ in range(2)]
        self._check(self.L.fb_get_pp_sizes(self.h, *[C.byref(x) for x in n], *[C.byref(x) for x in b]))
        self.npp, self.nppx, self.nppp, self.ntrip_pp = (x.value for x in n)
        self.nsvnl, self.nvnl = (x.value for x in b)
        return dict(npp=self.npp, nppx=self.nppx, nppp=self.nppp, ntrip=self.ntrip_pp, nsvnl=self.nsvnl,
                    nvnl=self.nvnl)

    def pp_neighbors(self, which):
        """One PP map (FB_PP_MAP, FB_PPX_MAP, FB_PPP_MAP), 1-based."""
        N = self.natoms
        cnt = {FB_PP_MAP: self.npp, FB_PPX_MAP: self.nppx, FB_PPP_MAP: self.nppp}[which]
        neighn, self_ = np.zeros(N, np.int32), np.zeros(N, np.int32)
        jj, bb, mp, pt = (np.zeros(max(cnt, 1), np.int32) for _ in range(4))
        self._check(self.L.fb_get_pp_neighbors(self.h, which, _ptr(neighn), _ptr(jj), _ptr(bb), _ptr(self_),
                                               _ptr(mp) if which != FB_PPP_MAP else None,
                                               _ptr(pt) if which == FB_PPX_MAP else None))
        d = dict(neighn=neighn, neigh_j=jj[:cnt], neigh_b=bb[:cnt], self=self_)
        if which != FB_PPP_MAP:
            d["map"] = mp[:cnt]
        if which == FB_PPX_MAP:
            d["point"] = pt[:cnt]
        return d

    def pp_common(self):
        N, T = self.natoms, self.ntrip_pp
        nc = np.zeros(N, np.int32)
        arr = [np.zeros(max(T, 1), np.int32) for _ in range(7)]
        self._check(self.L.fb_get_pp_common(self.h, _ptr(nc), *[_ptr(x) for x in arr]))
        return dict(ncommon=nc, iatom_j=arr[0][:T], iatom_b=arr[1][:T], jatom_j=arr[2][:T], jatom_b=arr[3][:T],
                    neigh_common=arr[4][:T], m31=arr[5][:T], m32=arr[6][:T])

    def ewald(self):
        """The N x N Ewald matrix of the last FB_EWALD assembly."""
        out = np.zeros(self.natoms * self.natoms)
        self._check(self.L.fb_get_ewald(self.h, out))
        return out.reshape(self.natoms, self.natoms)

    def set_denmat_pp(self, rho_pp):
        self._check(self.L.fb_set_denmat_pp(self.h, np.ascontiguousarray(rho_pp, np.float64)))

    def set_denmat_pp_device(self, ptr):
        self._check(self.L.fb_set_denmat_pp_device(self.h, C.c_void_p(ptr)))

    def common_neighbors(self):
        N, T = self.natoms, self.ntrip
        nc = np.zeros(N, np.int32)
        arrs = [np.zeros(max(T, 1), np.int32) for _ in range(5)]
        self._check(self.L.fb_get_common(self.h, _ptr(nc), *[_ptr(a) for a in arrs]))
        names = ["iatom_common_j", "iatom_common_b", "jatom_common_j", "jatom_common_b", "neigh_common"]
        out = {k: a[:T] for k, a in zip(names, arrs)}
        out["ncommon"] = nc
        return out

    # ---- assembly (j.ASSEMBLERS) ---------------------------------------------
    def assemble(self, what=FB_ALL):
        self._check(self.L.fb_assemble(self.h, what))

    def assemble_S(self):
        self.assemble(FB_S)

    def assemble_T(self):
        self.assemble(FB_T)

    def assemble_vna_2c(self):
        self.assemble(FB_VNA2C)

    def assemble_vna_3c(self):
        self.assemble(FB_VNA3C)

    def assemble_graph(self, what=FB_ALL | FB_FORCES):
        """Value pass (+ force pass with FB_FORCES) as one CUDA graph launch,
        captured once and replayed while the system stays the same."""
        self._check(self.L.fb_assemble_graph(self.h, what))

    def set_launch(self, kernel, threads, ctas_per_sm=0, chunk=1):
        self._check(self.L.fb_set_launch(self.h, kernel.encode(), threads, ctas_per_sm, chunk))

    def get_launch(self, kernel):
        t, c, k = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.fb_get_launch(self.h, kernel.encode(), C.byref(t), C.byref(c), C.byref(k)))
        return dict(threads=t.value, ctas_per_sm=c.value, chunk=k.value)

    def autotune(self, what=FB_ALL | FB_FORCES, reps=3):
        """Pick the fastest launch shape of each selected kernel; returns
        {kernel: (best ms per launch, shape)}.  Outputs must be recomputed
        afterwards."""
        best = np.zeros(4)
        self._check(self.L.fb_autotune(self.h, what, reps, _ptr(best)))
        return {k: (float(best[i]), self.get_launch(k)) for i, k in enumerate(TUNABLE) if best[i] > 0}

    # ---- Bloch sums (h.SOLVESH/M_kspace_Lowdin.f90) ----------------------------
    def bloch(self, kpts, H=True, S=True):
        """Dense complex H(k) (T + vna + vnao) and S(k), shape (nk, n, n)."""
        k = np.ascontiguousarray(kpts, np.float64).reshape(-1, 3)
        n = int(self.L.fb_norbitals(self.h))
        hk = np.zeros(len(k) * 2 * n * n) if H else None
        sk = np.zeros(len(k) * 2 * n * n) if S else None
        self._check(self.L.fb_bloch(self.h, len(k), k.ravel(), _ptr(hk), _ptr(sk)))

        def cplx(a):
            if a is None:
                return None
            m = a.reshape(len(k), n, n, 2)   # column-major: [k][col][row][re, im]
            return np.transpose(m[..., 0] + 1j * m[..., 1], (0, 2, 1))
        return cplx(hk), cplx(sk)

    def bloch_device(self, kpts, hk_ptr, sk_ptr, extra_ptr=None):
        k = np.ascontiguousarray(kpts, np.float64).reshape(-1, 3)
        self._check(self.L.fb_bloch_device(self.h, len(k), k.ravel(),
                                           None if extra_ptr is None else C.c_void_p(extra_ptr),
                                           None if hk_ptr is None else C.c_void_p(hk_ptr),
                                           None if sk_ptr is None else C.c_void_p(sk_ptr)))

    def step_forces(self, ratom, rho, cape, S=None, T=None, vna=None, vnao=None, ftot=None):
        """One value + force step through host arrays (fb_step_forces).  The
        outputs (C-contiguous float64 arrays of nblock or 3*natoms, or None)
        are filled in place; pinned arrays let the copies overlap."""
        ins = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (ratom, rho, cape)]
        outs = (S, T, vna, vnao, ftot)
        for o in outs:
            if o is not None and not (o.dtype == np.float64 and o.flags.c_contiguous):
                raise ValueError("outputs must be C-contiguous float64 arrays")
        ptr = lambda x: None if x is None else C.c_void_p(x.ctypes.data)
        self._check(self.L.fb_step_forces(self.h, *[ptr(x) for x in ins], *[ptr(o) for o in outs]))

    def solve_k(self, kpts, c_ptr=None, extra_ptr=None):
        """kspace_Lowdin per k-point: (band energies (nk, n) ascending,
        dropped overlap eigenvalues per k-point).  c_ptr: device buffer for
        the eigenvectors (nk column-major n x n complex), or None."""
        k = np.ascontiguousarray(kpts, np.float64).reshape(-1, 3)
        n = int(self.L.fb_norbitals(self.h))
        eig = np.zeros(len(k) * n)
        dropped = np.zeros(len(k), np.int32)
        self._check(self.L.fb_solve_k(self.h, len(k), k.ravel(), None if extra_ptr is None else C.c_void_p(extra_ptr),
                                      eig, None if c_ptr is None else C.c_void_p(c_ptr),
                                      dropped.ctypes.data_as(C.c_void_p)))
        return eig.reshape(len(k), n), dropped

    # ---- MLP-3c surrogate ------------------------------------------------------
    def mlp_init(self, seed=1):
        self._check(self.L.fb_mlp_init(self.h, seed))
        off = np.zeros(10, np.int64)
        self._check(self.L.fb_mlp_layout(self.h, _ptr(off)))
        self.mlp_offsets = off
        self.mlp_nparams = int(off[-1])
        self.mlp_ntriple = (int(off[1]) - int(off[0])) // 16
        return off

    def mlp_params(self):
        p = np.zeros(self.mlp_nparams, np.float32)
        self._check(self.L.fb_mlp_get_params(self.h, _ptr(p)))
        return p

    def mlp_scales(self):
        s = np.zeros((self.mlp_ntriple, 64), np.float32)
        self._check(self.L.fb_mlp_scales(self.h, _ptr(s)))
        return s

    def mlp_train(self, nsamples=1 << 22, epochs=20, batch=4096, lr=2e-3, seed=7):
        hist = np.zeros(epochs)
        self._check(self.L.fb_mlp_train(self.h, int(nsamples), int(epochs), int(batch), float(lr), int(seed),
                                        _ptr(hist)))
        return hist

    def mlp_samples(self, n, seed=3):
        f = np.zeros((n, 3), np.float32)
        t = np.zeros(n, np.int32)
        y = np.zeros((n, 64), np.float32)
        self._check(self.L.fb_mlp_samples(self.h, int(n), int(seed), _ptr(f), _ptr(t), _ptr(y)))
        return f, t, y

    def mlp_grad(self, feat3, trip, target):
        f = np.ascontiguousarray(feat3, np.float32)
        t = np.ascontiguousarray(trip, np.int32)
        y = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.mlp_nparams, np.float32)
        loss = C.c_double()
        self._check(self.L.fb_mlp_grad(self.h, len(t), _ptr(f), _ptr(t), _ptr(y), _ptr(g), C.byref(loss)))
        return loss.value, g

    def mlp_forward(self, feat3, trip):
        f = np.ascontiguousarray(feat3, np.float32)
        t = np.ascontiguousarray(trip, np.int32)
        out = np.zeros((len(t), 64), np.float32)
        self._check(self.L.fb_mlp_forward(self.h, len(t), _ptr(f), _ptr(t), _ptr(out)))
        return out

    def mlp_validate(self, samples_per_bin=64, seed=17):
        """Largest per-bin error of the network against the FP64 tables."""
        m = C.c_double()
        self._check(self.L.fb_mlp_validate(self.h, int(samples_per_bin), int(seed), C.byref(m)))
        return m.value

    def mlp_bin_errors(self):
        n = C.c_longlong()
        self._check(self.L.fb_mlp_bin_errors(self.h, None, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        self._check(self.L.fb_mlp_bin_errors(self.h, _ptr(out), C.byref(n)))
        return out

    def mlp_gate(self, tol_ha):
        """Approve the bins whose error keeps |dH| <= tol_ha (Hartree) in the
        worst case; returns (tau, coverage)."""
        tau, cov = C.c_double(), C.c_double()
        self._check(self.L.fb_mlp_gate(self.h, float(tol_ha), C.byref(tau), C.byref(cov)))
        return tau.value, cov.value

    def mlp_set_mode(self, mode):
        self._check(self.L.fb_mlp_set_mode(self.h, int(mode)))

    def mlp_eval_points(self, pts, triple, derivs=True):
        """The assembly's network evaluation at (x, y, cos) points:
        [n][4][10] = value, d/dcos, d/dx, d/dy (or [n][10] values)."""
        p = np.ascontiguousarray(pts, np.float32)
        t = np.ascontiguousarray(triple, np.int32)
        out = np.zeros((len(t), 4 if derivs else 1, 10), np.float32)
        self._check(self.L.fb_mlp_eval_points(self.h, len(t), _ptr(p), _ptr(t), int(bool(derivs)), _ptr(out)))
        return out if derivs else out[:, 0]

    def mlp_set_engine(self, engine):
        """FB_MLP_ENGINE_MMA (mma.sync) or FB_MLP_ENGINE_TC (tcgen05 + TMEM)."""
        self._check(self.L.fb_mlp_set_engine(self.h, int(engine)))

    def mlp_routed(self):
        a, b = C.c_int(), C.c_int()
        self._check(self.L.fb_mlp_routed(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def blocks(self, which):
        if which in ("svnl", "dsvnl"):
            n = self.nsvnl * (3 if which == "dsvnl" else 1)
        elif which in ("vnl", "rho_pp"):
            n = self.nvnl
        elif which in ("wrho_in", "wrho_bond"):
            n = 9 * self.npairs
        else:
            n = self.nblock * (3 if which in ("dS", "dT") else 1)
        out = np.zeros(max(n, 1))
        self._check(self.L.fb_get_blocks(self.h, BLOCK[which], out))
        return out[:n]

    def device_blocks(self, which):
        p = C.c_void_p()
        self._check(self.L.fb_device_blocks(self.h, BLOCK[which], C.byref(p)))
        return p.value

    # ---- forces (k.DASSEMBLERS, build_forces) --------------------------------
    def set_denmat(self, rho, cape=None):
        rho = np.ascontiguousarray(rho, np.float64)
        cape = None if cape is None else np.ascontiguousarray(cape, np.float64)
        self._check(self.L.fb_set_denmat(self.h, rho, _ptr(cape)))
        self._cape_keep = cape

    def set_denmat_device(self, rho_ptr, cape_ptr=None):
        self._check(self.L.fb_set_denmat_device(self.h, C.c_void_p(rho_ptr),
                                                None if cape_ptr is None else C.c_void_p(cape_ptr)))

    def Dassemble(self, what=FB_ALL, keep_dblocks=False):
        self._check(self.L.fb_dassemble(self.h, what | (FB_KEEP_DBLOCKS if keep_dblocks else 0)))

    def forces(self, which):
        n = 3 * {"vna_ontop": self.npairs, "vna_atom": self.npairs, "ewaldsr": self.npairs,
                 "vxc_off_site": self.npairs, "vxc_on_site": self.npairs}.get(which, self.natoms)
        if which == "vnl_atom":
            n = 3 * self.npp
        elif which == "vnl_ontop":
            n = 3 * self.nppx
        out = np.zeros(max(n, 1))
        self._check(self.L.fb_get_forces(self.h, FORCE[which], out))
        return out[:n]

    def build_forces(self):
        """All force arrays of the assembly terms (after Dassemble)."""
        return {k: self.forces(k) for k in FORCE}

    def assemble_step(self, ratom, S, T, vna, vnao):
        self._check(self.L.fb_assemble_step(self.h, _ptr(ratom), _ptr(S), _ptr(T), _ptr(vna), _ptr(vnao)))

    def kernel_launches(self):
        return int(self.L.fb_kernel_launches(self.h))

    def set_timing(self, enable=True):
        self._check(self.L.fb_set_timing(self.h, int(bool(enable))))

    def timing(self):
        """{kernel: (total device ms, launches)} since set_timing(True)."""
        out = {}
        for k in KERNELS:
            ms, n = C.c_double(), C.c_longlong()
            self._check(self.L.fb_get_timing(self.h, k.encode(), C.byref(ms), C.byref(n)))
            out[k] = (ms.value, n.value)
        return out

    def probe_fp32(self):
        """Measured FP32 FMA throughput, TFLOP/s."""
        t = C.c_double()
        self._check(self.L.fb_probe_fp32(self.h, C.byref(t)))
        return t.value

    def probe_fp64(self):
        """Measured FP64 FMA throughput, TFLOP/s."""
        t = C.c_double()
        self._check(self.L.fb_probe_fp64(self.h, C.byref(t)))
        return t.value
