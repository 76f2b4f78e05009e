// fb_internal.h -- device-visible data types and compile-time basis plans of
// libfbgpu (GB300 FIREBALL Harris assembly).  Shared by host and device code.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace fb {

constexpr int MAXSP = 8;         // species per Fdata set
constexpr int NTHETA = 5;        // Legendre terms of the 3c tables
constexpr double P_eq2 = 14.39975;   // include/constants.h:4
constexpr double P_abohr = 0.529177; // include/constants.h:2
constexpr double P_Hartree = P_eq2 / P_abohr;  // include/constants.h:5 (eV)
constexpr int P_mbox = 4;            // c.SYSTEM/M_configuraciones.f90:359
// periodic images of make_cells (c.SYSTEM/make_cells.f90:125-144): a
// (2 P_mbox + 1)^3 box, mbeta = 0 .. 728.  Every structure of a batch owns
// XL_STRIDE doubles of image vectors, xl(:, mbeta) at 3 * mbeta.
constexpr int NIMG = (2 * P_mbox + 1) * (2 * P_mbox + 1) * (2 * P_mbox + 1);
constexpr int XL_STRIDE = 3 * NIMG;
// MLP-3c results per triplet: 10 values (the bcna matrix elements of an sp x
// sp pair), and in the force pass 4 such rows: F, dF/dcos, dF/dx, dF/dy
constexpr int MLP_ME_STRIDE = 10;
constexpr int MAXSUB = 3;        // charged-shell sub-cells (isorp = 1..nssh) of the DOGS tables

// Basis patterns: the shell lists this build compiles rotation code for.
// PAT_S = [s], PAT_SP = [s, p], PAT_SPD = [s, p, d]; orbital order inside a
// shell is m = -l..l, p = (y, z, x) (c.SYSTEM/M_species.f90:1196-1208).
enum { PAT_S = 0, PAT_SP = 1, PAT_SPD = 2, NPAT = 3 };

__host__ __device__ constexpr int pat_norb(int P) { return P == PAT_S ? 1 : (P == PAT_SP ? 4 : 9); }
__host__ __device__ constexpr int pat_nssh(int P) { return P + 1; }
// shell of orbital o, its l and its 0-based m index within the shell
__host__ __device__ constexpr int orb_shell(int o) { return o == 0 ? 0 : (o < 4 ? 1 : 2); }
__host__ __device__ constexpr int shell_l(int s) { return s; }
__host__ __device__ constexpr int shell_off(int s) { return s == 0 ? 0 : (s == 1 ? 1 : 4); }
__host__ __device__ constexpr int orb_m(int o) { return o - shell_off(orb_shell(o)); }

// Matrix-element maps; 0-based orbital indices.
struct MEMap {
  int n;
  int mu[48];
  int nu[48];
  int mv[48];
};

// make_munu (c.SYSTEM/M_integrals_2c.f90:232-340); make_munu_atom is
// make_munu(PA, PA) (:379-488).
__host__ __device__ constexpr MEMap make_munu(int PA, int PB) {
  MEMap m{};
  int n1 = 0;
  for (int a = 0; a < pat_nssh(PA); a++) {
    int l1 = shell_l(a);
    n1 += l1 + 1;
    int n2 = 0;
    for (int b = 0; b < pat_nssh(PB); b++) {
      int l2 = shell_l(b);
      n2 += l2 + 1;
      int lm = l1 < l2 ? l1 : l2;
      for (int q = -lm; q <= lm; q++) {
        m.mu[m.n] = n1 + q - 1;
        m.nu[m.n] = n2 + q - 1;
        m.mv[m.n] = 0;
        m.n++;
      }
      n2 += l2;
    }
    n1 += l1;
  }
  return m;
}

// make_munu_3c (c.SYSTEM/M_integrals_3c.f90:230-587)
// make_munuS / make_munuS_atom / make_munuS_3c (c.SYSTEM/M_integrals_2c.f90:
// 521-755, M_integrals_3c.f90:623-753): one shell-level channel per shell
// pair, issh outer, mvalue 0.
__host__ __device__ constexpr MEMap make_munu_s(int PA, int PB) {
  MEMap m{};
  for (int a = 0; a < pat_nssh(PA); a++)
    for (int b = 0; b < pat_nssh(PB); b++) {
      m.mu[m.n] = a;
      m.nu[m.n] = b;
      m.mv[m.n] = 0;
      m.n++;
    }
  return m;
}

__host__ __device__ constexpr MEMap make_munu_3c(int PA, int PB) {
  MEMap m = make_munu(PA, PB);
  int n1 = 0;
  for (int a = 0; a < pat_nssh(PA); a++) {
    int l1 = shell_l(a);
    n1 += l1 + 1;
    int n2 = 0;
    for (int b = 0; b < pat_nssh(PB); b++) {
      int l2 = shell_l(b);
      n2 += l2 + 1;
      auto add = [&m](int mu, int nu, int mv) {
        m.mu[m.n] = mu - 1;
        m.nu[m.n] = nu - 1;
        m.mv[m.n] = mv;
        m.n++;
      };
      if (l1 == 0 && l2 != 0) add(n1, n2 + 1, 1);
      if (l1 == 1) {
        add(n1 + 1, n2, 1);
        if (l2 != 0) add(n1, n2 + 1, 1);
        if (l2 == 2) {
          add(n1 + 1, n2 + 2, 1);
          add(n1 - 1, n2 - 2, 1);
        }
      }
      if (l1 == 2) {
        add(n1 + 1, n2, 1);
        if (l2 != 0) {
          add(n1, n2 + 1, 1);
          add(n1 - 2, n2 - 1, 1);
          add(n1 + 2, n2 + 1, 1);
        }
        if (l2 == 2) {
          add(n1 + 1, n2 + 2, 1);
          add(n1 - 1, n2 - 2, 1);
        }
      }
      n2 += l2;
    }
    n1 += l1;
  }
  n1 = 0;
  for (int a = 0; a < pat_nssh(PA); a++) {
    int l1 = shell_l(a);
    n1 += l1 + 1;
    int n2 = 0;
    for (int b = 0; b < pat_nssh(PB); b++) {
      int l2 = shell_l(b);
      n2 += l2 + 1;
      if (l1 == 2) {
        m.mu[m.n] = n1 + 2 - 1; m.nu[m.n] = n2 - 1; m.mv[m.n] = 2; m.n++;
      }
      if (l2 == 2) {
        m.mu[m.n] = n1 - 1; m.nu[m.n] = n2 + 2 - 1; m.mv[m.n] = 2; m.n++;
      }
      n2 += l2;
    }
    n1 += l1;
  }
  return m;
}

// Per-species device record.
struct SpeciesDev {
  int pattern;   // PAT_*
  int norb;
  int nssh;      // shells
  double rcA;    // max shell cutoff, Angstrom
  double rcmin;  // min shell cutoff from 99, Angstrom (the DOGS smoothing range)
  // pseudopotential projectors: shell pattern (PAT_*, -1 if none of s, sp,
  // spd), orbitals, cutoff (as info.dat gives it) and cl per projector orbital
  int pp_pattern, norb_pp;
  double rc_pp;
  double cl[9];
  double q0;     // sum of the shells' Qneutral
  double qn[MAXSUB];  // Qneutral per shell
};

// One 2c interaction cell (T_Fdata_cell_2c, e.FDATA/M_Fdata_2c.f90:83-96).
// Values stored point-major: F[off + ix*nME + e] (all MEs of a grid point
// contiguous, so a 7-point stencil is one contiguous run).
struct Cell2cDev {
  int nx, nME;
  double dx, xmax;
  double inv_dx6;     // 1/dx^6 for the Lagrange weights
  long long off;      // -1 if the cell is absent
};

// One species triple of 3c bcna tables (T_Fdata_cell_3c, 5 theta cells).
// F[off + ((iy*nx + ix)*NTHETA + itheta)*nME + e]; per grid node the
// gradient switch of getMEs_Fdata_3c (M_Fdata_3c.f90:383-385) is
// precomputed: lin[node] = gg < 1e-6, gxy[2*node] = (gx, gy).
struct Cell3cDev {
  int nx, ny, nME;
  double dx, dy, xmax, ymax;
  double idxd, idyd;                 // 1/dx, 1/dy (the FP64 derivative weights)
  float idx_h, idx_l, idy_h, idy_l;  // 1/dx, 1/dy as hi + lo floats (the df derivative weights)
  long long off;      // -1 if absent
  long long node_off; // into lin / gxy
};

struct FdataDev {
  int nspecies;
  int have_d;
  int have_dogs;  // the DOGS sub-cells and the z-dipole table are present
  int have_pp;    // every species pair has its vnl table and a supported projector basis
  SpeciesDev sp[MAXSP];
  Cell2cDev c2[MAXSP][MAXSP][5];       // itype 1..5 -> [itype-1]
  Cell3cDev c3[MAXSP][MAXSP][MAXSP];   // (in1, in2, indna)
  // DOGS: charged-shell sub-cells isorp = 1..nssh of vna_ontopL, vna_ontopR,
  // vna_atom ([0..2][isorp-1]) and bcna, and the z-dipole table (itype 10)
  Cell2cDev c2s[MAXSP][MAXSP][3][MAXSUB];
  Cell2cDev c2dip[MAXSP][MAXSP];
  // non-local pseudopotential <basis of in1 | projector of in2> (itype 6)
  Cell2cDev c2vnl[MAXSP][MAXSP];
  Cell3cDev c3s[MAXSP][MAXSP][MAXSP][MAXSUB];
  // McWEDA exchange-correlation: vxc_ontop (itype 7); the density
  // sub-cells isorp = 1..nssh of rho ontop L (shells of the first species),
  // R, atom (shells of the second), and of their shell-level forms rhoS
  // ([0..5] = itype 15, 16, 17, 19, 20, 21); the three-center densities
  // den3 and denS3 ([0..1] = itype 1, 2; shells of the third species); the
  // one-center V(issh, jssh) at [issh * MAXSUB + jssh]
  int have_vxc;
  Cell2cDev c2vxc[MAXSP][MAXSP];
  Cell2cDev c2rho[MAXSP][MAXSP][6][MAXSUB];
  Cell3cDev c3rho[MAXSP][MAXSP][MAXSP][2][MAXSUB];
  // the same tables summed over isorp with the third species' Qneutral
  // weights (interpolation is linear in the table values and in the
  // linear-branch gradients) where the sub-cells share the grid (off = -1
  // where they do not); the gradient switch of a node is 2 where the
  // sub-cells disagree on it, and a triplet there takes them one by one
  Cell3cDev c3rhoq[MAXSP][MAXSP][MAXSP][2];
  int vxc_qsum_all;  // every triple has both summed cells and no node is 2
  double vxc1c[MAXSP][MAXSUB * MAXSUB];
};

// device status flags (bit mask, OR-ed by kernels)
enum : unsigned {
  DEVERR_XLARGE = 1u,
  DEVERR_CLOSE = 2u,
  DEVERR_SELF = 4u,
  DEVERR_BACK = 8u,
  DEVERR_TABLE = 16u,
  DEVERR_CAP = 32u,
  DEVERR_WATCHDOG = 64u,  // a bounded device wait ran out
};

}  // namespace fb
