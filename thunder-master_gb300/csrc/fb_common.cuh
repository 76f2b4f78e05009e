// fb_common.cuh -- device contexts and shared per-pair / per-triplet
// routines of the libfbgpu assembly kernels.
#pragma once
#include <cuda_runtime.h>
#include "fb_device.cuh"
#include "fb_df.cuh"
#include "fb_launch.h"
#include "fb_sched.cuh"

namespace fb {

#define FB_LAUNCH_CHECK()                         \
  do {                                            \
    cudaError_t e_ = cudaGetLastError();          \
    if (e_ != cudaSuccess) return (int)e_;        \
  } while (0)

// ===========================================================================
// 2c assembly: assemble_S, assemble_T, assemble_vna_2c
// (j.ASSEMBLERS/M_assemble_2c_Harris.f90:89-649).  One warp per atom i,
// one lane per neighbor pair; the vna_atom terms of i's pairs are summed by
// a warp reduction into i's self block.
// ===========================================================================
struct Ctx2c {
  int N, P;
  const int *pair_owner;
  const double *ratom;
  const int *sid;
  const int *isp;
  const FdataDev *fd;
  const double *table2c;
  const double *xl;
  const int *pair_off, *neigh_j, *neigh_b, *neigh_self;
  const long long *blk_off;
  double *S, *T, *vb, *vbo;
  unsigned *status;
  // DOGS: shell charges dq[atom * MAXSUB + isorp - 1] and the z-dipole blocks
  int dogs;
  const double *dq;
  double *dip;
};

// smoother (b.FUNCTIONS/smoother.f90:100-146), the scaler = 1 branch
__device__ __forceinline__ double smoother(double r, double rend, double x) {
  double rbegin = x * rend;
  if (r > rend) return 0.0;
  if (r < rbegin) return 1.0;
  double ratio = (r - rbegin) / (rend - rbegin);
  double sm = 1.0 - ratio * ratio;
  return sm * sm;
}

// Integer cell shift (ix, iy, iz) of image mbeta in the make_cells order
// (c.SYSTEM/make_cells.f90:125-144): iz outer, ix inner, the origin skipped.
__device__ __forceinline__ void mbeta_shift(int mb, int &sx, int &sy, int &sz) {
  int L = (mb == 0) ? 364 : (mb <= 364 ? mb - 1 : mb);
  sx = L % 9 - 4;
  sy = (L / 9) % 9 - 4;
  sz = L / 81 - 4;
}
__device__ __forceinline__ int shift_mbeta(int sx, int sy, int sz) {
  int L = (sz + 4) * 81 + (sy + 4) * 9 + (sx + 4);
  return L == 364 ? 0 : (L < 364 ? L + 1 : L);
}

// returns true when epsilon's frame is the standard one (y along r2 x sighat)
__device__ __forceinline__ bool pair_geom(const Ctx2c &c, int i, int p, double *r1, double *r2, double &z,
                                          double e[3][3]) {
  int j = c.neigh_j[p], mb = c.neigh_b[p];
  const double *xl = c.xl + (long long)c.sid[i] * XL_STRIDE;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r1[k] = c.ratom[3 * i + k];
    r2[k] = __dadd_rn(c.ratom[3 * j + k], xl[3 * mb + k]);
  }
  z = dist_rn(r1, r2);
  double sig[3];
  if (z < 1.0e-05) {
    sig[0] = 0.0;
    sig[1] = 0.0;
    sig[2] = 1.0;
  } else {
    double iz = 1.0 / z;
#pragma unroll
    for (int k = 0; k < 3; k++) sig[k] = (r2[k] - r1[k]) * iz;
  }
  return epsilon_fn(r2, sig, e);
}

// interpolate one 2c cell at the weights (getMEs_Fdata_2c :378-401)
template <int NE>
__device__ __forceinline__ void interp2c(const double *__restrict__ tab, const Cell2cDev &cell, int i0,
                                         const double w[7], double *v) {
  const double *F = tab + cell.off + (long long)i0 * NE;
#pragma unroll
  for (int e = 0; e < NE; e++) v[e] = w[0] * __ldg(F + e);
#pragma unroll
  for (int s = 1; s < 7; s++)
#pragma unroll
    for (int e = 0; e < NE; e++) v[e] = fma(w[s], __ldg(F + s * NE + e), v[e]);
}

__device__ __forceinline__ bool same_grid(const Cell2cDev &a, const Cell2cDev &b) {
  return a.nx == b.nx && a.dx == b.dx;
}

// ===========================================================================
// 3c assembly: assemble_vna_3c (j.ASSEMBLERS/M_assemble_3c_Harris.f90:82-227)
// One thread per triplet; bcna blocks accumulate by FP64 atomics into the
// vna block of pair (iatom, mneigh).
// ===========================================================================
struct Ctx3c {
  int N, T;
  const double *ratom;
  const int *sid;
  const int *isp;
  const FdataDev *fd;
  const double *table3c;
  const unsigned char *lin;
  const double *gxy;
  const double *xl;
  const int *trip_alpha, *ci_j, *ci_b, *cj_j, *cj_b, *tdst;
  const int *tperm;
  const long long *blk_off;
  double *vb;
  // force pass
  const double *rho;
  double *f3naa, *f3nab, *f3nac;
  // double-float copies (table values and rho blocks as hi + lo floats)
  const df *table3c_df;
  const df *rho_df;
  // MLP-3c results per list position (F or F, dF/dcos, dF/dx, dF/dy; 10 each)
  const float *mlpF;
  // DOGS: shell charges, overlap and z-dipole blocks of the pairs
  int dogs;
  const double *dq;
  const double *S, *dip;
  const double *dogs_ps;
};

struct TripGeom {
  double r1[3], r2[3], rna[3], r21[3], rnabc[3], sighat[3], rhat[3], z, x, cost;
  double e[3][3];
  bool estd;  // e has its y axis along sighat x rhat (not the collinear fallback)
};

// set-up of M_assemble_3c_Harris.f90:154-189
__device__ __forceinline__ void trip_geom(const Ctx3c &c, int t, int &ia, int &iat, int &jat, TripGeom &g) {
  ia = c.trip_alpha[t];
  iat = c.ci_j[t];
  jat = c.cj_j[t];
  int ib = c.ci_b[t], jb = c.cj_b[t];
  const double *xl = c.xl + (long long)c.sid[ia] * XL_STRIDE;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    g.rna[k] = c.ratom[3 * ia + k];
    g.r1[k] = __dadd_rn(c.ratom[3 * iat + k], xl[3 * ib + k]);
    g.r2[k] = __dadd_rn(c.ratom[3 * jat + k], xl[3 * jb + k]);
    g.r21[k] = __dsub_rn(g.r2[k], g.r1[k]);
  }
  g.z = dist_rn(g.r1, g.r2);
  if (g.z < 1.0e-05) {
    g.sighat[0] = 0.0;
    g.sighat[1] = 0.0;
    g.sighat[2] = 1.0;
  } else {
    double iz = 1.0 / g.z;
#pragma unroll
    for (int k = 0; k < 3; k++) g.sighat[k] = g.r21[k] * iz;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) g.rnabc[k] = __dsub_rn(g.rna[k], __dadd_rn(g.r1[k], g.r21[k] * 0.5));
  g.x = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(g.rnabc[0], g.rnabc[0]), __dmul_rn(g.rnabc[1], g.rnabc[1])),
                             __dmul_rn(g.rnabc[2], g.rnabc[2])));
  if (g.x < 1.0e-05) {
    g.rhat[0] = g.rhat[1] = g.rhat[2] = 0.0;
  } else {
    double ix = 1.0 / g.x;
#pragma unroll
    for (int k = 0; k < 3; k++) g.rhat[k] = g.rnabc[k] * ix;
  }
  g.cost = g.sighat[0] * g.rhat[0] + g.sighat[1] * g.rhat[1] + g.sighat[2] * g.rhat[2];
  g.estd = epsilon_unit(g.rhat, g.sighat, g.e);
}

// The frame-derivative terms of a triplet's three-center forces for s and p
// shells: hA_c = sum_e M_e H_c(e) for d/dratm and hB_c for d/dr1, H the
// Dtwister derivative (M_Drotations.f90:456-471) contracted with the
// density, through the rotation rates of the frame (frame_rates_3c; the
// collinear fallback frame through frame_extra_3c).  Gf is L^T rho L over
// the whole block (mol_G_full), M the molecular-frame block at the ME
// positions.
template <int PA, int PB>
__device__ __forceinline__ void frame_terms_3c(const TripGeom &g, const double *Gf, const double *M, double hA[3],
                                               double hB[3]) {
  double tau[3];
  mol_tau<PA, PB>(Gf, M, tau);
  FrameRates3c w;
  frame_rates_3c(g.r2, g.r21, g.z, g.rna, g.rnabc, g.e, w);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    hA[q] = w.axy[q] * tau[0];
    hB[q] = fma(w.bxz[q], tau[2], fma(w.byz[q], tau[1], w.bxy[q] * tau[0]));
  }
  if (!g.estd) {
    FrameExtra3c x;
    frame_extra_3c(g.r1, g.r2, g.r21, g.rna, g.rnabc, g.e, x);
    double kd, kzy;
    mol_kappa_extra<PA, PB>(Gf, M, kd, kzy);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      hA[q] = fma(x.psiA[q], kd, hA[q]);
      hB[q] = fma(x.chiB[q] + w.byz[q], kzy, fma(x.psiB[q], kd, hB[q]));
    }
  }
}

// getMEs_Fdata_3c / getDMEs_Fdata_3c (e.FDATA/M_Fdata_3c.f90:293-846):
// Legendre sum over the 5 theta tables of a bicubic (or, where the table is
// flat, three-point linear) interpolation.  F, and with DERIV DpF, DxF, DyF,
// are returned before the sin(theta) factor of the mvalue = 1 channels.
template <int NE, bool DERIV>
__device__ __forceinline__ void interp3c(const Ctx3c &c, const Cell3cDev &cell, double x, double y, double cost,
                                         double *F, double *DpF, double *DxF, double *DyF) {
  double cost2 = cost * cost;
  double pl[5] = {1.0, cost, 0.5 * (3.0 * cost2 - 1.0), 0.5 * cost * (5.0 * cost2 - 3.0),
                  0.125 * (3.0 - cost2 * (30.0 - 35.0 * cost2))};
  double dpl[5] = {0.0, 1.0, 3.0 * cost, (15.0 * cost2 - 3.0) * 0.5, 0.5 * cost * (35.0 * cost2 - 15.0)};
  int ix = (int)(x / cell.dx) + 1;
  int iy = (int)(y / cell.dy) + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > cell.nx - 2) ix = cell.nx - 2;
  if (iy > cell.ny - 2) iy = cell.ny - 2;
  double px = x / cell.dx - ix + 1.0;
  double py = y / cell.dy - iy + 1.0;
  int nx = cell.nx;
  long long node0 = (long long)(iy - 1) * nx + (ix - 1);  // 0-based node of (ix, iy)
  const double *tab = c.table3c + cell.off;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    F[e] = 0.0;
    if (DERIV) DpF[e] = DxF[e] = DyF[e] = 0.0;
  }
  if (c.lin[cell.node_off + node0]) {
    // METHOD 1, three-point linear (:406-410, :684-691)
    double gx = c.gxy[2 * (cell.node_off + node0)], gy = c.gxy[2 * (cell.node_off + node0) + 1];
    double w00 = 1.0 - px - py;
    const double *T00 = tab + node0 * NTHETA * NE;
    const double *T10 = tab + (node0 + 1) * NTHETA * NE;
    const double *T01 = tab + (node0 + nx) * NTHETA * NE;
#pragma unroll
    for (int th = 0; th < NTHETA; th++)
#pragma unroll
      for (int e = 0; e < NE; e++) {
        double I = w00 * __ldg(T00 + th * NE + e) + px * __ldg(T10 + th * NE + e) + py * __ldg(T01 + th * NE + e);
        F[e] = fma(pl[th], I, F[e]);
        if (DERIV) {
          DpF[e] = fma(dpl[th], I, DpF[e]);
          DxF[e] = fma(pl[th], gx, DxF[e]);
          DyF[e] = fma(pl[th], gy, DyF[e]);
        }
      }
    return;
  }
  const double *Tb = tab + (node0 - nx - 1) * NTHETA * NE;  // node (ix-1, iy-1)
  if constexpr (DERIV) {
    // METHOD 3 with derivatives (:721-798).  The interpolation is linear in
    // the table values, so the Legendre sums are taken first at each of the
    // 16 stencil nodes, g = sum_th P_th T_th and gp = sum_th P'_th T_th, and
    // the stencil weights then contract g (value, d/dx, d/dy) and gp
    // (d/dcos), as a tensor product: along each stencil row the x weights
    // give A = sum_k wx g, B = sum_k wx' g, C = sum_k wx gp, and the row's y
    // weight adds wy A, wy B, wy' A, wy C.  11 FP64 FMAs per node and element
    // instead of 15 + 20/16 for the per-theta contraction, and no products of
    // the x and y weights.  The sums differ from the reference's order only
    // by rounding.
    double wx[4], wy[4], dwx[4], dwy[4];
    lagrange4(px, wx, dwx);
    lagrange4(py, wy, dwy);
    const double idx = cell.idxd, idy = cell.idyd;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      dwx[k] *= idx;
      dwy[k] *= idy;
    }
#pragma unroll 1
    for (int j = 0; j < 4; j++) {
      double wyj = wy[j], dwyj = dwy[j];
      const double *Tr = Tb + (long long)j * nx * NTHETA * NE;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        double A = 0.0, B = 0.0, C = 0.0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const double *Tn = Tr + k * NTHETA * NE + e;
          double t0 = __ldg(Tn), t1 = __ldg(Tn + NE), t2 = __ldg(Tn + 2 * NE);
          double t3 = __ldg(Tn + 3 * NE), t4 = __ldg(Tn + 4 * NE);
          double g = fma(pl[4], t4, fma(pl[3], t3, fma(pl[2], t2, fma(pl[1], t1, t0))));
          double gp = fma(dpl[4], t4, fma(dpl[3], t3, fma(dpl[2], t2, t1)));
          if (k == 0) {
            A = wx[0] * g;
            B = dwx[0] * g;
            C = wx[0] * gp;
          } else {
            A = fma(wx[k], g, A);
            B = fma(dwx[k], g, B);
            C = fma(wx[k], gp, C);
          }
        }
        F[e] = fma(wyj, A, F[e]);
        DxF[e] = fma(wyj, B, DxF[e]);
        DyF[e] = fma(dwyj, A, DyF[e]);
        DpF[e] = fma(wyj, C, DpF[e]);
      }
    }
    return;
  }
  // METHOD 3, 16-point bicubic (:425-481) as a tensor product of 4-point
  // Lagrange weights
  double wx[4], wy[4], dwx[4], dwy[4];
  lagrange4(px, wx, DERIV ? dwx : nullptr);
  lagrange4(py, wy, DERIV ? dwy : nullptr);
  double W[16], Wx[16], Wy[16];
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      W[4 * j + k] = wx[k] * wy[j];
      if (DERIV) {
        Wx[4 * j + k] = dwx[k] * wy[j] / cell.dx;
        Wy[4 * j + k] = wx[k] * dwy[j] / cell.dy;
      }
    }
#pragma unroll
  for (int th = 0; th < NTHETA; th++) {
    double I[NE], Ix[NE], Iy[NE];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const double *Tn = Tb + ((long long)j * nx + k) * NTHETA * NE + th * NE;
#pragma unroll
        for (int e = 0; e < NE; e++) {
          double tv = __ldg(Tn + e);
          if (j == 0 && k == 0) {
            I[e] = W[0] * tv;
            if (DERIV) {
              Ix[e] = Wx[0] * tv;
              Iy[e] = Wy[0] * tv;
            }
          } else {
            I[e] = fma(W[4 * j + k], tv, I[e]);
            if (DERIV) {
              Ix[e] = fma(Wx[4 * j + k], tv, Ix[e]);
              Iy[e] = fma(Wy[4 * j + k], tv, Iy[e]);
            }
          }
        }
      }
#pragma unroll
    for (int e = 0; e < NE; e++) {
      F[e] = fma(pl[th], I[e], F[e]);
      if (DERIV) {
        DpF[e] = fma(dpl[th], I[e], DpF[e]);
        DxF[e] = fma(pl[th], Ix[e], DxF[e]);
        DyF[e] = fma(pl[th], Iy[e], DyF[e]);
      }
    }
  }
}

// ===========================================================================
// 2c forces: Dassemble_S, Dassemble_T, Dassemble_vna_2c
// (k.DASSEMBLERS/M_Dassemble_2c_Harris.f90:96-869).  One warp per atom, one
// lane per pair.  Produces per pair: the kinetic and Pulay contractions
// sum rho.dT and sum cape.dS (build_forces :234-301, :473-537), vna_ontop
// and vna_atom; optionally the dS, dT Dblocks.
// ===========================================================================
struct CtxD2c {
  Ctx2c b;
  const double *rho, *cape;
  double *dS, *dT;        // optional Dblocks
  double *sumT, *sumS;    // per pair 3-vectors
  double *ontop, *atomf;  // per pair 3-vectors
  bool keep;
  double *dogs_ps;        // DOGS: 8 rho-weighted sums per pair for the 3c pass
};

// Dsmoother (b.FUNCTIONS/Dsmoother.f90:102-135), the scaler = 1 branch
__device__ __forceinline__ double dsmoother(double r, double rend, double x) {
  double rbegin = x * rend;
  if (r > rend || r < rbegin) return 0.0;
  double ratio = (r - rbegin) / (rend - rbegin);
  return -2.0 * (1.0 - ratio * ratio) * (2.0 * ratio) / (rend - rbegin);
}

// value and x-derivative of one 2c cell (getDMEs_Fdata_2c, :446-600)
template <int NE>
__device__ __forceinline__ void interp2c_d(const double *__restrict__ tab, const Cell2cDev &cell, double z, bool tiny,
                                           double *v, double *dv, unsigned *status) {
  if (z > cell.xmax * (1.0 + 1.0e-5)) atomicOr(status, DEVERR_XLARGE);
  if (tiny) {
#pragma unroll
    for (int e = 0; e < NE; e++) {
      v[e] = __ldg(tab + cell.off + e);
      dv[e] = 0.0;
    }
    return;
  }
  int i0;
  double w[7], dw[7];
  lagrange7(z, cell, i0, w, dw);
  const double *F = tab + cell.off + (long long)i0 * NE;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    double f = __ldg(F + e);
    v[e] = w[0] * f;
    dv[e] = dw[0] * f;
  }
#pragma unroll
  for (int s = 1; s < 7; s++)
#pragma unroll
    for (int e = 0; e < NE; e++) {
      double f = __ldg(F + s * NE + e);
      v[e] = fma(w[s], f, v[e]);
      dv[e] = fma(dw[s], f, dv[e]);
    }
}

// vdsm(:,mu,nu) = -eta(:) dsm(mu,nu) when z > 1e-3
// (k.DASSEMBLERS/M_Dassemble_2c_Harris.f90:237-241)
template <int NE>
__device__ __forceinline__ void vec2c(double z, const double *eta, const double *dv, double *vd) {
  bool on = z > 1.0e-3;
#pragma unroll
  for (int e = 0; e < NE; e++)
#pragma unroll
    for (int k = 0; k < 3; k++) vd[k + 3 * e] = on ? -eta[k] * dv[e] : 0.0;
}

// sum_{mu,nu} blk(mu,nu) d/dr_q [L M R^T](mu,nu) for M given by v (values)
// and vd (its Cartesian derivatives) at the ME positions, from the
// molecular-frame density G of the block (mol_rho)
template <int PA, int PB, int K>
__device__ __forceinline__ void contract_g(const MolRho<PA, PB, K> &G, const double *v, const double *vd,
                                           double out[3]) {
  constexpr int NE = Plan<PA, PB, K>::m.n;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    double s = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
      s = fma(v[e], G.H[q][e], s);
      s = fma(vd[q + 3 * e], G.G[e], s);
    }
    out[q] = s;
  }
}

template <int PA, int PB, int K, bool HASD>
__device__ __forceinline__ void contract(const RotM &R, const DRotM &D, const double *blk, const double *v,
                                         const double *vd, double out[3]) {
  MolRho<PA, PB, K> G;
  mol_rho<PA, PB, K>(R, D, blk, G);
  contract_g<PA, PB, K>(G, v, vd, out);
}

// The same contraction (s and p shells) through the rotation rates of the
// frame: Gf = L^T blk L over the whole block (mol_G_full), W[pair][q] the
// rates W^xy, W^yz, W^xz of component q (frame_rates_2c):
// out_q = sum_pair W[pair][q] tau^pair + sum_e vd_q(e) G(e)
template <int PA, int PB, int K>
__device__ __forceinline__ void contract_rates(const double *Gf, const double (*W)[3], const double *v,
                                               const double *vd, double out[3]) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA;
  double tau[3];
  mol_tau<PA, PB, K>(Gf, v, tau);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    double s = fma(W[2][q], tau[2], fma(W[1][q], tau[1], W[0][q] * tau[0]));
    sfor<PL::m.n>([&](auto E) {
      constexpr int e = decltype(E)::value;
      constexpr int at = PL::m.mu[e] + NA * PL::m.nu[e];
      s = fma(vd[q + 3 * e], Gf[at], s);
    });
    out[q] = s;
  }
}

inline Ctx2c make2c(const AsmArgs &a) {
  Ctx2c c;
  c.N = a.N;
  c.P = a.P;
  c.pair_owner = a.pair_owner;
  c.ratom = a.ratom;
  c.sid = a.sid;
  c.isp = a.isp;
  c.fd = a.fd;
  c.table2c = a.table2c;
  c.xl = a.xl;
  c.pair_off = a.pair_off;
  c.neigh_j = a.neigh_j;
  c.neigh_b = a.neigh_b;
  c.neigh_self = a.neigh_self;
  c.blk_off = a.blk_off;
  c.S = a.S;
  c.T = a.T;
  c.vb = a.vb;
  c.vbo = a.vbo;
  c.status = a.status;
  c.dogs = a.dogs;
  c.dq = a.dq;
  c.dip = a.dip;
  return c;
}

inline Ctx3c make3c(const AsmArgs &a) {
  Ctx3c c;
  c.N = a.N;
  c.T = a.ntrip;
  c.ratom = a.ratom;
  c.sid = a.sid;
  c.isp = a.isp;
  c.fd = a.fd;
  c.table3c = a.table3c;
  c.lin = a.lin;
  c.gxy = a.gxy;
  c.xl = a.xl;
  c.trip_alpha = a.trip_alpha;
  c.ci_j = a.ci_j;
  c.ci_b = a.ci_b;
  c.cj_j = a.cj_j;
  c.cj_b = a.cj_b;
  c.tdst = a.tdst;
  c.tperm = a.tperm;
  c.blk_off = a.blk_off;
  c.vb = a.vb;
  c.rho = a.rho;
  c.f3naa = a.f3naa;
  c.f3nab = a.f3nab;
  c.f3nac = a.f3nac;
  c.table3c_df = reinterpret_cast<const df *>(a.table3c_df);
  c.rho_df = reinterpret_cast<const df *>(a.rho_df);
  c.mlpF = a.mlpF;
  c.dogs = a.dogs;
  c.dq = a.dq;
  c.S = a.S;
  c.dip = a.dip;
  c.dogs_ps = a.dogs_ps;
  return c;
}

}  // namespace fb
