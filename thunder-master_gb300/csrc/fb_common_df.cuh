// fb_common_df.cuh -- double-float three-center interpolation
// (getMEs_Fdata_3c / getDMEs_Fdata_3c, e.FDATA/M_Fdata_3c.f90:293-846) on
// the FP32 pipe.  The grid cell, the stencil origin and the gradient switch
// are decided in FP64 exactly as the reference does; the Legendre sum of the
// bicubic (or three-point linear) interpolations runs in df.
#pragma once
#include "fb_common.cuh"
#include "fb_device_df.cuh"

namespace fb {

// reciprocal of a df by one Newton step from the float reciprocal
__device__ __forceinline__ df df_rcp(df a) {
  float r = __frcp_rn(a.h);
  df e = df_one() - a * r;  // 1 - a r, small
  return df_make(r) + e * r;
}

// P_eq2 (include/constants.h:4) as hi + lo floats
__device__ __forceinline__ df peq2_df() { return df_make(14.39975f, 2.4414064e-07f); }

__device__ __forceinline__ df cross_df(const df *a, const df *b, int k) {
  return k == 0 ? a[1] * b[2] - a[2] * b[1] : (k == 1 ? a[2] * b[0] - a[0] * b[2] : a[0] * b[1] - a[1] * b[0]);
}

// Triplet set-up (M_assemble_3c_Harris.f90:160-189) with FP64 kept where the
// reference's integer decisions depend on it -- the bond length z and the
// distance x that select the table cell -- and everything else (unit
// vectors, cos(theta), the local frame) in df.
struct GeomDF {
  int ia, iat, jat;
  double x, z;
  df u[3];    // r21 = r2 - r1
  df v[3];    // rna - r1
  df sig[3];  // sighat
  df rh[3];   // rhat
  df cost, iz, ix;
  df e[3][3];  // epsilon(rhat, sighat)
  bool estd;   // e has its y axis along sighat x rhat (not the collinear fallback)
};

// FP64 part of the set-up: what the table cell depends on, and the exact
// difference vectors the df quantities are formed from
struct GeomFP64 {
  int ia, iat, jat;
  double x, z;
  double r21[3], rn[3], v[3];
};

__device__ __forceinline__ void trip_geom_fp64(const Ctx3c &c, int t, GeomFP64 &h) {
  h.ia = c.trip_alpha[t];
  h.iat = c.ci_j[t];
  h.jat = c.cj_j[t];
  int ib = c.ci_b[t], jb = c.cj_b[t];
  const double *xl = c.xl + (long long)c.sid[h.ia] * XL_STRIDE;
  double r1[3], r2[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r1[k] = __dadd_rn(c.ratom[3 * h.iat + k], xl[3 * ib + k]);
    r2[k] = __dadd_rn(c.ratom[3 * h.jat + k], xl[3 * jb + k]);
    h.r21[k] = __dsub_rn(r2[k], r1[k]);
    h.rn[k] = __dsub_rn(c.ratom[3 * h.ia + k], __dadd_rn(r1[k], h.r21[k] * 0.5));
    h.v[k] = c.ratom[3 * h.ia + k] - r1[k];
  }
  h.z = dist_rn(r1, r2);
  h.x = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(h.rn[0], h.rn[0]), __dmul_rn(h.rn[1], h.rn[1])),
                             __dmul_rn(h.rn[2], h.rn[2])));
}

// cos(theta) alone (for the interpolation), in df
__device__ __forceinline__ df trip_cost_df(const GeomFP64 &h) {
  if (h.x < 1.0e-05) return df_zero();
  df s = df_zero();
#pragma unroll
  for (int k = 0; k < 3; k++) s = s + df_from(h.r21[k]) * df_from(h.rn[k]);
  if (h.z < 1.0e-05) return df_from(h.rn[2]) * df_rcp(df_from(h.x));
  return s * (df_rcp(df_from(h.z)) * df_rcp(df_from(h.x)));
}

__device__ __forceinline__ void trip_geom_df_from(const GeomFP64 &h, GeomDF &g) {
  g.ia = h.ia;
  g.iat = h.iat;
  g.jat = h.jat;
  g.x = h.x;
  g.z = h.z;
  df rnd[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    g.u[k] = df_from(h.r21[k]);
    g.v[k] = df_from(h.v[k]);
    rnd[k] = df_from(h.rn[k]);
  }
  if (g.z < 1.0e-05) {
    g.sig[0] = df_zero();
    g.sig[1] = df_zero();
    g.sig[2] = df_one();
    g.iz = df_zero();
  } else {
    g.iz = df_rcp(df_from(g.z));
#pragma unroll
    for (int k = 0; k < 3; k++) g.sig[k] = g.u[k] * g.iz;
  }
  bool hasr = g.x >= 1.0e-05;
  if (hasr) {
    g.ix = df_rcp(df_from(g.x));
#pragma unroll
    for (int k = 0; k < 3; k++) g.rh[k] = rnd[k] * g.ix;
  } else {
    g.ix = df_zero();
    g.rh[0] = g.rh[1] = g.rh[2] = df_zero();
  }
  g.cost = g.sig[0] * g.rh[0] + g.sig[1] * g.rh[1] + g.sig[2] * g.rh[2];
  // epsilon_function(rhat, sighat) (b.FUNCTIONS/epsilon.f90:73-202); both
  // arguments are unit vectors (or rhat = 0), so their normalisations are
  // the identity to within a few ulps and are omitted
  df yp[3];
  float ypm2 = 0.0f;
  if (hasr) {
#pragma unroll
    for (int k = 0; k < 3; k++) yp[k] = cross_df(g.sig, g.rh, k);
    ypm2 = (yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]).h;
  }
  g.estd = hasr && !(ypm2 < 1.0e-8f);
  if (!g.estd) {
    // colinear fallback (:148-168), first non-zero component of zphat
    if (fabsf(g.sig[0].h) > 1.0e-4f) {
      yp[0] = -(g.sig[1] + g.sig[2]) * df_rcp(g.sig[0]);
      yp[1] = df_one();
      yp[2] = df_one();
    } else if (fabsf(g.sig[1].h) > 1.0e-4f) {
      yp[0] = df_one();
      yp[1] = -(g.sig[0] + g.sig[2]) * df_rcp(g.sig[1]);
      yp[2] = df_one();
    } else {
      yp[0] = df_one();
      yp[1] = df_one();
      yp[2] = -(g.sig[0] + g.sig[1]) * df_rcp(g.sig[2]);
    }
  }
  df iy = df_rcp(df_sqrt(yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]));
#pragma unroll
  for (int k = 0; k < 3; k++) yp[k] = yp[k] * iy;
  df xp[3];
#pragma unroll
  for (int k = 0; k < 3; k++) xp[k] = cross_df(yp, g.sig, k);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    g.e[k][0] = xp[k];
    g.e[k][1] = yp[k];
    g.e[k][2] = g.sig[k];
  }
}

__device__ __forceinline__ void trip_geom_df(const Ctx3c &c, int t, GeomDF &g) {
  GeomFP64 h;
  trip_geom_fp64(c, t, h);
  trip_geom_df_from(h, g);
}

__device__ __forceinline__ df sel3(const df *a, int k) {
  df r = a[0];
  r = k == 1 ? a[1] : r;
  r = k == 2 ? a[2] : r;
  return r;
}

// element j of a 4-array by selects (keeps the array in registers when j
// is a loop variable)
__device__ __forceinline__ df sel4(const df *a, int j) {
  df r = a[0];
  r = j == 1 ? a[1] : r;
  r = j == 2 ? a[2] : r;
  r = j == 3 ? a[3] : r;
  return r;
}

// element th of a 5-array by selects (keeps the array in registers when th
// is a loop variable)
__device__ __forceinline__ df sel5(const df *a, int th) {
  df r = a[0];
  r = th == 1 ? a[1] : r;
  r = th == 2 ? a[2] : r;
  r = th == 3 ? a[3] : r;
  r = th == 4 ? a[4] : r;
  return r;
}

template <int NE, bool DERIV>
__device__ __forceinline__ void interp3c_df(const Ctx3c &c, const Cell3cDev &cell, double x, double y, df cost,
                                            df *F, df *DpF, df *DxF, df *DyF) {
  // Legendre P_0..P_4 and their derivatives (:348-354, :625-629)
  df c2 = cost * cost;
  df pl[5], dpl[5];
  pl[0] = df_one();
  pl[1] = cost;
  pl[2] = (c2 * 3.0f - df_one()) * 0.5f;
  pl[3] = (cost * (c2 * 5.0f - df_make(3.0f))) * 0.5f;
  pl[4] = (df_make(3.0f) - c2 * (df_make(30.0f) - c2 * 35.0f)) * 0.125f;
  if (DERIV) {
    dpl[0] = df_zero();
    dpl[1] = df_one();
    dpl[2] = cost * 3.0f;
    dpl[3] = (c2 * 15.0f - df_make(3.0f)) * 0.5f;
    dpl[4] = (cost * (c2 * 35.0f - df_make(15.0f))) * 0.5f;
  }
  // grid cell and offsets, FP64 as the reference (:367-379)
  double qx = __ddiv_rn(x, cell.dx), qy = __ddiv_rn(y, cell.dy);
  int ix = (int)qx + 1;
  int iy = (int)qy + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > cell.nx - 2) ix = cell.nx - 2;
  if (iy > cell.ny - 2) iy = cell.ny - 2;
  df px = df_from(qx - ix + 1.0);
  df py = df_from(qy - iy + 1.0);
  int nx = cell.nx;
  long long node0 = (long long)(iy - 1) * nx + (ix - 1);
  const df *tab = c.table3c_df + cell.off;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    F[e] = df_zero();
    if (DERIV) DpF[e] = DxF[e] = DyF[e] = df_zero();
  }
  if (c.lin[cell.node_off + node0]) {
    // METHOD 1, three-point linear (:406-410, :684-691)
    df gx = df_from(c.gxy[2 * (cell.node_off + node0)]), gy = df_from(c.gxy[2 * (cell.node_off + node0) + 1]);
    df w00 = (df_one() - px) - py;
    const df *T00 = tab + node0 * NTHETA * NE;
    const df *T10 = tab + (node0 + 1) * NTHETA * NE;
    const df *T01 = tab + (node0 + nx) * NTHETA * NE;
#pragma unroll
    for (int th = 0; th < NTHETA; th++)
#pragma unroll
      for (int e = 0; e < NE; e++) {
        dacc a;
        dacc_first(a, w00, T00[th * NE + e]);
        dacc_add(a, px, T10[th * NE + e]);
        dacc_add(a, py, T01[th * NE + e]);
        df I = dacc_val(a);
        F[e] = F[e] + pl[th] * I;
        if (DERIV) {
          DpF[e] = DpF[e] + dpl[th] * I;
          DxF[e] = DxF[e] + pl[th] * gx;
          DyF[e] = DyF[e] + pl[th] * gy;
        }
      }
    return;
  }
  // METHOD 3, 16-point bicubic as a tensor product of Lagrange weights
  df wx[4], wy[4], dwx[4], dwy[4];
  lagrange4_df(px, wx, DERIV ? dwx : nullptr);
  lagrange4_df(py, wy, DERIV ? dwy : nullptr);
  if (DERIV) {
    df idx = df_make(cell.idx_h, cell.idx_l), idy = df_make(cell.idy_h, cell.idy_l);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      dwx[k] = dwx[k] * idx;
      dwy[k] = dwy[k] * idy;
    }
  }
  const df *Tb = tab + (node0 - nx - 1) * NTHETA * NE;
  if constexpr (DERIV) {
    // The interpolation is linear in the table values, so the Legendre sums
    // come first at each of the 16 stencil nodes, g = sum_th P_th T_th and
    // gp = sum_th P'_th T_th (dacc sums, the P_0 = 1 and P'_1 = 1 terms as
    // their starting values), and the stencil weights then accumulate g
    // (value, d/dx, d/dy) and gp (d/dcos) in four dacc sums per element:
    // 4 + 3 + 4 accumulations per node and element instead of the 15 of the
    // per-theta contraction.  The sums differ from the reference's order by
    // rounding only.  Stencil rows and columns are rolled
    // (instruction-cache footprint), the matrix elements unrolled.
    dacc aF[NE], aDp[NE], aDx[NE], aDy[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) aF[e] = aDp[e] = aDx[e] = aDy[e] = dacc{0.0f, 0.0f};
#pragma unroll 1
    for (int j = 0; j < 4; j++) {
      const df wyj = sel4(wy, j), dwyj = sel4(dwy, j);
#pragma unroll 1
      for (int k = 0; k < 4; k++) {
        const df wxk = sel4(wx, k), dwxk = sel4(dwx, k);
        const df W = wxk * wyj, Wx = dwxk * wyj, Wy = wxk * dwyj;
        const df *Tn = Tb + ((long long)j * nx + k) * NTHETA * NE;
#pragma unroll
        for (int e = 0; e < NE; e++) {
          const df t0 = Tn[e], t1 = Tn[NE + e], t2 = Tn[2 * NE + e], t3 = Tn[3 * NE + e], t4 = Tn[4 * NE + e];
          dacc g{t0.h, t0.l}, gp{t1.h, t1.l};
          dacc_add(g, pl[1], t1);
          dacc_add(g, pl[2], t2);
          dacc_add(g, pl[3], t3);
          dacc_add(g, pl[4], t4);
          dacc_add(gp, dpl[2], t2);
          dacc_add(gp, dpl[3], t3);
          dacc_add(gp, dpl[4], t4);
          const df gv = dacc_val(g), gpv = dacc_val(gp);
          dacc_add(aF[e], W, gv);
          dacc_add(aDx[e], Wx, gv);
          dacc_add(aDy[e], Wy, gv);
          dacc_add(aDp[e], W, gpv);
        }
      }
    }
#pragma unroll
    for (int e = 0; e < NE; e++) {
      F[e] = dacc_val(aF[e]);
      DpF[e] = dacc_val(aDp[e]);
      DxF[e] = dacc_val(aDx[e]);
      DyF[e] = dacc_val(aDy[e]);
    }
  } else {
    // value only: the per-theta contraction I_theta -> F; the theta loop is
    // kept rolled (instruction-cache footprint, registers)
#pragma unroll 1
    for (int th = 0; th < NTHETA; th++) {
      const df plt = sel5(pl, th);
      dacc I[NE];
      // stencil rows rolled (instruction-cache footprint)
#pragma unroll
      for (int e = 0; e < NE; e++) I[e] = dacc{0.0f, 0.0f};
#pragma unroll 1
      for (int j = 0; j < 4; j++) {
        const df wyj = sel4(wy, j);
        const df *Tr = Tb + (long long)j * nx * NTHETA * NE + th * NE;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          df w = wx[k] * wyj;
#pragma unroll
          for (int e = 0; e < NE; e++) dacc_add(I[e], w, Tr[k * NTHETA * NE + e]);
        }
      }
#pragma unroll
      for (int e = 0; e < NE; e++) F[e] = F[e] + plt * dacc_val(I[e]);
    }
  }
}

// ---------------------------------------------------------------------------
// three-center force helpers shared by the df force kernels
// ---------------------------------------------------------------------------
// The scalars of Depsilon_3c (b.FUNCTIONS/Depsilon_3c.f90:49-189) in df,
// evaluated with the origin at atom 1.  Its expressions are translation
// invariant (the three coefficients of each bracket sum to zero), and
// relative coordinates avoid the cancellation of absolute squared norms:
// u = r2 - r1, v = ratm - r1.
struct DepsPre {
  df ic, A1, A2, B1, B2;
  df vu[3];
  bool zero;  // sighat x rnabc below 1e-3: all derivatives vanish
};

__device__ __forceinline__ void depsilon_pre_df(const df u[3], const df v[3], DepsPre &p) {
  df rn[3] = {v[0] - u[0] * 0.5f, v[1] - u[1] * 0.5f, v[2] - u[2] * 0.5f};
  df c0 = u[1] * rn[2] - u[2] * rn[1];
  df c1 = u[2] * rn[0] - u[0] * rn[2];
  df c2 = u[0] * rn[1] - u[1] * rn[0];
  df cm = df_sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  p.zero = cm.h < 1.0e-3f;
  p.ic = p.zero ? df_zero() : df_rcp(cm);
#pragma unroll
  for (int k = 0; k < 3; k++) p.vu[k] = v[k] - u[k];
  p.A1 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  p.A2 = -(u[0] * v[0] + u[1] * v[1] + u[2] * v[2]);
  p.B1 = u[0] * p.vu[0] + u[1] * p.vu[1] + u[2] * p.vu[2];
  p.B2 = -(v[0] * p.vu[0] + v[1] * p.vu[1] + v[2] * p.vu[2]);
}

// Molecular-frame density of a triplet's block: Gf = L^T rho L over the
// whole block and G at the ME positions
template <int PA, int PB>
__device__ __forceinline__ void mol_density_df(const RotDF &R, const df *rb, df *Gf, df *G) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA;
  mol_G_full_df<PA, PB>(R, rb, Gf);
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int at = PL::m.mu[e] + NA * PL::m.nu[e];
    G[e] = Gf[at];
  });
}

// The frame-derivative terms of a triplet's three-center forces (s and p
// shells) in df: hA_c = sum_e M_e H_c(e) for d/dratm, hB_c for d/dr1, H the
// Dtwister derivative contracted with the density, through the rotation
// rates of the frame (frame_rates_3c and frame_extra_3c in fb_device.cuh),
// with the origin at atom 1: u = r21, v = ratm - r1, ratm - r2 = v - u.
template <int PA, int PB>
__device__ __forceinline__ void frame_terms_3c_df(const GeomDF &g, const df *Gf, const df *M, df hA[3], df hB[3]) {
  df tau[3];
  mol_tau_df<PA, PB>(Gf, M, tau);
  DepsPre pre;
  depsilon_pre_df(g.u, g.v, pre);
  const df izr = pre.zero ? df_zero() : g.iz;
  df ex[3], ey[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ex[k] = g.e[k][0];
    ey[k] = g.e[k][1];
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    df axy = pre.ic * cross_df(ex, g.u, k);
    df bxy = pre.ic * cross_df(ex, pre.vu, k);
    hA[k] = axy * tau[0];
    hB[k] = bxy * tau[0] - (izr * ey[k]) * tau[1] - (izr * ex[k]) * tau[2];
  }
  if (!g.estd) {
    // epsilon's collinear fallback frame: V = A1 v + A2 u, V' = B1 v + B2 u
    df kd, kzy;
    mol_kappa_extra_df<PA, PB>(Gf, M, kd, kzy);
    df ez[3] = {g.e[0][2], g.e[1][2], g.e[2][2]};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      df V = pre.A1 * g.v[k] + pre.A2 * g.u[k];
      df Vb = pre.B1 * g.v[k] + pre.B2 * g.u[k];
      df psiA = pre.ic * (cross_df(ey, g.u, k) - pre.ic * V);
      df psiB = pre.ic * (cross_df(ey, pre.vu, k) - pre.ic * Vb);
      df chiB = pre.ic * cross_df(ez, pre.vu, k);
      hA[k] = hA[k] + psiA * kd;
      hB[k] = hB[k] + psiB * kd + (chiB - izr * ey[k]) * kzy;
    }
  }
}

}  // namespace fb
