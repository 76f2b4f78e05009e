// fb_dasm3c_df.cu -- sm_103a three-center force derivatives
// (Dassemble_vna_3c, k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136-408) with
// the table contractions, frame derivatives and density contraction in
// double-float on the FP32 pipe.
#include "fb_common_df.cuh"

namespace fb {

// Depsilon_3c (b.FUNCTIONS/Depsilon_3c.f90:49-189) in df, evaluated with the
// origin at atom 1.  Its expressions are translation invariant (the three
// coefficients of each bracket sum to zero), and relative coordinates avoid
// the cancellation of absolute squared norms: u = r2 - r1, v = ratm - r1.
// The quantities shared by the three Cartesian components:
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

// component ix of deps/dratm (dA[imu][k]) and deps/dr1 (dB[imu][k])
__device__ __forceinline__ void depsilon_comp_df(int ix, const df u[3], const df v[3], df iz, const df e[3][3],
                                                 const DepsPre &p, df dA[3][3], df dB[3][3]) {
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) dA[a][b] = dB[a][b] = df_zero();
  if (p.zero) return;
#pragma unroll
  for (int imu = 0; imu < 3; imu++) {
    df sa = df_zero(), sb = df_zero();
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double lv = levi(ix, imu, k);
      if (lv > 0.0) {
        sa = sa + u[k];
        sb = sb + p.vu[k];
      } else if (lv < 0.0) {
        sa = sa - u[k];
        sb = sb - p.vu[k];
      }
    }
    df ei = e[imu][1] * p.ic;
    dA[imu][1] = p.ic * (sa - ei * (p.A1 * v[ix] + p.A2 * u[ix]));
    dB[imu][1] = p.ic * (sb - ei * (p.B1 * v[ix] + p.B2 * u[ix]));
    df t = e[imu][2] * e[ix][2];
    dB[imu][2] = iz * ((ix == imu) ? t - df_one() : t);
  }
  dA[0][0] = e[2][2] * dA[1][1] - e[1][2] * dA[2][1];
  dA[1][0] = e[0][2] * dA[2][1] - e[2][2] * dA[0][1];
  dA[2][0] = e[1][2] * dA[0][1] - e[0][2] * dA[1][1];
  dB[0][0] = e[2][2] * dB[1][1] - e[2][1] * dB[1][2] - e[1][2] * dB[2][1] + e[1][1] * dB[2][2];
  dB[1][0] = e[0][2] * dB[2][1] - e[0][1] * dB[2][2] - e[2][2] * dB[0][1] + e[2][1] * dB[0][2];
  dB[2][0] = e[1][2] * dB[0][1] - e[1][1] * dB[0][2] - e[0][2] * dB[1][1] + e[0][1] * dB[1][2];
}

// sum_e M_e H(e) for one Cartesian component, H = dL^T rho R + L^T rho dR at
// the ME positions (the dL M R^T and L M dR^T terms of Dmatrix,
// M_Drotations.f90:456-471, contracted with rho); dP is that component of
// the p-shell rotation derivative (Dtwister, :236-249): dP[a][b] =
// deps(perm a, perm b)
template <int PA, int PB>
__device__ __forceinline__ df mol_HM_df(const RotDF &R, const df dP[3][3], const df *rho, const df *rR,
                                        const df *M) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA;
  df acc = df_zero();
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
    df h = df_zero();
    if constexpr (sa > 0) {
      sfor<3>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        h = h + dP[k][ma] * rR[(oa + k) + NA * b];
      });
    }
    if constexpr (sb > 0) {
      sfor<2 * sa + 1>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        df t = df_zero();
        sfor<3>([&](auto NU) {
          constexpr int q = decltype(NU)::value;
          t = t + rho[(oa + k) + NA * (ob + q)] * dP[q][mb];
        });
        h = h + ((sa == 0) ? t : Lrot_df<sa>(R, k, ma) * t);
      });
    }
    acc = acc + M[e] * h;
  });
  return acc;
}

// MLP: F and its cos / x / y derivatives come from the MLP-3c results of
// list position i instead of the tables
template <int PA, int PB, bool MLP>
__device__ void trip_3c_force_df(const Ctx3c &c, int t, int i) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  // interpolation first: it needs only x, z and cos(theta)
  GeomFP64 h;
  trip_geom_fp64(c, t, h);
  const int ia = h.ia, iat = h.iat, jat = h.jat;
  df F[NE], DpF[NE], DxF[NE], DyF[NE];
  if constexpr (MLP) {
    const float *m = c.mlpF + (long long)i * 4 * MLP_ME_STRIDE;
#pragma unroll
    for (int e = 0; e < NE; e++) {
      F[e] = df_make(m[e]);
      DpF[e] = df_make(m[MLP_ME_STRIDE + e]);
      DxF[e] = df_make(m[2 * MLP_ME_STRIDE + e]);
      DyF[e] = df_make(m[3 * MLP_ME_STRIDE + e]);
    }
  } else {
    const Cell3cDev &cell = c.fd->c3[c.isp[iat]][c.isp[jat]][c.isp[ia]];
    interp3c_df<NE, true>(c, cell, h.x, h.z, trip_cost_df(h), F, DpF, DxF, DyF);
  }
  GeomDF g;
  trip_geom_df_from(h, g);
  const df cost = g.cost, iz = g.iz;
  // mvalue = 1 channels carry sin(theta) (M_Fdata_3c.f90:822-832)
  df s2 = df_one() - cost * cost;
  df sint = df_sqrt(s2.h > 1.0e-5f ? s2 : df_make(1.0e-5f, 2.5262125e-13f));
  df isint = df_rcp(sint);
  sfor<NE>([&](auto E) {
    constexpr int ee = decltype(E)::value;
    if constexpr (PL::m.mv[ee] == 1) {
      DpF[ee] = DpF[ee] * sint - cost * F[ee] * isint;
      F[ee] = F[ee] * sint;
      DxF[ee] = DxF[ee] * sint;
      DyF[ee] = DyF[ee] * sint;
    }
  });
  RotDF R;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = g.e[pperm(a)][pperm(b)];
  const df *rho = c.rho_df + c.blk_off[c.tdst[t]];
  df rb[NA * NB], rR[NA * NB], G[NE];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = rho[q];
  mol_rR_df<PA, PB, K3C>(R, rb, rR);
  mol_G_df<PA, PB, K3C>(R, rR, G);
  // the f3naMa / f3naMb terms (:334-344) enter only through
  // sum_e Ma(q,e) G(e) = rhat_q Sx + amt_q Sp and
  // sum_e Mb(q,e) G(e) = bmt_q Sp - sighat_q Sy - (rhat_q Sx + amt_q Sp)/2
  df Sx = df_zero(), Sy = df_zero(), Sp = df_zero();
#pragma unroll
  for (int e = 0; e < NE; e++) {
    Sx = Sx + DxF[e] * G[e];
    Sy = Sy + DyF[e] * G[e];
    Sp = Sp + DpF[e] * G[e];
  }
  DepsPre pre;
  depsilon_pre_df(g.u, g.v, pre);
  const df peq2 = peq2_df();
  double fa[3], fb[3];
#pragma unroll 1
  for (int q = 0; q < 3; q++) {
    df dA[3][3], dB[3][3];
    depsilon_comp_df(q, g.u, g.v, iz, g.e, pre, dA, dB);
    df dPA[3][3], dPB[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) {
        dPA[a][b] = dA[pperm(a)][pperm(b)];
        dPB[a][b] = dB[pperm(a)][pperm(b)];
      }
    df amt = (g.x > 1.0e-5) ? (sel3(g.sig, q) - cost * sel3(g.rh, q)) * g.ix : df_zero();
    df bmt = (cost * sel3(g.sig, q) - sel3(g.rh, q)) * iz;
    df ga = sel3(g.rh, q) * Sx + amt * Sp;
    df sa = mol_HM_df<PA, PB>(R, dPA, rb, rR, F) + ga;
    df sb = mol_HM_df<PA, PB>(R, dPB, rb, rR, F) + ((bmt * Sp - sel3(g.sig, q) * Sy) - ga * 0.5f);
    double va = -df_to(sa * peq2), vb = -df_to(sb * peq2);
    fa[0] = q == 0 ? va : fa[0];
    fa[1] = q == 1 ? va : fa[1];
    fa[2] = q == 2 ? va : fa[2];
    fb[0] = q == 0 ? vb : fb[0];
    fb[1] = q == 1 ? vb : fb[1];
    fb[2] = q == 2 ? vb : fb[2];
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(c.f3naa + 3 * ia + q, fa[q]);
    atomicAdd(c.f3nab + 3 * iat + q, fb[q]);
    atomicAdd(c.f3nac + 3 * jat + q, -fa[q] - fb[q]);
  }
}

template <bool MLP>
__global__ void __launch_bounds__(256) k_dassemble_3c_df(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    int i = t;
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    switch (pa * 3 + pb) {
      case PAT_SP * 3 + PAT_SP: trip_3c_force_df<PAT_SP, PAT_SP, MLP>(c, t, i); break;
      case PAT_SP * 3 + PAT_S: trip_3c_force_df<PAT_SP, PAT_S, MLP>(c, t, i); break;
      case PAT_S * 3 + PAT_SP: trip_3c_force_df<PAT_S, PAT_SP, MLP>(c, t, i); break;
      case PAT_S * 3 + PAT_S: trip_3c_force_df<PAT_S, PAT_S, MLP>(c, t, i); break;
      default: break;
    }
  });
}

int launch_dassemble_3c_df(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d3c, (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block, q);
  if (e) return e;
  k_dassemble_3c_df<false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dassemble_3c_mlp(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d3c, (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block, q);
  if (e) return e;
  k_dassemble_3c_df<true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
