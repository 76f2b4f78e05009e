// fb_vxc_df.cu -- sm_103a three-center McWEDA densities (assemble_rho_3c +
// assemble_rho_weighted_3c, j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90:
// 298-403, :645-741) with the table contraction and rotation in
// double-float on the FP32 pipe, as the Harris neutral-atom three-center
// kernel does.  The Qneutral-weighted sum over the shells of the third atom
// is taken in the molecular frame and rotated once.
#include "fb_common_df.cuh"
#include "fb_vxc.h"

namespace fb {

namespace {

// as qsum_fast of the FP64 kernels: the summed cells exist and the
// triplet's stencil node has one gradient switch for every sub-cell
__device__ __forceinline__ bool qsum_node_ok_df(const unsigned char *lin, const Cell3cDev &cell, double x, double y) {
  if (cell.off < 0) return false;
  int ix = (int)__ddiv_rn(x, cell.dx) + 1, iy = (int)__ddiv_rn(y, cell.dy) + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > cell.nx - 2) ix = cell.nx - 2;
  if (iy > cell.ny - 2) iy = cell.ny - 2;
  return lin[cell.node_off + (long long)(iy - 1) * cell.nx + (ix - 1)] != 2;
}
__device__ __forceinline__ bool qsum_fast_df(const Ctx3c &c, int in1, int in2, int in3, double x, double y) {
  const FdataDev &fd = *c.fd;
  return qsum_node_ok_df(c.lin, fd.c3rhoq[in1][in2][in3][0], x, y) &&
         qsum_node_ok_df(c.lin, fd.c3rhoq[in1][in2][in3][1], x, y);
}

template <int PA, int PB, bool QSUM>
__device__ __forceinline__ void trip_rho3c_df(const Ctx3c &c, const VxcArgs &v, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB), NS = SA * SB;
  GeomDF g;
  trip_geom_df(c, t, g);
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[g.iat], in2 = c.isp[g.jat], indna = c.isp[g.ia];
  if (qsum_fast_df(c, in1, in2, indna, g.x, g.z) != QSUM) return;
  int nk = fd.sp[indna].nssh;
  const double *qk = fd.sp[indna].qn;
  df m[NE];
  if constexpr (QSUM) {
    interp3c_df<NE, false>(c, fd.c3rhoq[in1][in2][indna][0], g.x, g.z, g.cost, m, nullptr, nullptr, nullptr);
  } else {
    df F[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) m[e] = df_zero();
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c_df<NE, false>(c, fd.c3rho[in1][in2][indna][0][isorp], g.x, g.z, g.cost, F, nullptr, nullptr,
                             nullptr);
      df Q = df_from(qk[isorp]);
#pragma unroll
      for (int e = 0; e < NE; e++) m[e] = m[e] + F[e] * Q;
    }
  }
  // sint = sqrt(max(1e-5, 1 - cost^2)) (M_Fdata_3c.f90:349) for mvalue = 1
  df s2 = df_one() - g.cost * g.cost;
  df sint = df_sqrt(s2.h > 1.0e-5f ? s2 : df_make(1.0e-5f, 2.5262125e-13f));
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    if constexpr (PL::m.mv[e] == 1) m[e] = m[e] * sint;
  });
  RotDF R;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = g.e[pperm(a)][pperm(b)];
  df X[NA * NB];
  rotate_plan_df<PA, PB, K3C>(R, m, X);
  int p = c.tdst[t];
  double *dst = v.rho_in + c.blk_off[p];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, df_to(X[q]));
  // shell level: no rotation, channel (a, b) at a * SB + b
  df ws[NS];
  if constexpr (QSUM) {
    interp3c_df<NS, false>(c, fd.c3rhoq[in1][in2][indna][1], g.x, g.z, g.cost, ws, nullptr, nullptr, nullptr);
  } else {
    df Fs[NS];
#pragma unroll
    for (int e = 0; e < NS; e++) ws[e] = df_zero();
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c_df<NS, false>(c, fd.c3rho[in1][in2][indna][1][isorp], g.x, g.z, g.cost, Fs, nullptr, nullptr,
                             nullptr);
      df Q = df_from(qk[isorp]);
#pragma unroll
      for (int e = 0; e < NS; e++) ws[e] = ws[e] + Fs[e] * Q;
    }
  }
  double *wd = v.wrho_in + (long long)VXC_WSH * p;
#pragma unroll
  for (int e = 0; e < NS; e++) atomicAdd(wd + (e / SB) + SA * (e % SB), df_to(ws[e]));
}

template <bool QSUM>
__global__ void __launch_bounds__(128) k_rho_3c_df(Ctx3c c, VxcArgs v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.T; i += gridDim.x * blockDim.x) {
    int t = c.tperm ? c.tperm[i] : i;
    int in1 = c.isp[c.ci_j[t]], in2 = c.isp[c.cj_j[t]];
    switch (c.fd->sp[in1].pattern * 3 + c.fd->sp[in2].pattern) {
      case PAT_SP * 3 + PAT_SP: trip_rho3c_df<PAT_SP, PAT_SP, QSUM>(c, v, t); break;
      case PAT_SP * 3 + PAT_S: trip_rho3c_df<PAT_SP, PAT_S, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_SP: trip_rho3c_df<PAT_S, PAT_SP, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_S: trip_rho3c_df<PAT_S, PAT_S, QSUM>(c, v, t); break;
      default: break;
    }
  }
}

// Dassemble_vxc_3c (k.DASSEMBLERS/M_Dassemble_vxc_3c_McWEDA_Harris.f90:
// 97-514) in df: the three-center force terms of the Harris neutral atom
// with the den3 sub-cells (Qneutral-summed) for the table, the per-pair
// weights rho dmuxc_in for rho, and no P_eq2; the shell-level denS3
// derivatives enter through their gd-weighted sums of dx, dy, dcos, which
// have the form of the orbital terms' sums of dx G, dy G, dcos G.
template <int PA, int PB, bool QSUM>
__device__ void trip_dvxc_df(const Ctx3c &c, const VxcArgs &v, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB), NS = SA * SB;
  GeomFP64 h;
  trip_geom_fp64(c, t, h);
  const int ia = h.ia, iat = h.iat, jat = h.jat;
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
  if (qsum_fast_df(c, in1, in2, indna, h.x, h.z) != QSUM) return;
  int nk = fd.sp[indna].nssh;
  const double *qk = fd.sp[indna].qn;
  int p = c.tdst[t];
  df cost0 = trip_cost_df(h);
  // shell level: gd-weighted sums of the denS3 derivatives
  df gp = df_zero(), gx = df_zero(), gy = df_zero();
  {
    df s0[NS], Dp[NS], Dx[NS], Dy[NS];
    if constexpr (QSUM) {
      interp3c_df<NS, true>(c, fd.c3rhoq[in1][in2][indna][1], h.x, h.z, cost0, s0, Dp, Dx, Dy);
    } else {
      df s1[NS], s2[NS], s3[NS];
#pragma unroll
      for (int e = 0; e < NS; e++) Dp[e] = Dx[e] = Dy[e] = df_zero();
#pragma unroll 1
      for (int isorp = 0; isorp < nk; isorp++) {
        interp3c_df<NS, true>(c, fd.c3rho[in1][in2][indna][1][isorp], h.x, h.z, cost0, s0, s1, s2, s3);
        df Q = df_from(qk[isorp]);
#pragma unroll
        for (int e = 0; e < NS; e++) {
          Dp[e] = Dp[e] + s1[e] * Q;
          Dx[e] = Dx[e] + s2[e] * Q;
          Dy[e] = Dy[e] + s3[e] * Q;
        }
      }
    }
    const double *gd = v.gd + (long long)VXC_WSH * p;
#pragma unroll
    for (int a = 0; a < SA; a++)
#pragma unroll
      for (int b = 0; b < SB; b++) {
        df w = df_from(gd[a + SA * b]);
        gp = gp + w * Dp[a * SB + b];
        gx = gx + w * Dx[a * SB + b];
        gy = gy + w * Dy[a * SB + b];
      }
  }
  df F[NE], DpF[NE], DxF[NE], DyF[NE];
  if constexpr (QSUM) {
    interp3c_df<NE, true>(c, fd.c3rhoq[in1][in2][indna][0], h.x, h.z, cost0, F, DpF, DxF, DyF);
  } else {
    df t0[NE], t1[NE], t2[NE], t3[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) F[e] = DpF[e] = DxF[e] = DyF[e] = df_zero();
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c_df<NE, true>(c, fd.c3rho[in1][in2][indna][0][isorp], h.x, h.z, cost0, t0, t1, t2, t3);
      df Q = df_from(qk[isorp]);
#pragma unroll
      for (int e = 0; e < NE; e++) {
        F[e] = F[e] + t0[e] * Q;
        DpF[e] = DpF[e] + t1[e] * Q;
        DxF[e] = DxF[e] + t2[e] * Q;
        DyF[e] = DyF[e] + t3[e] * Q;
      }
    }
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
  const double *wdp = v.wd + c.blk_off[p];
  df rb[NA * NB], Gf[NA * NB], G[NE];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = df_from(__ldg(wdp + q));
  mol_density_df<PA, PB>(R, rb, Gf, G);
  df Sx = gx, Sy = gy, Sp = gp;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    Sx = Sx + DxF[e] * G[e];
    Sy = Sy + DyF[e] * G[e];
    Sp = Sp + DpF[e] * G[e];
  }
  df hA[3], hB[3];
  frame_terms_3c_df<PA, PB>(g, Gf, F, hA, hB);
  double fa[3], fb[3];
#pragma unroll 1
  for (int q = 0; q < 3; q++) {
    df amt = (g.x > 1.0e-5) ? (sel3(g.sig, q) - cost * sel3(g.rh, q)) * g.ix : df_zero();
    df bmt = (cost * sel3(g.sig, q) - sel3(g.rh, q)) * iz;
    df ga = sel3(g.rh, q) * Sx + amt * Sp;
    df sa = sel3(hA, q) + ga;
    df sb = sel3(hB, q) + ((bmt * Sp - sel3(g.sig, q) * Sy) - ga * 0.5f);
    double va = -df_to(sa), vb = -df_to(sb);
    fa[0] = q == 0 ? va : fa[0];
    fa[1] = q == 1 ? va : fa[1];
    fa[2] = q == 2 ? va : fa[2];
    fb[0] = q == 0 ? vb : fb[0];
    fb[1] = q == 1 ? vb : fb[1];
    fb[2] = q == 2 ? vb : fb[2];
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(v.f3a + 3 * ia + q, fa[q]);
    atomicAdd(v.f3b + 3 * iat + q, fb[q]);
    atomicAdd(v.f3c + 3 * jat + q, -fa[q] - fb[q]);
  }
}

template <bool QSUM>
__global__ void __launch_bounds__(128) k_dvxc_3c_df(Ctx3c c, VxcArgs v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.T; i += gridDim.x * blockDim.x) {
    int t = c.tperm ? c.tperm[i] : i;
    int in1 = c.isp[c.ci_j[t]], in2 = c.isp[c.cj_j[t]];
    switch (c.fd->sp[in1].pattern * 3 + c.fd->sp[in2].pattern) {
      case PAT_SP * 3 + PAT_SP: trip_dvxc_df<PAT_SP, PAT_SP, QSUM>(c, v, t); break;
      case PAT_SP * 3 + PAT_S: trip_dvxc_df<PAT_SP, PAT_S, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_SP: trip_dvxc_df<PAT_S, PAT_SP, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_S: trip_dvxc_df<PAT_S, PAT_S, QSUM>(c, v, t); break;
      default: break;
    }
  }
}

}  // namespace

int launch_rho_3c_df(const VxcArgs &v, cudaStream_t s) {
  if (v.a.ntrip == 0) return 0;
  Ctx3c c = make3c(v.a);
  int threads = 128;
  long long need = ((long long)v.a.ntrip + threads - 1) / threads;
  int blocks = (int)(need < 152LL * 64 ? need : 152LL * 64);
  k_rho_3c_df<true><<<blocks, threads, 0, s>>>(c, v);
  if (!v.qsum_all) k_rho_3c_df<false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dvxc_3c_df(const VxcArgs &v, cudaStream_t s) {
  if (v.a.ntrip == 0) return 0;
  Ctx3c c = make3c(v.a);
  int threads = 128;
  long long need = ((long long)v.a.ntrip + threads - 1) / threads;
  int blocks = (int)(need < 152LL * 64 ? need : 152LL * 64);
  k_dvxc_3c_df<true><<<blocks, threads, 0, s>>>(c, v);
  if (!v.qsum_all) k_dvxc_3c_df<false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
