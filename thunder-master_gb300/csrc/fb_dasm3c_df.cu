// fb_dasm3c_df.cu -- sm_103a three-center force derivatives
// (Dassemble_vna_3c, k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136-408) with
// the table contractions, frame derivatives and density contraction in
// double-float on the FP32 pipe.
#include "fb_common_df.cuh"

namespace fb {

// MLP: F and its cos / x / y derivatives come from the MLP-3c results of
// list position i instead of the tables.  FUSE: also the triplet's
// value-pass term of assemble_vna_3c (M_assemble_3c_Harris.f90:82-227),
// rot(F sint^mvalue) P_eq2 into the vna block, from the same F.
template <int PA, int PB, bool MLP, bool FUSE>
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
  if constexpr (FUSE) {
    // the value-pass term in FP64 on the otherwise idle FP64 pipe: a few
    // dozen instructions instead of the double-float rotation's several
    // hundred (code size, issue slots), from the df values and frame
    RotM Rd;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) Rd.p[a][b] = df_to(R.p[a][b]);
    double Md[NE], X[NA * NB];
#pragma unroll
    for (int e = 0; e < NE; e++) Md[e] = df_to(F[e]) * P_eq2;
    rotate_plan<PA, PB, K3C>(Rd, Md, X);
    double *dst = c.vb + c.blk_off[c.tdst[t]];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, X[q]);
  }
  const df *rho = c.rho_df + c.blk_off[c.tdst[t]];
  df rb[NA * NB], Gf[NA * NB], G[NE];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = rho[q];
  mol_density_df<PA, PB>(R, rb, Gf, G);
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
  // frame-derivative terms (Dtwister contracted with rho) through the
  // rotation rates of the frame
  df hA[3], hB[3];
  frame_terms_3c_df<PA, PB>(g, Gf, F, hA, hB);
  const df peq2 = peq2_df();
  double fa[3], fb[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    df amt = (g.x > 1.0e-5) ? (g.sig[q] - cost * g.rh[q]) * g.ix : df_zero();
    df bmt = (cost * g.sig[q] - g.rh[q]) * iz;
    df ga = g.rh[q] * Sx + amt * Sp;
    df sa = ga + hA[q];
    df sb = ((bmt * Sp - g.sig[q] * Sy) - ga * 0.5f) + hB[q];
    fa[q] = -df_to(sa * peq2);
    fb[q] = -df_to(sb * peq2);
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(c.f3naa + 3 * ia + q, fa[q]);
    atomicAdd(c.f3nab + 3 * iat + q, fb[q]);
    atomicAdd(c.f3nac + 3 * jat + q, -fa[q] - fb[q]);
  }
}

// At most 128 threads per CTA and 3 CTAs per SM: 168 registers per thread,
// 12 warps per SM instead of the 8 that 255 registers allow.  The kernel is
// issue- and latency-bound: the extra warps are worth more than the
// 0.7-1 KB of spills per thread the cap costs (7.42 -> 6.71 ms on SiC4096,
// the fused form 9.03 -> 7.41 ms).
// The network-fed tail (MLP) has no interpolation and fewer live values: 4
// CTAs per SM (128 registers, 16 warps) for 0.4-0.65 KB of spills.
constexpr int DF_FORCE_THREADS = 128;
template <bool MLP, bool FUSE>
__global__ void __launch_bounds__(DF_FORCE_THREADS, MLP ? 4 : 3) k_dassemble_3c_df(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    int i = t;
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    switch (pa * 3 + pb) {
      case PAT_SP * 3 + PAT_SP: trip_3c_force_df<PAT_SP, PAT_SP, MLP, FUSE>(c, t, i); break;
      case PAT_SP * 3 + PAT_S: trip_3c_force_df<PAT_SP, PAT_S, MLP, FUSE>(c, t, i); break;
      case PAT_S * 3 + PAT_SP: trip_3c_force_df<PAT_S, PAT_SP, MLP, FUSE>(c, t, i); break;
      case PAT_S * 3 + PAT_S: trip_3c_force_df<PAT_S, PAT_S, MLP, FUSE>(c, t, i); break;
      default: break;
    }
  });
}

// the three-center force shape, with the block size capped at the df
// kernels' launch bound
static KCfg df_force_cfg(const KCfg &cfg) {
  KCfg k = cfg;
  if (k.threads <= 0 || k.threads > DF_FORCE_THREADS) k.threads = DF_FORCE_THREADS;
  return k;
}

int launch_dassemble_3c_df(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(df_force_cfg(a.cfg_d3c), (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block,
                       q);
  if (e) return e;
  if (a.fuse_value) k_dassemble_3c_df<false, true><<<grid, block, 0, s>>>(c, q);
  else k_dassemble_3c_df<false, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dassemble_3c_mlp(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(df_force_cfg(a.cfg_d3c), (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block,
                       q);
  if (e) return e;
  if (a.fuse_value) k_dassemble_3c_df<true, true><<<grid, block, 0, s>>>(c, q);
  else k_dassemble_3c_df<true, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
