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

__device__ __forceinline__ bool qsum_triple_df(const FdataDev &fd, int in1, int in2, int in3) {
  return fd.c3rhoq[in1][in2][in3][0].off >= 0 && fd.c3rhoq[in1][in2][in3][1].off >= 0;
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
    if (qsum_triple_df(*c.fd, in1, in2, c.isp[c.trip_alpha[t]]) != QSUM) continue;
    switch (c.fd->sp[in1].pattern * 3 + c.fd->sp[in2].pattern) {
      case PAT_SP * 3 + PAT_SP: trip_rho3c_df<PAT_SP, PAT_SP, QSUM>(c, v, t); break;
      case PAT_SP * 3 + PAT_S: trip_rho3c_df<PAT_SP, PAT_S, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_SP: trip_rho3c_df<PAT_S, PAT_SP, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_S: trip_rho3c_df<PAT_S, PAT_S, QSUM>(c, v, t); break;
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

}  // namespace fb
