// fb_asm3c_df.cu -- sm_103a three-center neutral-atom assembly
// (assemble_vna_3c, j.ASSEMBLERS/M_assemble_3c_Harris.f90:82-227) with the
// table contraction and rotation in double-float on the FP32 pipe.
#include "fb_common_df.cuh"

namespace fb {

// MLP: F comes from the MLP-3c results of list position i instead of the tables
template <int PA, int PB, bool MLP>
__device__ __forceinline__ void trip_3c_df(const Ctx3c &c, int t, int i) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  GeomDF g;
  trip_geom_df(c, t, g);
  df F[NE];
  if constexpr (MLP) {
#pragma unroll
    for (int e = 0; e < NE; e++) F[e] = df_make(c.mlpF[(long long)i * MLP_ME_STRIDE + e]);
  } else {
    const Cell3cDev &cell = c.fd->c3[c.isp[g.iat]][c.isp[g.jat]][c.isp[g.ia]];
    interp3c_df<NE, false>(c, cell, g.x, g.z, g.cost, F, nullptr, nullptr, nullptr);
  }
  // sint = sqrt(max(1e-5, 1 - cost^2)) (:349) for the mvalue = 1 channels
  df s2 = df_one() - g.cost * g.cost;
  df sint = df_sqrt(s2.h > 1.0e-5f ? s2 : df_make(1.0e-5f, 2.5262125e-13f));
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    if constexpr (PL::m.mv[e] == 1) F[e] = F[e] * sint;
  });
  RotDF R;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = g.e[pperm(a)][pperm(b)];
  df X[NA * NB];
  rotate_plan_df<PA, PB, K3C>(R, F, X);
  double *dst = c.vb + c.blk_off[c.tdst[t]];
  const df peq2 = peq2_df();
#pragma unroll
  for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, df_to(X[q] * peq2));
}

template <bool MLP>
__global__ void __launch_bounds__(256) k_assemble_3c_df(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    int i = t;
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    switch (pa * 3 + pb) {
      case PAT_SP * 3 + PAT_SP: trip_3c_df<PAT_SP, PAT_SP, MLP>(c, t, i); break;
      case PAT_SP * 3 + PAT_S: trip_3c_df<PAT_SP, PAT_S, MLP>(c, t, i); break;
      case PAT_S * 3 + PAT_SP: trip_3c_df<PAT_S, PAT_SP, MLP>(c, t, i); break;
      case PAT_S * 3 + PAT_S: trip_3c_df<PAT_S, PAT_S, MLP>(c, t, i); break;
      default: break;
    }
  });
}

int launch_assemble_3c_df(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a3c, (long long)a.ntrip, a.queue ? a.queue + 1 : nullptr, s, grid, block, q);
  if (e) return e;
  k_assemble_3c_df<false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_assemble_3c_mlp(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a3c, (long long)a.ntrip, a.queue ? a.queue + 1 : nullptr, s, grid, block, q);
  if (e) return e;
  k_assemble_3c_df<true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

// rho blocks as hi + lo float pairs, once per force pass
__global__ void k_split_rho(const double *__restrict__ rho, float2 *__restrict__ out, long long n) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  df v = df_from(rho[k]);
  out[k] = make_float2(v.h, v.l);
}

int launch_split_rho(const AsmArgs &a, long long nblock, cudaStream_t s) {
  if (nblock == 0) return 0;
  int threads = 256;
  long long blocks = (nblock + threads - 1) / threads;
  k_split_rho<<<(unsigned)blocks, threads, 0, s>>>(a.rho, a.rho_df, nblock);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
