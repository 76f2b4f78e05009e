// fb_asm3c.cu -- sm_103a kernel of the 3c neutral-atom assembly.
#include "fb_common.cuh"

namespace fb {

template <int PA, int PB, bool HASD>
__device__ __forceinline__ void trip_3c(const Ctx3c &c, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  int ia, iat, jat;
  TripGeom g;
  trip_geom(c, t, ia, iat, jat, g);
  const Cell3cDev &cell = c.fd->c3[c.isp[iat]][c.isp[jat]][c.isp[ia]];
  double F[NE];
  interp3c<NE, false>(c, cell, g.x, g.z, g.cost, F, nullptr, nullptr, nullptr);
  double sint = sqrt(fmax(1.0e-5, 1.0 - g.cost * g.cost));
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    if constexpr (PL::m.mv[e] == 1) F[e] = F[e] * sint;
  });
  RotM R;
  twister<HASD>(g.e, R);
  double X[NA * NB];
  rotate_plan<PA, PB, K3C>(R, F, X);
  double *dst = c.vb + c.blk_off[c.tdst[t]];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, X[q] * P_eq2);
}

template <bool HASD>
__global__ void __launch_bounds__(256) k_assemble_3c(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_3c<PAT_SP, PAT_SP, HASD>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c<PAT_SP, PAT_S, HASD>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c<PAT_S, PAT_SP, HASD>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c<PAT_S, PAT_S, HASD>(c, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_3c<PAT_SPD, PAT_SPD, HASD>(c, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_3c<PAT_SPD, PAT_SP, HASD>(c, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_3c<PAT_SP, PAT_SPD, HASD>(c, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_3c<PAT_SPD, PAT_S, HASD>(c, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_3c<PAT_S, PAT_SPD, HASD>(c, t);
        }
    }
  });
}

int launch_assemble_3c(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a3c, (long long)a.ntrip, a.queue ? a.queue + 1 : nullptr, s, grid, block, q);
  if (e) return e;
  if (a.have_d) k_assemble_3c<true><<<grid, block, 0, s>>>(c, q);
  else k_assemble_3c<false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
