// fb_dasm3c.cu -- sm_103a kernel of the 3c force derivatives.
#include "fb_common.cuh"

namespace fb {

// ===========================================================================
// 3c forces: Dassemble_vna_3c (k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136-408)
// ===========================================================================
template <int PA, int PB, bool HASD>
__device__ void trip_3c_force(const Ctx3c &c, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  int ia, iat, jat;
  TripGeom g;
  trip_geom(c, t, ia, iat, jat, g);
  const Cell3cDev &cell = c.fd->c3[c.isp[iat]][c.isp[jat]][c.isp[ia]];
  double dA[3][3][3], dB[3][3][3];
  depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.e, dA, dB);
  double amt[3], bmt[3];
  if (g.x > 1.0e-5) {
    double ix = 1.0 / g.x;
#pragma unroll
    for (int k = 0; k < 3; k++) amt[k] = (g.sighat[k] - g.cost * g.rhat[k]) * ix;
  } else {
    amt[0] = amt[1] = amt[2] = 0.0;
  }
  double iz = 1.0 / g.z;
#pragma unroll
  for (int k = 0; k < 3; k++) bmt[k] = (g.cost * g.sighat[k] - g.rhat[k]) * iz;
  double F[NE], DpF[NE], DxF[NE], DyF[NE];
  interp3c<NE, true>(c, cell, g.x, g.z, g.cost, F, DpF, DxF, DyF);
  double sint = sqrt(fmax(1.0e-5, 1.0 - g.cost * g.cost));
  double M[NE], Ma[3 * NE], Mb[3 * NE];
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    double m = F[e], dp = DpF[e], dx = DxF[e], dy = DyF[e];
    if constexpr (PL::m.mv[e] == 1) {
      dp = DpF[e] * sint - g.cost * F[e] / sint;
      m = F[e] * sint;
      dx = DxF[e] * sint;
      dy = DyF[e] * sint;
    }
    M[e] = m;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double a = g.rhat[q] * dx + amt[q] * dp;
      Ma[q + 3 * e] = a;
      Mb[q + 3 * e] = -g.sighat[q] * dy + bmt[q] * dp - a * 0.5;
    }
  });
  RotM R;
  twister<HASD>(g.e, R);
  DRotM DA, DB;
  dtwister<HASD>(g.e, dA, DA);
  dtwister<HASD>(g.e, dB, DB);
  const double *rho = c.rho + c.blk_off[c.tdst[t]];
  double rb[NA * NB];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = __ldg(rho + q);
  MolRho<PA, PB, K3C> GA, GB;
  mol_rho<PA, PB, K3C>(R, DA, rb, GA);
  mol_rho<PA, PB, K3C>(R, DB, rb, GB);
  double fa[3], fb[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    double sa = 0.0, sb = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
      sa = fma(M[e], GA.H[q][e], sa);
      sa = fma(Ma[q + 3 * e], GA.G[e], sa);
      sb = fma(M[e], GB.H[q][e], sb);
      sb = fma(Mb[q + 3 * e], GB.G[e], sb);
    }
    fa[q] = -sa * P_eq2;
    fb[q] = -sb * P_eq2;
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(c.f3naa + 3 * ia + q, fa[q]);
    atomicAdd(c.f3nab + 3 * iat + q, fb[q]);
    atomicAdd(c.f3nac + 3 * jat + q, -fa[q] - fb[q]);
  }
}

template <bool HASD>
__global__ void __launch_bounds__(256) k_dassemble_3c(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_3c_force<PAT_SP, PAT_SP, HASD>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c_force<PAT_SP, PAT_S, HASD>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c_force<PAT_S, PAT_SP, HASD>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c_force<PAT_S, PAT_S, HASD>(c, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_3c_force<PAT_SPD, PAT_SPD, HASD>(c, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_3c_force<PAT_SPD, PAT_SP, HASD>(c, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_3c_force<PAT_SP, PAT_SPD, HASD>(c, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_3c_force<PAT_SPD, PAT_S, HASD>(c, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_3c_force<PAT_S, PAT_SPD, HASD>(c, t);
        }
    }
  });
}

int launch_dassemble_3c(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d3c, (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block, q);
  if (e) return e;
  if (a.have_d) k_dassemble_3c<true><<<grid, block, 0, s>>>(c, q);
  else k_dassemble_3c<false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
