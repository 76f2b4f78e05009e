// fb_dasm2c.cu -- sm_103a kernel of the 2c force derivatives.
#include "fb_common.cuh"

namespace fb {

template <int PA, int PB, bool HASD>
__device__ __forceinline__ void pair_d2c(const CtxD2c &c, int i, int p, unsigned what) {
  using PL = Plan<PA, PB, K2C>;
  using PLA = Plan<PA, PA, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n, NEA = PLA::m.n;
  const Ctx2c &b = c.b;
  int j = b.neigh_j[p];
  int in1 = b.isp[i], in2 = b.isp[j];
  double r1[3], r2[3], z, e[3][3];
  pair_geom(b, i, p, r1, r2, z, e);
  double dd[3][3][3];
  depsilon_2c(r1, r2, z, e, dd);
  RotM R;
  DRotM D;
  twister<HASD>(e, R);
  dtwister<HASD>(e, dd, D);
  double eta[3] = {e[0][2], e[1][2], e[2][2]};
  const FdataDev &fd = *b.fd;
  long long o = b.blk_off[p];
  bool self = (i == j && b.neigh_b[p] == 0);
  double rb[NA * NB];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = __ldg(c.rho + o + q);
  constexpr int NM = NE > NEA ? NE : NEA;
  double v[NM], dv[NM], vd[3 * NM];
  bool tiny = z < 1.0e-5;  // getDMEs_Fdata_2c early return (:510-520)
  double out[3];
  if (what & 1u) {
    interp2c_d<NE>(b.table2c, fd.c2[in1][in2][0], z, tiny, v, dv, b.status);
    vec2c<NE>(z, eta, dv, vd);
    if (c.keep) {
      double Xd[3 * NA * NB];
      drotate_plan<PA, PB, K2C>(R, D, v, vd, Xd);
#pragma unroll
      for (int q = 0; q < 3 * NA * NB; q++) c.dS[3 * o + q] = Xd[q];
    }
    double cb[NA * NB];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) cb[q] = __ldg(c.cape + o + q);
    contract<PA, PB, K2C, HASD>(R, D, cb, v, vd, out);
#pragma unroll
    for (int q = 0; q < 3; q++) c.sumS[3 * p + q] = out[q];
  }
  if (what & 2u) {
    interp2c_d<NE>(b.table2c, fd.c2[in1][in2][1], z, tiny, v, dv, b.status);
    vec2c<NE>(z, eta, dv, vd);
    if (c.keep) {
      double Xd[3 * NA * NB];
      drotate_plan<PA, PB, K2C>(R, D, v, vd, Xd);
#pragma unroll
      for (int q = 0; q < 3 * NA * NB; q++) c.dT[3 * o + q] = Xd[q];
    }
    contract<PA, PB, K2C, HASD>(R, D, rb, v, vd, out);
#pragma unroll
    for (int q = 0; q < 3; q++) c.sumT[3 * p + q] = out[q];
  }
  if (what & 4u) {
    double f[3] = {0.0, 0.0, 0.0};
    if (!self) {
#pragma unroll
      for (int w2 = 2; w2 <= 3; w2++) {
        interp2c_d<NE>(b.table2c, fd.c2[in1][in2][w2], z, tiny, v, dv, b.status);
        vec2c<NE>(z, eta, dv, vd);
        contract<PA, PB, K2C, HASD>(R, D, rb, v, vd, out);
#pragma unroll
        for (int q = 0; q < 3; q++) f[q] -= out[q] * P_eq2;
      }
    }
#pragma unroll
    for (int q = 0; q < 3; q++) c.ontop[3 * p + q] = f[q];
    // atom case, contracted with rho of the self block of i
    interp2c_d<NEA>(b.table2c, fd.c2[in1][in2][4], z, tiny, v, dv, b.status);
    vec2c<NEA>(z, eta, dv, vd);
    double rs[NA * NA];
    long long os = b.blk_off[b.pair_off[i] + b.neigh_self[i]];
#pragma unroll
    for (int q = 0; q < NA * NA; q++) rs[q] = __ldg(c.rho + os + q);
    contract<PA, PA, K2C, HASD>(R, D, rs, v, vd, out);
#pragma unroll
    for (int q = 0; q < 3; q++) c.atomf[3 * p + q] = -out[q] * P_eq2;
  }
}

template <int PA, bool HASD>
__device__ void atom_d2c(const CtxD2c &c, int i, int lane, unsigned what) {
  int p0 = c.b.pair_off[i], p1 = c.b.pair_off[i + 1];
  for (int p = p0 + lane; p < p1; p += 32) {
    int pb = c.b.fd->sp[c.b.isp[c.b.neigh_j[p]]].pattern;
    if (pb == PAT_SP) pair_d2c<PA, PAT_SP, HASD>(c, i, p, what);
    else if (pb == PAT_S) pair_d2c<PA, PAT_S, HASD>(c, i, p, what);
    else if constexpr (HASD) pair_d2c<PA, PAT_SPD, HASD>(c, i, p, what);
  }
}

template <bool HASD>
__global__ void __launch_bounds__(256) k_dassemble_2c(CtxD2c c, unsigned what, Sched q) {
  for_each_warp_item(c.b.N, q, [&](int i, int lane) {
    int pa = c.b.fd->sp[c.b.isp[i]].pattern;
    if (pa == PAT_SP) atom_d2c<PAT_SP, HASD>(c, i, lane, what);
    else if (pa == PAT_S) atom_d2c<PAT_S, HASD>(c, i, lane, what);
    else if constexpr (HASD) atom_d2c<PAT_SPD, HASD>(c, i, lane, what);
  });
}

int launch_dassemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s) {
  CtxD2c c;
  c.b = make2c(a);
  c.rho = a.rho;
  c.cape = a.cape;
  c.dS = a.dS;
  c.dT = a.dT;
  c.sumT = a.sumT;
  c.sumS = a.sumS;
  c.ontop = a.ontop;
  c.atomf = a.atomf;
  c.keep = a.keep_dblocks;
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d2c, (long long)a.N * 32, a.queue ? a.queue + 2 : nullptr, s, grid, block, q);
  if (e) return e;
  if (a.have_d) k_dassemble_2c<true><<<grid, block, 0, s>>>(c, what, q);
  else k_dassemble_2c<false><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
