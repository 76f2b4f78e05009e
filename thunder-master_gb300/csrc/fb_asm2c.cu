// fb_asm2c.cu -- sm_103a kernel of the 2c assembly (S, T, vna 2c) and the force reduction.
#include "fb_common.cuh"

namespace fb {

// what: 1 overlap, 2 kinetic, 4 vna (ontop + atom), 64 z-dipole.  With DOGS
// the vna terms add the charged shells (M_assemble_2c_DOGS.f90:640-814):
// ontop L / R the sub-cells of the atom the potential sits on weighted by
// its shell charges, the atom case the smoothed effective monopole
// emnpl = S(i, self) / z (Sself, the self overlap block of atom i).
template <int PA, int PB, bool HASD, bool DOGS>
__device__ __forceinline__ void pair_2c(const Ctx2c &c, int i, int p, unsigned what, double *Xatom,
                                        const double *Sself) {
  using PL = Plan<PA, PB, K2C>;
  using PLA = Plan<PA, PA, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n, NEA = PLA::m.n;
  int j = c.neigh_j[p];
  int in1 = c.isp[i], in2 = c.isp[j];
  double r1[3], r2[3], z, e[3][3];
  pair_geom(c, i, p, r1, r2, z, e);
  RotM R;
  twister<HASD>(e, R);
  const FdataDev &fd = *c.fd;
  long long o = c.blk_off[p];
  bool self = (i == j && c.neigh_b[p] == 0);
  double w[7], v[NE > NEA ? NE : NEA], X[NA * NB];
  int i0 = 0;
  const Cell2cDev *last = nullptr;
  auto weights = [&](const Cell2cDev &cell) {
    if (z > cell.xmax * (1.0 + 1.0e-5)) atomicOr(c.status, DEVERR_XLARGE);
    if (!last || !same_grid(*last, cell)) lagrange7(z, cell, i0, w, nullptr);
    last = &cell;
  };
  if (what & 1u) {  // overlap
    const Cell2cDev &cell = fd.c2[in1][in2][0];
    weights(cell);
    interp2c<NE>(c.table2c, cell, i0, w, v);
    rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
    for (int q = 0; q < NA * NB; q++) c.S[o + q] = X[q];
  }
  if (what & 2u) {  // kinetic
    const Cell2cDev &cell = fd.c2[in1][in2][1];
    weights(cell);
    interp2c<NE>(c.table2c, cell, i0, w, v);
    rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
    for (int q = 0; q < NA * NB; q++) c.T[o + q] = X[q];
  }
  if (what & 64u) {  // z-dipole (assemble_dipole_z, M_assemble_2c_DOGS.f90:376-499)
    const Cell2cDev &cell = fd.c2dip[in1][in2];
    weights(cell);
    interp2c<NE>(c.table2c, cell, i0, w, v);
    rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
    for (int q = 0; q < NA * NB; q++) c.dip[o + q] = X[q];
  }
  if (what & 4u) {  // vna: ontop L + R into blocko; zero block
    double acc[NA * NB];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) acc[q] = 0.0;
    if (!self) {
      const Cell2cDev &cL = fd.c2[in1][in2][2];
      weights(cL);
      interp2c<NE>(c.table2c, cL, i0, w, v);
      rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
      for (int q = 0; q < NA * NB; q++) acc[q] = X[q] * P_eq2;
      if constexpr (DOGS) {
#pragma unroll 1
        for (int isorp = 1; isorp <= fd.sp[in1].nssh; isorp++) {
          const Cell2cDev &cs = fd.c2s[in1][in2][0][isorp - 1];
          weights(cs);
          interp2c<NE>(c.table2c, cs, i0, w, v);
          rotate_plan<PA, PB, K2C>(R, v, X);
          double dq = c.dq[i * MAXSUB + isorp - 1];
#pragma unroll
          for (int q = 0; q < NA * NB; q++) acc[q] = acc[q] + dq * X[q] * P_eq2;
        }
      }
      const Cell2cDev &cR = fd.c2[in1][in2][3];
      weights(cR);
      interp2c<NE>(c.table2c, cR, i0, w, v);
      rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
      for (int q = 0; q < NA * NB; q++) acc[q] = acc[q] + X[q] * P_eq2;
      if constexpr (DOGS) {
#pragma unroll 1
        for (int isorp = 1; isorp <= fd.sp[in2].nssh; isorp++) {
          const Cell2cDev &cs = fd.c2s[in1][in2][1][isorp - 1];
          weights(cs);
          interp2c<NE>(c.table2c, cs, i0, w, v);
          rotate_plan<PA, PB, K2C>(R, v, X);
          double dq = c.dq[j * MAXSUB + isorp - 1];
#pragma unroll
          for (int q = 0; q < NA * NB; q++) acc[q] = acc[q] + dq * X[q] * P_eq2;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NA * NB; q++) c.vbo[o + q] = acc[q];
    if (!self) {
#pragma unroll
      for (int q = 0; q < NA * NB; q++) c.vb[o + q] = 0.0;
    }
    // atom case <i|v(j)|i>, rotated with (in1, in1)
    const Cell2cDev &cA = fd.c2[in1][in2][4];
    weights(cA);
    interp2c<NEA>(c.table2c, cA, i0, w, v);
    double XA[NA * NA];
    rotate_plan<PA, PA, K2C>(R, v, XA);
#pragma unroll
    for (int q = 0; q < NA * NA; q++) Xatom[q] = fma(XA[q], P_eq2, Xatom[q]);
    if constexpr (DOGS) {
      // smoothing of the charged shells (M_assemble_2c_DOGS.f90:744-812)
      double smooth = smoother(z, fd.sp[in1].rcmin + fd.sp[in2].rcmin, 0.8);
      double iz = z > 1.0e-4 ? 1.0 / z : 0.0;
#pragma unroll 1
      for (int isorp = 1; isorp <= fd.sp[in2].nssh; isorp++) {
        const Cell2cDev &cs = fd.c2s[in1][in2][2][isorp - 1];
        weights(cs);
        interp2c<NEA>(c.table2c, cs, i0, w, v);
        rotate_plan<PA, PA, K2C>(R, v, XA);
        double dq = c.dq[j * MAXSUB + isorp - 1];
#pragma unroll
        for (int q = 0; q < NA * NA; q++)
          Xatom[q] = Xatom[q] + P_eq2 * dq * ((1.0 - smooth) * (Sself[q] * iz) + smooth * XA[q]);
      }
    }
  }
}

template <int PA, bool HASD, bool DOGS>
__device__ __forceinline__ void pair_2c_dispatch(const Ctx2c &c, int i, int p, unsigned what, double *Xatom,
                                                 const double *Sself) {
  int pb = c.fd->sp[c.isp[c.neigh_j[p]]].pattern;
  if (pb == PAT_SP) pair_2c<PA, PAT_SP, HASD, DOGS>(c, i, p, what, Xatom, Sself);
  else if (pb == PAT_S) pair_2c<PA, PAT_S, HASD, DOGS>(c, i, p, what, Xatom, Sself);
  else if constexpr (HASD) pair_2c<PA, PAT_SPD, HASD, DOGS>(c, i, p, what, Xatom, Sself);
}

template <int PA, bool HASD, bool DOGS>
__device__ void atom_2c(const Ctx2c &c, int i, int lane, unsigned what) {
  constexpr int NA = pat_norb(PA);
  double Xatom[NA * NA];
#pragma unroll
  for (int q = 0; q < NA * NA; q++) Xatom[q] = 0.0;
  int p0 = c.pair_off[i], p1 = c.pair_off[i + 1];
  double Sself[DOGS ? NA * NA : 1];
  if (DOGS && (what & 4u)) {
    // the self overlap block S(i, neigh_self(i)) the DOGS atom terms scale
    // (the same interpolation and frame as the overlap pass gives it)
    using PLA = Plan<PA, PA, K2C>;
    int ps = p0 + c.neigh_self[i];
    double r1[3], r2[3], z, e[3][3];
    pair_geom(c, i, ps, r1, r2, z, e);
    RotM R;
    twister<HASD>(e, R);
    const Cell2cDev &cell = c.fd->c2[c.isp[i]][c.isp[i]][0];
    double w[7], v[PLA::m.n];
    int i0 = 0;
    lagrange7(z, cell, i0, w, nullptr);
    interp2c<PLA::m.n>(c.table2c, cell, i0, w, v);
    rotate_plan<PA, PA, K2C>(R, v, Sself);
  }
  for (int p = p0 + lane; p < p1; p += 32) pair_2c_dispatch<PA, HASD, DOGS>(c, i, p, what, Xatom, Sself);
  if (what & 4u) {
#pragma unroll
    for (int q = 0; q < NA * NA; q++) {
      double v = Xatom[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      Xatom[q] = v;
    }
    if (lane == 0) {
      // (a missing self pair is reported by the neighbor fill; stay in bounds)
      long long os = c.blk_off[p0 + max(c.neigh_self[i], 0)];
#pragma unroll
      for (int q = 0; q < NA * NA; q++) c.vb[os + q] = Xatom[q];
    }
  }
}

template <bool HASD, bool DOGS>
__global__ void __launch_bounds__(256) k_assemble_2c(Ctx2c c, unsigned what, Sched q) {
  for_each_warp_item(c.N, q, [&](int i, int lane) {
    int pa = c.fd->sp[c.isp[i]].pattern;
    if (pa == PAT_SP) atom_2c<PAT_SP, HASD, DOGS>(c, i, lane, what);
    else if (pa == PAT_S) atom_2c<PAT_S, HASD, DOGS>(c, i, lane, what);
    else if constexpr (HASD) atom_2c<PAT_SPD, HASD, DOGS>(c, i, lane, what);
  });
}

#if FB_IN_PART(0)
// build_forces, assembly terms (c.SYSTEM/M_build_forces.f90:172-588).  The
// j-side contribution of pair (i -> j) is gathered by atom j through
// neigh_back, which maps j's own pair list one-to-one onto the pairs whose
// neighbor is j, so no atomics are needed.  One warp per atom, lanes over
// its pairs, a warp reduction of the nine sums.
__global__ void k_build_forces(int N, const int *__restrict__ pair_off, const int *__restrict__ neigh_j,
                               const int *__restrict__ neigh_back, const double *__restrict__ sumT,
                               const double *__restrict__ sumS, const double *__restrict__ ontop,
                               const double *__restrict__ atomf, const double *__restrict__ f3a,
                               const double *__restrict__ f3b, const double *__restrict__ f3c,
                               double *__restrict__ kin, double *__restrict__ vna, double *__restrict__ pul,
                               double *__restrict__ ftot, unsigned what) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= N) return;
  double k[3] = {0, 0, 0}, v[3] = {0, 0, 0}, pu[3] = {0, 0, 0};
  for (int p = pair_off[i] + lane; p < pair_off[i + 1]; p += 32) {
    int j = neigh_j[p];
    int pb = pair_off[j] + neigh_back[p];  // pair (j -> i)
#pragma unroll
    for (int q = 0; q < 3; q++) {
      if (what & 2u) k[q] += -sumT[3 * p + q] + sumT[3 * pb + q];
      if (what & 1u) pu[q] += -sumS[3 * p + q] + sumS[3 * pb + q];
      if (what & 4u) v[q] += atomf[3 * p + q] + ontop[3 * p + q] - atomf[3 * pb + q] - ontop[3 * pb + q];
    }
  }
#pragma unroll
  for (int q = 0; q < 3; q++)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      k[q] += __shfl_xor_sync(0xffffffffu, k[q], off);
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
      pu[q] += __shfl_xor_sync(0xffffffffu, pu[q], off);
    }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      kin[3 * i + q] = k[q];
      vna[3 * i + q] = v[q];
      pul[3 * i + q] = pu[q];
      double f3 = (what & 8u) ? f3a[3 * i + q] + f3b[3 * i + q] + f3c[3 * i + q] : 0.0;
      ftot[3 * i + q] = k[q] + v[q] + f3 - pu[q];
    }
  }
}
#endif

// The four instantiations (HASD, DOGS) of k_assemble_2c build as four parts of
// this source (FB_IN_PART); part 0 also holds the launcher.
int launch_assemble_2c_v(int v, const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_2c_v0(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_2c_v1(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_2c_v2(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_2c_v3(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);

#if FB_IN_PART(0)
int launch_assemble_2c_v(int v, const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  switch (v) {
    case 0: return launch_assemble_2c_v0(c, what, q, grid, block, s);
    case 1: return launch_assemble_2c_v1(c, what, q, grid, block, s);
    case 2: return launch_assemble_2c_v2(c, what, q, grid, block, s);
    case 3: return launch_assemble_2c_v3(c, what, q, grid, block, s);
  }
  return (int)cudaErrorInvalidValue;
}

int launch_assemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s) {
  Ctx2c c = make2c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a2c, (long long)a.N * 32, a.queue ? a.queue + 0 : nullptr, s, grid, block, q);
  if (e) return e;
  bool dogs = a.dogs && (what & 4u);
  int v = (a.have_d ? 2 : 0) + (dogs ? 1 : 0);
  return launch_assemble_2c_v(v, c, what, q, grid, block, s);
}
#endif

#if FB_IN_PART(0)
int launch_assemble_2c_v0(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_2c<false, false><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(1)
int launch_assemble_2c_v1(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_2c<false, true><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(2)
int launch_assemble_2c_v2(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_2c<true, false><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(3)
int launch_assemble_2c_v3(const Ctx2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_2c<true, true><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(0)
int launch_build_forces(const AsmArgs &a, unsigned what, cudaStream_t s) {
  int threads = 128, blocks = (a.N * 32 + threads - 1) / threads;
  k_build_forces<<<blocks, threads, 0, s>>>(a.N, a.pair_off, a.neigh_j, a.neigh_back, a.sumT, a.sumS, a.ontop,
                                            a.atomf, a.f3naa, a.f3nab, a.f3nac, a.kin, a.vna, a.pul, a.ftot, what);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

}  // namespace fb
