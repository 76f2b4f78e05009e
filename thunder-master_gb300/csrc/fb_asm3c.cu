// fb_asm3c.cu -- sm_103a kernel of the 3c neutral-atom assembly.
#include "fb_common.cuh"

namespace fb {

// With DOGS the charged shells of the potential atom ialpha add
// dq * (stinky * bcna(isorp) + (1 - stinky) * emnpl), the sub-cell values
// smoothed into the effective monopole of the pair's overlap and z-dipole
// blocks, emnpl = (S/2 - dip/z) / d13 + (S/2 + dip/z) / d23
// (M_assemble_3c_DOGS.f90:158-322).
template <int PA, int PB, bool HASD, bool DOGS>
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
  long long o = c.blk_off[c.tdst[t]];
  double *dst = c.vb + o;
  if constexpr (DOGS) {
    const FdataDev &fd = *c.fd;
    int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
    int nssh = fd.sp[indna].nssh;
    double acc[NA * NB];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) acc[q] = X[q] * P_eq2;
    if (nssh > 0) {
      double d13 = 0.0, d23 = 0.0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        d13 += (g.rna[k] - g.r1[k]) * (g.rna[k] - g.r1[k]);
        d23 += (g.rna[k] - g.r2[k]) * (g.rna[k] - g.r2[k]);
      }
      d13 = sqrt(d13);
      d23 = sqrt(d23);
      double rc3 = fd.sp[indna].rcmin;
      double stinky = smoother(d13, fd.sp[in1].rcmin + rc3, 0.8) * smoother(d23, fd.sp[in2].rcmin + rc3, 0.8);
      const double *Sb = c.S + o, *Db = c.dip + o;
#pragma unroll 1
      for (int isorp = 1; isorp <= nssh; isorp++) {
        const Cell3cDev &cs = fd.c3s[in1][in2][indna][isorp - 1];
        interp3c<NE, false>(c, cs, g.x, g.z, g.cost, F, nullptr, nullptr, nullptr);
        sfor<NE>([&](auto E) {
          constexpr int e = decltype(E)::value;
          if constexpr (PL::m.mv[e] == 1) F[e] = F[e] * sint;
        });
        rotate_plan<PA, PB, K3C>(R, F, X);
        double dq = c.dq[ia * MAXSUB + isorp - 1];
#pragma unroll
        for (int q = 0; q < NA * NB; q++) {
          double sterm = Sb[q] / 2.0, dterm = Db[q] / g.z;
          double emnpl = (sterm - dterm) / d13 + (sterm + dterm) / d23;
          acc[q] = acc[q] + dq * (stinky * X[q] + (1.0 - stinky) * emnpl) * P_eq2;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, acc[q]);
  } else {
#pragma unroll
    for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, X[q] * P_eq2);
  }
}

template <bool HASD, bool DOGS>
__global__ void __launch_bounds__(256) k_assemble_3c(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_3c<PAT_SP, PAT_SP, HASD, DOGS>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c<PAT_SP, PAT_S, HASD, DOGS>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c<PAT_S, PAT_SP, HASD, DOGS>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c<PAT_S, PAT_S, HASD, DOGS>(c, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_3c<PAT_SPD, PAT_SPD, HASD, DOGS>(c, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_3c<PAT_SPD, PAT_SP, HASD, DOGS>(c, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_3c<PAT_SP, PAT_SPD, HASD, DOGS>(c, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_3c<PAT_SPD, PAT_S, HASD, DOGS>(c, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_3c<PAT_S, PAT_SPD, HASD, DOGS>(c, t);
        }
    }
  });
}

// The four instantiations (HASD, DOGS) of k_assemble_3c build as four parts of
// this source (FB_IN_PART); part 0 also holds the launcher.
int launch_assemble_3c_v(int v, const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_3c_v0(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_3c_v1(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_3c_v2(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_assemble_3c_v3(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);

#if FB_IN_PART(0)
int launch_assemble_3c_v(int v, const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  switch (v) {
    case 0: return launch_assemble_3c_v0(c, q, grid, block, s);
    case 1: return launch_assemble_3c_v1(c, q, grid, block, s);
    case 2: return launch_assemble_3c_v2(c, q, grid, block, s);
    case 3: return launch_assemble_3c_v3(c, q, grid, block, s);
  }
  return (int)cudaErrorInvalidValue;
}

int launch_assemble_3c(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a3c, (long long)a.ntrip, a.queue ? a.queue + 1 : nullptr, s, grid, block, q);
  if (e) return e;
  int v = (a.have_d ? 2 : 0) + (a.dogs ? 1 : 0);
  return launch_assemble_3c_v(v, c, q, grid, block, s);
}
#endif

#if FB_IN_PART(0)
int launch_assemble_3c_v0(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_3c<false, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(1)
int launch_assemble_3c_v1(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_3c<false, true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(2)
int launch_assemble_3c_v2(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_3c<true, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(3)
int launch_assemble_3c_v3(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_assemble_3c<true, true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

}  // namespace fb
