// fb_dasm3c.cu -- sm_103a kernel of the 3c force derivatives.
#include "fb_common.cuh"

namespace fb {

// ===========================================================================
// 3c forces: Dassemble_vna_3c (k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136-408)
// ===========================================================================
// With DOGS the charged shells of ialpha add (M_Dassemble_3c_DOGS.f90:
// 355-520) sum_isorp dq * (stinky dX + dstn X - dstn emnpl + (1 - stinky)
// demnpl): the sub-cells are linear in their tables, so the dq-weighted sum
// of the sub-cells goes through the same derivative rotations as the
// neutral term (scaled by stinky); the smoother and monopole terms are
// contracted with rho through the per-pair sums of rho S, rho dip, rho dS
// and rho ddip the 2c kernel left in dogs_ps.
// FUSE (Harris only): the same triplet's value-pass term of assemble_vna_3c
// (j.ASSEMBLERS/M_assemble_3c_Harris.f90:82-227), rot(F sint^mvalue) P_eq2
// into the vna block (i, mneigh), is added from the F this kernel
// interpolates anyway, so a step with forces interpolates every triplet once.
template <int PA, int PB, bool HASD, bool DOGS, bool FUSE>
__device__ void trip_3c_force(const Ctx3c &c, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  int ia, iat, jat;
  TripGeom g;
  trip_geom(c, t, ia, iat, jat, g);
  const Cell3cDev &cell = c.fd->c3[c.isp[iat]][c.isp[jat]][c.isp[ia]];
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
  // DOGS: Fq = sum dq * sub-cell (values, for the smoother term), and
  // F += stinky * sum dq * sub-cell (values and derivatives)
  double Fq[DOGS ? NE : 1], stinky = 0.0, dsum = 0.0, dstnA[3], dstnB[3], rA1[3], rA2[3], d13 = 0.0, d23 = 0.0;
  if constexpr (DOGS) {
    const FdataDev &fd = *c.fd;
    int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      d13 += (g.rna[k] - g.r1[k]) * (g.rna[k] - g.r1[k]);
      d23 += (g.rna[k] - g.r2[k]) * (g.rna[k] - g.r2[k]);
    }
    d13 = sqrt(d13);
    d23 = sqrt(d23);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      rA1[k] = d13 > 1.0e-5 ? (g.rna[k] - g.r1[k]) / d13 : 0.0;
      rA2[k] = d23 > 1.0e-5 ? (g.rna[k] - g.r2[k]) / d23 : 0.0;
    }
    double rc3 = fd.sp[indna].rcmin;
    double rend1 = fd.sp[in1].rcmin + rc3, rend2 = fd.sp[in2].rcmin + rc3;
    double s13 = smoother(d13, rend1, 0.8), ds13 = dsmoother(d13, rend1, 0.8);
    double s23 = smoother(d23, rend2, 0.8), ds23 = dsmoother(d23, rend2, 0.8);
    stinky = s13 * s23;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      dstnB[k] = -ds13 * s23 * rA1[k];
      double dstnC = -s13 * ds23 * rA2[k];
      dstnA[k] = -dstnB[k] - dstnC;
    }
    double Gq[NE], Gp[NE], Gx[NE], Gy[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) Fq[e] = 0.0;
#pragma unroll 1
    for (int isorp = 1; isorp <= fd.sp[indna].nssh; isorp++) {
      interp3c<NE, true>(c, fd.c3s[in1][in2][indna][isorp - 1], g.x, g.z, g.cost, Gq, Gp, Gx, Gy);
      double dq = c.dq[ia * MAXSUB + isorp - 1];
      dsum += dq;
      double w = dq * stinky;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        Fq[e] = fma(dq, Gq[e], Fq[e]);
        F[e] = fma(w, Gq[e], F[e]);
        DpF[e] = fma(w, Gp[e], DpF[e]);
        DxF[e] = fma(w, Gx[e], DxF[e]);
        DyF[e] = fma(w, Gy[e], DyF[e]);
      }
    }
    sfor<NE>([&](auto E) {
      constexpr int e = decltype(E)::value;
      if constexpr (PL::m.mv[e] == 1) Fq[e] = Fq[e] * sint;
    });
  }
  // molecular-frame value and derivatives with the sin(theta) factor of
  // the mvalue = 1 channels (M_Fdata_3c.f90:814-833)
  double M[NE], Dp[NE], Dx[NE], Dy[NE];
  const double cs = g.cost / sint;
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    M[e] = F[e];
    Dp[e] = DpF[e];
    Dx[e] = DxF[e];
    Dy[e] = DyF[e];
    if constexpr (PL::m.mv[e] == 1) {
      Dp[e] = fma(DpF[e], sint, -cs * F[e]);
      M[e] = F[e] * sint;
      Dx[e] = DxF[e] * sint;
      Dy[e] = DyF[e] * sint;
    }
  });
  RotM R;
  twister<HASD>(g.e, R);
  if constexpr (FUSE) {
    double X[NA * NB];
    rotate_plan<PA, PB, K3C>(R, M, X);
    double *dst = c.vb + c.blk_off[c.tdst[t]];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, X[q] * P_eq2);
  }
  const double *rho = c.rho + c.blk_off[c.tdst[t]];
  double rb[NA * NB];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = __ldg(rho + q);
  // G(e): the density in the molecular frame at the ME positions; hA, hB:
  // sum_e M_e H_c(e), the frame-derivative terms of the neutral atom's and
  // atom 1's coordinates (Dtwister, M_Drotations.f90:456-471, contracted
  // with rho)
  double Ge[NE], hA[3], hB[3];
  if constexpr (NA <= 4 && NB <= 4) {
    double Gf[NA * NB];
    mol_G_full<PA, PB>(R, rb, Gf);
    sfor<NE>([&](auto E) {
      constexpr int e = decltype(E)::value;
      constexpr int at = PL::m.mu[e] + NA * PL::m.nu[e];
      Ge[e] = Gf[at];
    });
    frame_terms_3c<PA, PB>(g, Gf, M, hA, hB);
  } else {
    double dA[3][3][3], dB[3][3][3];
    depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.e, dA, dB);
    DRotM DA, DB;
    dtwister<HASD>(g.e, dA, DA);
    dtwister<HASD>(g.e, dB, DB);
    MolRho<PA, PB, K3C> GA, GB;
    mol_rho_ab<PA, PB, K3C>(R, DA, DB, rb, GA, GB);
#pragma unroll
    for (int e = 0; e < NE; e++) Ge[e] = GA.G[e];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double sa = 0.0, sb = 0.0;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        sa = fma(M[e], GA.H[q][e], sa);
        sb = fma(M[e], GB.H[q][e], sb);
      }
      hA[q] = sa;
      hB[q] = sb;
    }
  }
  // f3naMa(q, e) = rhat_q dx + amt_q dp and f3naMb(q, e) = -sighat_q dy +
  // bmt_q dp - f3naMa(q, e) / 2 (:334-344) enter only through their sums
  // with G(e): sum_e Ma(q, e) G(e) = rhat_q Sx + amt_q Sp, and
  // sum_e Mb(q, e) G(e) = -sighat_q Sy + bmt_q Sp - (rhat_q Sx + amt_q Sp) / 2
  double Sx = 0.0, Sy = 0.0, Sp = 0.0;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    Sx = fma(Dx[e], Ge[e], Sx);
    Sy = fma(Dy[e], Ge[e], Sy);
    Sp = fma(Dp[e], Ge[e], Sp);
  }
  double fa[3], fb[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    double ga = fma(g.rhat[q], Sx, amt[q] * Sp);
    double sa = ga + hA[q];
    double sb = fma(-g.sighat[q], Sy, fma(bmt[q], Sp, -0.5 * ga)) + hB[q];
    fa[q] = -sa * P_eq2;
    fb[q] = -sb * P_eq2;
  }
  if constexpr (DOGS) {
    // dstn * sum rho rot(Fq), and the effective monopole emnpl =
    // (S/2 - dip/z)/d13 + (S/2 + dip/z)/d23 with its derivatives, all
    // contracted with rho of the pair
    double cx = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) cx = fma(Fq[e], Ge[e], cx);
    const double *ps = c.dogs_ps + 8 * (long long)c.tdst[t];
    double sterm = 0.5 * ps[0], dterm = ps[1] / g.z;
    double am = sterm - dterm, ap = sterm + dterm;
    double emnpl = am / d13 + ap / d23;
    double i13 = 1.0 / (d13 * d13), i23 = 1.0 / (d23 * d23);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double spterm = 0.5 * ps[2 + q];
      double dpterm = ps[5 + q] / g.z + dterm * g.sighat[q] / g.z;
      double dA = -am * rA1[q] * i13 - ap * rA2[q] * i23;
      double dB = am * rA1[q] * i13 + (spterm - dpterm) / d13 + (spterm + dpterm) / d23;
      fa[q] -= P_eq2 * (dstnA[q] * cx - dsum * dstnA[q] * emnpl + dsum * (1.0 - stinky) * dA);
      fb[q] -= P_eq2 * (dstnB[q] * cx - dsum * dstnB[q] * emnpl + dsum * (1.0 - stinky) * dB);
    }
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(c.f3naa + 3 * ia + q, fa[q]);
    atomicAdd(c.f3nab + 3 * iat + q, fb[q]);
    atomicAdd(c.f3nac + 3 * jat + q, -fa[q] - fb[q]);
  }
}

template <bool HASD, bool DOGS, bool FUSE>
__global__ void __launch_bounds__(256) k_dassemble_3c(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_3c_force<PAT_SP, PAT_SP, HASD, DOGS, FUSE>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c_force<PAT_SP, PAT_S, HASD, DOGS, FUSE>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c_force<PAT_S, PAT_SP, HASD, DOGS, FUSE>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c_force<PAT_S, PAT_S, HASD, DOGS, FUSE>(c, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_3c_force<PAT_SPD, PAT_SPD, HASD, DOGS, FUSE>(c, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_3c_force<PAT_SPD, PAT_SP, HASD, DOGS, FUSE>(c, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_3c_force<PAT_SP, PAT_SPD, HASD, DOGS, FUSE>(c, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_3c_force<PAT_SPD, PAT_S, HASD, DOGS, FUSE>(c, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_3c_force<PAT_S, PAT_SPD, HASD, DOGS, FUSE>(c, t);
        }
    }
  });
}

// The instantiations (HASD, DOGS) and the fused Harris value + force
// kernels (HASD) of k_dassemble_3c build as six parts of this source
// (FB_IN_PART); part 0 also holds the launcher.
int launch_dassemble_3c_v(int v, const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v0(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v1(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v2(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v3(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v4(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_3c_v5(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s);

#if FB_IN_PART(0)
int launch_dassemble_3c_v(int v, const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  switch (v) {
    case 0: return launch_dassemble_3c_v0(c, q, grid, block, s);
    case 1: return launch_dassemble_3c_v1(c, q, grid, block, s);
    case 2: return launch_dassemble_3c_v2(c, q, grid, block, s);
    case 3: return launch_dassemble_3c_v3(c, q, grid, block, s);
    case 4: return launch_dassemble_3c_v4(c, q, grid, block, s);
    case 5: return launch_dassemble_3c_v5(c, q, grid, block, s);
  }
  return (int)cudaErrorInvalidValue;
}

int launch_dassemble_3c(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d3c, (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block, q);
  if (e) return e;
  int v = (a.have_d ? 2 : 0) + (a.dogs ? 1 : 0);
  if (a.fuse_value && !a.dogs) v = a.have_d ? 5 : 4;
  return launch_dassemble_3c_v(v, c, q, grid, block, s);
}
#endif

#if FB_IN_PART(0)
int launch_dassemble_3c_v0(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<false, false, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(1)
int launch_dassemble_3c_v1(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<false, true, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(2)
int launch_dassemble_3c_v2(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<true, false, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(3)
int launch_dassemble_3c_v3(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<true, true, false><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(4)
int launch_dassemble_3c_v4(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<false, false, true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(5)
int launch_dassemble_3c_v5(const Ctx3c &c, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_3c<true, false, true><<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

}  // namespace fb
