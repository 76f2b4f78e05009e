// fb_dogs_df.cu -- sm_103a DOGS three-center kernels (assemble_vna_3c,
// j.ASSEMBLERS/M_assemble_3c_DOGS.f90:158-322; Dassemble_vna_3c,
// k.DASSEMBLERS/M_Dassemble_3c_DOGS.f90:136-520) with the table
// contractions, rotations and their derivatives in double-float on the FP32
// pipe, as the Harris three-center kernels do.  The smoothers, the monopole
// terms and everything contracted from the per-pair sums stay in FP64: they
// are a few scalars per triplet.
//
// The charged shells of ialpha enter as sum_isorp dq (stinky X_isorp +
// (1 - stinky) emnpl).  The sub-cells are linear in their tables, so the
// dq-weighted sum of the sub-cell interpolations, scaled by stinky, is added
// to the neutral table's before the one rotation (value pass) or derivative
// rotation (force pass).
#include "fb_common_df.cuh"

namespace fb {

namespace {

// smoother geometry of a triplet (M_assemble_3c_DOGS.f90:198-226): the
// distances of ialpha to both ends, their unit vectors, stinky and, for the
// force pass, its derivatives with respect to ialpha (A) and iatom (B)
struct Stinky {
  double d13, d23, stinky, rA1[3], rA2[3], dA[3], dB[3];
};

__device__ __forceinline__ void stinky_of(const FdataDev &fd, const GeomFP64 &h, int in1, int in2, int indna,
                                          bool deriv, Stinky &s) {
  double v2[3];
  s.d13 = 0.0;
  s.d23 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    v2[k] = h.v[k] - h.r21[k];  // rna - r2
    s.d13 += h.v[k] * h.v[k];
    s.d23 += v2[k] * v2[k];
  }
  s.d13 = sqrt(s.d13);
  s.d23 = sqrt(s.d23);
  double rc3 = fd.sp[indna].rcmin;
  double rend1 = fd.sp[in1].rcmin + rc3, rend2 = fd.sp[in2].rcmin + rc3;
  double s13 = smoother(s.d13, rend1, 0.8), s23 = smoother(s.d23, rend2, 0.8);
  s.stinky = s13 * s23;
  if (!deriv) return;
  double ds13 = dsmoother(s.d13, rend1, 0.8), ds23 = dsmoother(s.d23, rend2, 0.8);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s.rA1[k] = s.d13 > 1.0e-5 ? h.v[k] / s.d13 : 0.0;
    s.rA2[k] = s.d23 > 1.0e-5 ? v2[k] / s.d23 : 0.0;
    s.dB[k] = -ds13 * s23 * s.rA1[k];
    double dC = -s13 * ds23 * s.rA2[k];
    s.dA[k] = -s.dB[k] - dC;
  }
}

template <int PA, int PB>
__device__ __forceinline__ void trip_3c_dogs_df(const Ctx3c &c, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  GeomFP64 h;
  trip_geom_fp64(c, t, h);
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[h.iat], in2 = c.isp[h.jat], indna = c.isp[h.ia];
  Stinky sk;
  stinky_of(fd, h, in1, in2, indna, false, sk);
  df cost0 = trip_cost_df(h);
  df F[NE], G[NE];
  interp3c_df<NE, false>(c, fd.c3[in1][in2][indna], h.x, h.z, cost0, F, nullptr, nullptr, nullptr);
  int nssh = fd.sp[indna].nssh;
  double dsum = 0.0;
  df st = df_from(sk.stinky);
#pragma unroll 1
  for (int isorp = 0; isorp < nssh; isorp++) {
    interp3c_df<NE, false>(c, fd.c3s[in1][in2][indna][isorp], h.x, h.z, cost0, G, nullptr, nullptr, nullptr);
    double dq = c.dq[h.ia * MAXSUB + isorp];
    dsum += dq;
    df w = st * df_from(dq);
#pragma unroll
    for (int e = 0; e < NE; e++) F[e] = F[e] + w * G[e];
  }
  GeomDF g;
  trip_geom_df_from(h, g);
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
  long long o = c.blk_off[c.tdst[t]];
  const double *Sb = c.S + o, *Db = c.dip + o;
  double *dst = c.vb + o;
  const df peq2 = peq2_df();
  // the effective monopole of the pair, (S/2 - dip/z)/d13 + (S/2 + dip/z)/d23,
  // for the (1 - stinky) part of every charged shell
  double wm = dsum * (1.0 - sk.stinky) * P_eq2;
#pragma unroll
  for (int q = 0; q < NA * NB; q++) {
    double sterm = Sb[q] / 2.0, dterm = Db[q] / h.z;
    double emnpl = (sterm - dterm) / sk.d13 + (sterm + dterm) / sk.d23;
    atomicAdd(dst + q, df_to(X[q] * peq2) + wm * emnpl);
  }
}

template <int PA, int PB>
__device__ void trip_3c_force_dogs_df(const Ctx3c &c, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  GeomFP64 h;
  trip_geom_fp64(c, t, h);
  const int ia = h.ia, iat = h.iat, jat = h.jat;
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
  Stinky sk;
  stinky_of(fd, h, in1, in2, indna, true, sk);
  df cost0 = trip_cost_df(h);
  df F[NE], DpF[NE], DxF[NE], DyF[NE], Fq[NE];
  interp3c_df<NE, true>(c, fd.c3[in1][in2][indna], h.x, h.z, cost0, F, DpF, DxF, DyF);
  // the charged shells: Fq = sum dq sub-cell (values, for the dstinky
  // term), and stinky times the same sum (values and derivatives) added to
  // the neutral table's
#pragma unroll
  for (int e = 0; e < NE; e++) Fq[e] = df_zero();
  int nssh = fd.sp[indna].nssh;
  double dsum = 0.0;
  {
    df st = df_from(sk.stinky);
    df Gq[NE], Gp[NE], Gx[NE], Gy[NE];
#pragma unroll 1
    for (int isorp = 0; isorp < nssh; isorp++) {
      interp3c_df<NE, true>(c, fd.c3s[in1][in2][indna][isorp], h.x, h.z, cost0, Gq, Gp, Gx, Gy);
      double dqv = c.dq[ia * MAXSUB + isorp];
      dsum += dqv;
      df dq = df_from(dqv), w = st * dq;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        Fq[e] = Fq[e] + dq * Gq[e];
        F[e] = F[e] + w * Gq[e];
        DpF[e] = DpF[e] + w * Gp[e];
        DxF[e] = DxF[e] + w * Gx[e];
        DyF[e] = DyF[e] + w * Gy[e];
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
      Fq[ee] = Fq[ee] * sint;
    }
  });
  RotDF R;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = g.e[pperm(a)][pperm(b)];
  int p = c.tdst[t];
  const df *rho = c.rho_df + c.blk_off[p];
  df rb[NA * NB], Gf[NA * NB], G[NE];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) rb[q] = rho[q];
  mol_density_df<PA, PB>(R, rb, Gf, G);
  df Sx = df_zero(), Sy = df_zero(), Sp = df_zero(), Cx = df_zero();
#pragma unroll
  for (int e = 0; e < NE; e++) {
    Sx = Sx + DxF[e] * G[e];
    Sy = Sy + DyF[e] * G[e];
    Sp = Sp + DpF[e] * G[e];
    Cx = Cx + Fq[e] * G[e];
  }
  // sum rho rot(Fq) and the monopole terms from the per-pair sums rho S,
  // rho dip, rho dS, rho ddip (FP64, M_Dassemble_3c_DOGS.f90:440-520)
  double cx = df_to(Cx);
  const double *ps = c.dogs_ps + 8 * (long long)p;
  double sterm = 0.5 * ps[0], dterm = ps[1] / h.z;
  double am = sterm - dterm, ap = sterm + dterm;
  double emnpl = am / sk.d13 + ap / sk.d23;
  double i13 = 1.0 / (sk.d13 * sk.d13), i23 = 1.0 / (sk.d23 * sk.d23);
  df hA[3], hB[3];
  frame_terms_3c_df<PA, PB>(g, Gf, F, hA, hB);
  const df peq2 = peq2_df();
  double fa[3], fb[3];
#pragma unroll 1
  for (int q = 0; q < 3; q++) {
    df amt = (g.x > 1.0e-5) ? (sel3(g.sig, q) - cost * sel3(g.rh, q)) * g.ix : df_zero();
    df bmt = (cost * sel3(g.sig, q) - sel3(g.rh, q)) * iz;
    df ga = sel3(g.rh, q) * Sx + amt * Sp;
    df sa = sel3(hA, q) + ga;
    df sb = sel3(hB, q) + ((bmt * Sp - sel3(g.sig, q) * Sy) - ga * 0.5f);
    double va = -df_to(sa * peq2), vb = -df_to(sb * peq2);
    // DOGS extras
    double spterm = 0.5 * ps[2 + q];
    double sigq = df_to(sel3(g.sig, q));
    double dpterm = ps[5 + q] / h.z + dterm * sigq / h.z;
    double eA = -am * sk.rA1[q] * i13 - ap * sk.rA2[q] * i23;
    double eB = am * sk.rA1[q] * i13 + (spterm - dpterm) / sk.d13 + (spterm + dpterm) / sk.d23;
    va -= P_eq2 * (sk.dA[q] * cx - dsum * sk.dA[q] * emnpl + dsum * (1.0 - sk.stinky) * eA);
    vb -= P_eq2 * (sk.dB[q] * cx - dsum * sk.dB[q] * emnpl + dsum * (1.0 - sk.stinky) * eB);
    fa[0] = q == 0 ? va : fa[0];
    fa[1] = q == 1 ? va : fa[1];
    fa[2] = q == 2 ? va : fa[2];
    fb[0] = q == 0 ? vb : fb[0];
    fb[1] = q == 1 ? vb : fb[1];
    fb[2] = q == 2 ? vb : fb[2];
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(c.f3naa + 3 * ia + q, fa[q]);
    atomicAdd(c.f3nab + 3 * iat + q, fb[q]);
    atomicAdd(c.f3nac + 3 * jat + q, -fa[q] - fb[q]);
  }
}

__global__ void __launch_bounds__(256) k_assemble_3c_dogs_df(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    switch (pa * 3 + pb) {
      case PAT_SP * 3 + PAT_SP: trip_3c_dogs_df<PAT_SP, PAT_SP>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c_dogs_df<PAT_SP, PAT_S>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c_dogs_df<PAT_S, PAT_SP>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c_dogs_df<PAT_S, PAT_S>(c, t); break;
      default: break;
    }
  });
}

__global__ void __launch_bounds__(256) k_dassemble_3c_dogs_df(Ctx3c c, Sched q) {
  for_each_item(c.T, q, [&](int t) {
    if (c.tperm) t = c.tperm[t];
    int pa = c.fd->sp[c.isp[c.ci_j[t]]].pattern, pb = c.fd->sp[c.isp[c.cj_j[t]]].pattern;
    switch (pa * 3 + pb) {
      case PAT_SP * 3 + PAT_SP: trip_3c_force_dogs_df<PAT_SP, PAT_SP>(c, t); break;
      case PAT_SP * 3 + PAT_S: trip_3c_force_dogs_df<PAT_SP, PAT_S>(c, t); break;
      case PAT_S * 3 + PAT_SP: trip_3c_force_dogs_df<PAT_S, PAT_SP>(c, t); break;
      case PAT_S * 3 + PAT_S: trip_3c_force_dogs_df<PAT_S, PAT_S>(c, t); break;
      default: break;
    }
  });
}

}  // namespace

int launch_assemble_3c_dogs_df(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_a3c, (long long)a.ntrip, a.queue ? a.queue + 1 : nullptr, s, grid, block, q);
  if (e) return e;
  k_assemble_3c_dogs_df<<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dassemble_3c_dogs_df(const AsmArgs &a, cudaStream_t s) {
  if (a.ntrip == 0) return 0;
  Ctx3c c = make3c(a);
  dim3 grid, block;
  Sched q;
  int e = sched_launch(a.cfg_d3c, (long long)a.ntrip, a.queue ? a.queue + 3 : nullptr, s, grid, block, q);
  if (e) return e;
  k_dassemble_3c_dogs_df<<<grid, block, 0, s>>>(c, q);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
