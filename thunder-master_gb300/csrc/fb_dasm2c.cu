// fb_dasm2c.cu -- sm_103a kernel of the 2c force derivatives.
#include "fb_common.cuh"

namespace fb {

// what: 1 overlap, 2 kinetic, 4 vna ontop + atom, 8 (DOGS) the pair sums
// the 3c pass reads.  With DOGS the ontop terms add the charged-shell
// sub-cells weighted by the shell charges (linear, so the weighted tables
// go through one derivative rotation), and the atom term adds the smoothed
// charged shells with the smoother and monopole derivatives
// (M_Dassemble_2c_DOGS.f90:780-1196); sig = sum rho(i,self) S(i,self).
// RATES (s and p shells, no DOGS, no explicit derivative blocks): the
// frame-derivative terms through the rotation rates of the pair frame
// (frame_rates_2c, contract_rates) instead of Depsilon_2c and Dtwister's dL.
// Pairs in epsilon's collinear fallback frame, and calls that keep the
// derivative blocks (FB_KEEP_DBLOCKS), take the literal path (pair_d2c_at).
template <int PA, int PB, bool HASD, bool DOGS, bool RATES>
__device__ __forceinline__ void pair_d2c(const CtxD2c &c, int i, int p, unsigned what, double sig,
                                         const double *r1, const double *r2, double z, const double (*e)[3]) {
  using PL = Plan<PA, PB, K2C>;
  using PLA = Plan<PA, PA, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n, NEA = PLA::m.n;
  static_assert(!RATES || (!HASD && !DOGS), "rotation rates: s and p shells, no DOGS terms");
  const Ctx2c &b = c.b;
  int j = b.neigh_j[p];
  int in1 = b.isp[i], in2 = b.isp[j];
  double ee[3][3];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int k = 0; k < 3; k++) ee[a][k] = e[a][k];
  RotM R;
  DRotM D;
  twister<HASD>(ee, R);
  if constexpr (!RATES) {
    double dd[3][3][3];
    depsilon_2c(r1, r2, z, ee, dd);
    dtwister<HASD>(ee, dd, D);
  }
  double W[3][3];
  if constexpr (RATES) frame_rates_2c(r1, r2, z, ee, W);
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
    if (!RATES && c.keep) {
      double Xd[3 * NA * NB];
      drotate_plan<PA, PB, K2C>(R, D, v, vd, Xd);
#pragma unroll
      for (int q = 0; q < 3 * NA * NB; q++) c.dS[3 * o + q] = Xd[q];
    }
    double cb[NA * NB];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) cb[q] = __ldg(c.cape + o + q);
    if constexpr (RATES) {
      double Gf[NA * NB];
      mol_G_full<PA, PB>(R, cb, Gf);
      contract_rates<PA, PB, K2C>(Gf, W, v, vd, out);
    } else {
      contract<PA, PB, K2C, HASD>(R, D, cb, v, vd, out);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) c.sumS[3 * p + q] = out[q];
  }
  // the kinetic and on-top vna terms contract with the same density block:
  // the literal form takes its molecular-frame form (with H) once; the
  // rotation-rate form recomputes the cheaper L^T rho L at each use (fewer
  // live registers)
  MolRho<PA, PB, K2C> Grb;
  if constexpr (!RATES)
    if ((what & 2u) || ((what & 4u) && !self)) mol_rho<PA, PB, K2C>(R, D, rb, Grb);
  if (what & 2u) {
    interp2c_d<NE>(b.table2c, fd.c2[in1][in2][1], z, tiny, v, dv, b.status);
    vec2c<NE>(z, eta, dv, vd);
    if (!RATES && c.keep) {
      double Xd[3 * NA * NB];
      drotate_plan<PA, PB, K2C>(R, D, v, vd, Xd);
#pragma unroll
      for (int q = 0; q < 3 * NA * NB; q++) c.dT[3 * o + q] = Xd[q];
    }
    if constexpr (RATES) {
      double Grf[NA * NB];
      mol_G_full<PA, PB>(R, rb, Grf);
      contract_rates<PA, PB, K2C>(Grf, W, v, vd, out);
    } else {
      contract_g<PA, PB, K2C>(Grb, v, vd, out);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) c.sumT[3 * p + q] = out[q];
  }
  if (what & 4u) {
    double f[3] = {0.0, 0.0, 0.0};
    if (!self) {
      // ontop left + right are summed before one contraction (linear)
      double m[NE], dm[NE];
#pragma unroll
      for (int e = 0; e < NE; e++) m[e] = dm[e] = 0.0;
#pragma unroll
      for (int w2 = 2; w2 <= 3; w2++) {
        interp2c_d<NE>(b.table2c, fd.c2[in1][in2][w2], z, tiny, v, dv, b.status);
        if constexpr (DOGS) {
          int owner = w2 == 2 ? i : j, nsh = fd.sp[w2 == 2 ? in1 : in2].nssh;
          double vs[NE], dvs[NE];
#pragma unroll 1
          for (int isorp = 1; isorp <= nsh; isorp++) {
            interp2c_d<NE>(b.table2c, fd.c2s[in1][in2][w2 - 2][isorp - 1], z, tiny, vs, dvs, b.status);
            double dq = b.dq[owner * MAXSUB + isorp - 1];
#pragma unroll
            for (int e = 0; e < NE; e++) {
              v[e] = fma(dq, vs[e], v[e]);
              dv[e] = fma(dq, dvs[e], dv[e]);
            }
          }
        }
#pragma unroll
        for (int e = 0; e < NE; e++) m[e] += v[e], dm[e] += dv[e];
      }
      vec2c<NE>(z, eta, dm, vd);
      if constexpr (RATES) {
        double Grf[NA * NB];
        mol_G_full<PA, PB>(R, rb, Grf);
        contract_rates<PA, PB, K2C>(Grf, W, m, vd, out);
      } else {
        contract_g<PA, PB, K2C>(Grb, m, vd, out);
      }
#pragma unroll
      for (int q = 0; q < 3; q++) f[q] -= out[q] * P_eq2;
    }
#pragma unroll
    for (int q = 0; q < 3; q++) c.ontop[3 * p + q] = f[q];
    // atom case, contracted with rho of the self block of i
    interp2c_d<NEA>(b.table2c, fd.c2[in1][in2][4], z, tiny, v, dv, b.status);
    vec2c<NEA>(z, eta, dv, vd);
    double rs[NA * NA];
    long long os = b.blk_off[b.pair_off[i] + max(b.neigh_self[i], 0)];
#pragma unroll
    for (int q = 0; q < NA * NA; q++) rs[q] = __ldg(c.rho + os + q);
    if constexpr (RATES) {
      double Gs[NA * NA];
      mol_G_full<PA, PA>(R, rs, Gs);
      contract_rates<PA, PA, K2C>(Gs, W, v, vd, out);
    } else {
      contract<PA, PA, K2C, HASD>(R, D, rs, v, vd, out);
    }
    if constexpr (DOGS) {
      // charged shells of jatom, smoothed: sum of dq * (smooth dX - eta
      // dsmooth X + (1 - smooth) d(S/z) + eta dsmooth S/z) contracted with
      // rho(i, self)
      double rend = fd.sp[in1].rcmin + fd.sp[in2].rcmin;
      double smooth = smoother(z, rend, 0.8), dsm = dsmoother(z, rend, 0.8);
      double M[NEA], dM[NEA], vs[NEA], dvs[NEA], dsum = 0.0;
#pragma unroll
      for (int e = 0; e < NEA; e++) M[e] = dM[e] = 0.0;
#pragma unroll 1
      for (int isorp = 1; isorp <= fd.sp[in2].nssh; isorp++) {
        interp2c_d<NEA>(b.table2c, fd.c2s[in1][in2][2][isorp - 1], z, tiny, vs, dvs, b.status);
        double dq = b.dq[j * MAXSUB + isorp - 1];
        dsum += dq;
#pragma unroll
        for (int e = 0; e < NEA; e++) {
          M[e] = fma(dq, vs[e], M[e]);
          dM[e] = fma(dq, dvs[e], dM[e]);
        }
      }
      bool on = z > 1.0e-4;
      double vm[NEA], vdm[3 * NEA];
#pragma unroll
      for (int e = 0; e < NEA; e++) {
        vm[e] = smooth * M[e];
#pragma unroll
        for (int k = 0; k < 3; k++) vdm[k + 3 * e] = on ? -eta[k] * (smooth * dM[e]) : 0.0;
      }
      MolRho<PA, PA, K2C> Gs;
      mol_rho<PA, PA, K2C>(R, D, rs, Gs);
      double cx = 0.0;
#pragma unroll
      for (int e = 0; e < NEA; e++) cx = fma(M[e], Gs.G[e], cx);
      double mono = 0.0, dmono = 0.0;  // sum rho S/z and sum rho S/z^2
      if (on) {
        mono = sig / z;
        dmono = sig / (z * z);
      }
#pragma unroll
      for (int q = 0; q < 3; q++) {
        double s = 0.0;
#pragma unroll
        for (int e = 0; e < NEA; e++) {
          s = fma(vm[e], Gs.H[q][e], s);
          s = fma(vdm[q + 3 * e], Gs.G[e], s);
        }
        s = s - eta[q] * dsm * cx + dsum * ((1.0 - smooth) * eta[q] * dmono + eta[q] * dsm * mono);
        out[q] += s;
      }
    }
#pragma unroll
    for (int q = 0; q < 3; q++) c.atomf[3 * p + q] = -out[q] * P_eq2;
  }
  if constexpr (DOGS) {
    if (what & 8u) {
      // sum rho S, sum rho dip, sum rho dS, sum rho ddip of this pair: the
      // pieces of the 3c effective monopole and its derivatives
      MolRho<PA, PB, K2C> G;
      mol_rho<PA, PB, K2C>(R, D, rb, G);
      double *ps = c.dogs_ps + 8 * (long long)p;
#pragma unroll
      for (int w = 0; w < 2; w++) {
        const Cell2cDev &cell = w == 0 ? fd.c2[in1][in2][0] : fd.c2dip[in1][in2];
        interp2c_d<NE>(b.table2c, cell, z, tiny, v, dv, b.status);
        vec2c<NE>(z, eta, dv, vd);
        double s0 = 0.0, s3[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int e = 0; e < NE; e++) {
          s0 = fma(v[e], G.G[e], s0);
#pragma unroll
          for (int q = 0; q < 3; q++) s3[q] = fma(v[e], G.H[q][e], fma(vd[q + 3 * e], G.G[e], s3[q]));
        }
        ps[w] = s0;
#pragma unroll
        for (int q = 0; q < 3; q++) ps[2 + 3 * w + q] = s3[q];
      }
    }
  }
}

// the literal form out of line: it runs only for the rare collinear fallback
// frame and for FB_KEEP_DBLOCKS, and a call keeps its registers off the
// rotation-rate path
template <int PA, int PB, bool HASD, bool DOGS>
__device__ __noinline__ void pair_d2c_literal(const CtxD2c &c, int i, int p, unsigned what, double sig) {
  double r1[3], r2[3], z, e[3][3];
  pair_geom(c.b, i, p, r1, r2, z, e);
  pair_d2c<PA, PB, HASD, DOGS, false>(c, i, p, what, sig, r1, r2, z, e);
}

// one pair: its geometry, then the rotation-rate form unless the pair frame is
// epsilon's collinear fallback with non-zero Depsilon_2c derivatives
template <int PA, int PB, bool HASD, bool DOGS>
__device__ __forceinline__ void pair_d2c_at(const CtxD2c &c, int i, int p, unsigned what, double sig) {
  double r1[3], r2[3], z, e[3][3];
  bool estd = pair_geom(c.b, i, p, r1, r2, z, e);
  if constexpr (!HASD && !DOGS) {
    double cm;
    if (!c.keep && (estd || frame2c_degenerate(r1, r2, z, cm))) {
      pair_d2c<PA, PB, HASD, DOGS, true>(c, i, p, what, sig, r1, r2, z, e);
    } else {
      pair_d2c_literal<PA, PB, HASD, DOGS>(c, i, p, what, sig);
    }
  } else {
    pair_d2c<PA, PB, HASD, DOGS, false>(c, i, p, what, sig, r1, r2, z, e);
  }
}

template <int PA, bool HASD, bool DOGS>
__device__ void atom_d2c(const CtxD2c &c, int i, int lane, unsigned what) {
  int p0 = c.b.pair_off[i], p1 = c.b.pair_off[i + 1];
  double sig = 0.0;
  if (DOGS && (what & 4u)) {
    // sum rho(i, self) S(i, self): the self overlap block, interpolated and
    // rotated as the overlap pass does, contracted with rho of the self block
    using PLA = Plan<PA, PA, K2C>;
    constexpr int NA = PLA::NA;
    int ps = p0 + max(c.b.neigh_self[i], 0);
    double r1[3], r2[3], z, e[3][3];
    pair_geom(c.b, i, ps, r1, r2, z, e);
    RotM R;
    twister<HASD>(e, R);
    const Cell2cDev &cell = c.b.fd->c2[c.b.isp[i]][c.b.isp[i]][0];
    double w[7], v[PLA::m.n], X[NA * NA];
    int i0 = 0;
    lagrange7(z, cell, i0, w, nullptr);
    interp2c<PLA::m.n>(c.b.table2c, cell, i0, w, v);
    rotate_plan<PA, PA, K2C>(R, v, X);
    long long os = c.b.blk_off[ps];
#pragma unroll
    for (int q = 0; q < NA * NA; q++) sig = fma(__ldg(c.rho + os + q), X[q], sig);
  }
  for (int p = p0 + lane; p < p1; p += 32) {
    int pb = c.b.fd->sp[c.b.isp[c.b.neigh_j[p]]].pattern;
    if (pb == PAT_SP) pair_d2c_at<PA, PAT_SP, HASD, DOGS>(c, i, p, what, sig);
    else if (pb == PAT_S) pair_d2c_at<PA, PAT_S, HASD, DOGS>(c, i, p, what, sig);
    else if constexpr (HASD) pair_d2c_at<PA, PAT_SPD, HASD, DOGS>(c, i, p, what, sig);
  }
}

template <int PA, bool HASD>
__device__ __forceinline__ void pair_d2c_pb(const CtxD2c &c, int i, int p, unsigned what) {
  int pb = c.b.fd->sp[c.b.isp[c.b.neigh_j[p]]].pattern;
  if (pb == PAT_SP) pair_d2c_at<PA, PAT_SP, HASD, false>(c, i, p, what, 0.0);
  else if (pb == PAT_S) pair_d2c_at<PA, PAT_S, HASD, false>(c, i, p, what, 0.0);
  else if constexpr (HASD) pair_d2c_at<PA, PAT_SPD, HASD, false>(c, i, p, what, 0.0);
}

// DOGS: a warp per atom (the atom's self-overlap sum sig enters every pair);
// otherwise a thread per pair, so that no lane idles past the end of an
// atom's pair list
template <bool HASD, bool DOGS>
__global__ void __launch_bounds__(256) k_dassemble_2c(CtxD2c c, unsigned what, Sched q) {
  if constexpr (DOGS) {
    for_each_warp_item(c.b.N, q, [&](int i, int lane) {
      int pa = c.b.fd->sp[c.b.isp[i]].pattern;
      if (pa == PAT_SP) atom_d2c<PAT_SP, HASD, DOGS>(c, i, lane, what);
      else if (pa == PAT_S) atom_d2c<PAT_S, HASD, DOGS>(c, i, lane, what);
      else if constexpr (HASD) atom_d2c<PAT_SPD, HASD, DOGS>(c, i, lane, what);
    });
  } else {
    for_each_item(c.b.P, q, [&](int p) {
      int i = c.b.pair_owner[p];
      int pa = c.b.fd->sp[c.b.isp[i]].pattern;
      if (pa == PAT_SP) pair_d2c_pb<PAT_SP, HASD>(c, i, p, what);
      else if (pa == PAT_S) pair_d2c_pb<PAT_S, HASD>(c, i, p, what);
      else if constexpr (HASD) pair_d2c_pb<PAT_SPD, HASD>(c, i, p, what);
    });
  }
}

// The four instantiations (HASD, DOGS) of k_dassemble_2c build as four parts of
// this source (FB_IN_PART); part 0 also holds the launcher.
int launch_dassemble_2c_v(int v, const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_2c_v0(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_2c_v1(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_2c_v2(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);
int launch_dassemble_2c_v3(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s);

#if FB_IN_PART(0)
int launch_dassemble_2c_v(int v, const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  switch (v) {
    case 0: return launch_dassemble_2c_v0(c, what, q, grid, block, s);
    case 1: return launch_dassemble_2c_v1(c, what, q, grid, block, s);
    case 2: return launch_dassemble_2c_v2(c, what, q, grid, block, s);
    case 3: return launch_dassemble_2c_v3(c, what, q, grid, block, s);
  }
  return (int)cudaErrorInvalidValue;
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
  c.dogs_ps = a.dogs_ps;
  dim3 grid, block;
  Sched q;
  long long work = a.dogs ? (long long)a.N * 32 : (long long)a.P;
  int e = sched_launch(a.cfg_d2c, work, a.queue ? a.queue + 2 : nullptr, s, grid, block, q);
  if (e) return e;
  int v = (a.have_d ? 2 : 0) + (a.dogs ? 1 : 0);
  return launch_dassemble_2c_v(v, c, what, q, grid, block, s);
}
#endif

#if FB_IN_PART(0)
int launch_dassemble_2c_v0(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_2c<false, false><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(1)
int launch_dassemble_2c_v1(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_2c<false, true><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(2)
int launch_dassemble_2c_v2(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_2c<true, false><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(3)
int launch_dassemble_2c_v3(const CtxD2c &c, unsigned what, Sched q, dim3 grid, dim3 block, cudaStream_t s) {
  k_dassemble_2c<true, true><<<grid, block, 0, s>>>(c, what, q);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

}  // namespace fb
