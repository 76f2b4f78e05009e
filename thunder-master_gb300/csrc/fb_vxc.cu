// fb_vxc.cu -- sm_103a kernels of the McWEDA exchange-correlation assembly,
// Harris (PRB 71, 235101 (2005)):
//   k_rho_2c  assemble_rho_2c + assemble_rho_weighted_2c
//             (j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90:81-276, :427-622)
//   k_rho_3c  assemble_rho_3c + assemble_rho_weighted_3c (:298-403, :645-741)
//   k_vxc     assemble_vxc_SN + assemble_vxc_bond + vxc = bond + SN - SN_bond
//             (j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90:102-640)
// All FP64.  The density sub-cells of one pair share the pair's grid and
// frame, so the Qneutral-weighted sum over the shells is taken in the
// molecular frame and rotated once (the rotation is linear).
#include "fb_common.cuh"
#include "fb_vxc.h"

namespace fb {

namespace {

constexpr int cmax(int a, int b) { return a > b ? a : b; }

// lda_ceperley_alder (g.XC_FUNCTIONALS/lda_ceperley_alder.f90:56-190):
// muxc (eV), dmuxc and d2muxc (eV A^3, eV A^6).  The low-density branch's
// d2dec keeps the reference's (dden*3) factor (:142).
struct Lda {
  double muxc, dmuxc, d2muxc;
};

__device__ __forceinline__ Lda lda_ca(double rh) {
  const double a3 = P_abohr * P_abohr * P_abohr;
  double rhx = sqrt(rh * rh + 1.0e-6);
  double rho = rhx * a3;
  double rho_third = pow(rho, 1.0 / 3.0);
  double rs = 0.62035049 / rho_third;
  double exc, muxc, dec, ddec, d2dec;
  if (rho < 0.23873241) {
    double sqrs = sqrt(rs);
    double den = 1.0 + 1.0529 * sqrs + 0.3334 * rs;
    exc = -0.4581652 / rs - 0.1423 / den;
    muxc = exc - rs * (0.15273333 / (rs * rs) + (0.02497128 / sqrs + 0.01581427) / (den * den));
    double dden = 1.0529 / (2.0 * sqrs) + 0.3334;
    double d2den = (-0.5) * 1.0529 / (2.0 * rs * sqrs);
    double d3den = 0.75 * 1.0529 / (2.0 * (rs * rs) * sqrs);
    dec = 0.1423 * dden / (den * den);
    ddec = -2.0 * 0.1423 * dden * dden / (den * den * den) + 0.1423 * d2den / (den * den);
    d2dec = 6.0 * 0.1423 * (dden * 3) / (den * den * den * den) - 6.0 * 0.1423 * dden * d2den / (den * den * den) +
            0.1423 * d3den / (den * den);
  } else {
    double rsl = log(rs);
    exc = -0.4581652 / rs - 0.0480 + 0.0311 * rsl - 0.0116 * rs + 0.002 * rs * rsl;
    muxc = exc - rs * (0.15273333 / (rs * rs) + 0.01036667 / rs - 0.003866667 + 0.00066667 * (1.0 + rsl));
    dec = 0.0311 / rs - 0.0116 + 0.0020 * (rsl + 1.0);
    ddec = -0.0311 / (rs * rs) + 0.0020 / rs;
    d2dec = 2.0 * 0.0311 / (rs * rs * rs) - 0.0020 / (rs * rs);
  }
  double ex = -0.7385587664 * rho_third;
  double dexc = (muxc - exc) / rho;
  double r2 = rho * rho, r3 = r2 * rho;
  double d2nec = (4.0 * rs / (9.0 * r2)) * dec + (rs * rs / (9.0 * r2)) * ddec;
  double d2nex = -(2.0 / (9.0 * r2)) * ex;
  double dmuxc = 2.0 * dexc + rho * (d2nex + d2nec);
  double d3nec = (-28.0 * rs / (27.0 * r3)) * dec + (-4.0 * rs * rs / (9.0 * r3)) * ddec +
                 ((rs * rs * rs) / (-27.0 * r3)) * d2dec;
  double d3nex = (10.0 / (27.0 * r3)) * ex;
  double d2muxc = 3.0 * (d2nex + d2nec) + rho * (d3nex + d3nec);
  Lda o;
  o.muxc = muxc * P_Hartree;
  o.dmuxc = dmuxc * P_Hartree * a3;
  o.d2muxc = d2muxc * P_Hartree * (a3 * a3);
  return o;
}

// ---------------------------------------------------------------------------
// rho 2c: one warp per atom i, one lane per pair
// ---------------------------------------------------------------------------
template <int PA, int PB, bool HASD>
__device__ __forceinline__ void pair_rho2c(const Ctx2c &c, const VxcArgs &v, int i, int p, double *Xatom,
                                           double *Watom) {
  using PL = Plan<PA, PB, K2C>;
  using PLA = Plan<PA, PA, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n, NEA = PLA::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB);
  const FdataDev &fd = *c.fd;
  int j = c.neigh_j[p];
  int in1 = c.isp[i], in2 = c.isp[j];
  double r1[3], r2[3], z, e[3][3];
  pair_geom(c, i, p, r1, r2, z, e);
  RotM R;
  twister<HASD>(e, R);
  bool self = (i == j && c.neigh_b[p] == 0);
  constexpr int NT = cmax(cmax(NE, NEA), cmax(SA * SB, SA * SA));
  double w[7], t[NT];
  int i0 = 0;
  const Cell2cDev *last = nullptr;
  auto weights = [&](const Cell2cDev &cell) {
    if (z > cell.xmax * (1.0 + 1.0e-5)) atomicOr(c.status, DEVERR_XLARGE);
    if (!last || !same_grid(*last, cell)) lagrange7(z, cell, i0, w, nullptr);
    last = &cell;
  };
  const double *qi = fd.sp[in1].qn, *qj = fd.sp[in2].qn;
  double *W_in = v.wrho_in + (long long)VXC_WSH * p, *W_bo = v.wrho_bond + (long long)VXC_WSH * p;
  if (!self) {
    // ontop left (shells of i) + right (shells of j), :186-218
    double m[NE];
#pragma unroll
    for (int q = 0; q < NE; q++) m[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SA; isorp++) {
      const Cell2cDev &cl = fd.c2rho[in1][in2][0][isorp];
      weights(cl);
      interp2c<NE>(c.table2c, cl, i0, w, t);
#pragma unroll
      for (int q = 0; q < NE; q++) m[q] = fma(t[q], qi[isorp], m[q]);
    }
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      const Cell2cDev &cr = fd.c2rho[in1][in2][1][isorp];
      weights(cr);
      interp2c<NE>(c.table2c, cr, i0, w, t);
#pragma unroll
      for (int q = 0; q < NE; q++) m[q] = fma(t[q], qj[isorp], m[q]);
    }
    double X[NA * NB];
    rotate_plan<PA, PB, K2C>(R, m, X);
    long long o = c.blk_off[p];
#pragma unroll
    for (int q = 0; q < NA * NB; q++) {
      v.rho_in[o + q] = X[q];
      v.rho_bond[o + q] = X[q];
    }
    // shell-level ontop (no rotation), :524-555
    double ws[SA * SB];
#pragma unroll
    for (int q = 0; q < SA * SB; q++) ws[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SA; isorp++) {
      const Cell2cDev &cl = fd.c2rho[in1][in2][3][isorp];
      weights(cl);
      interp2c<SA * SB>(c.table2c, cl, i0, w, t);
#pragma unroll
      for (int q = 0; q < SA * SB; q++) ws[q] = fma(t[q], qi[isorp], ws[q]);
    }
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      const Cell2cDev &cr = fd.c2rho[in1][in2][4][isorp];
      weights(cr);
      interp2c<SA * SB>(c.table2c, cr, i0, w, t);
#pragma unroll
      for (int q = 0; q < SA * SB; q++) ws[q] = fma(t[q], qj[isorp], ws[q]);
    }
    // channel (a, b) of the shell map is element a + SA b of the block
#pragma unroll
    for (int q = 0; q < VXC_WSH; q++) {
      double val = 0.0;
      if (q < SA * SB) {
        int a = q % SA, b = q / SA;
        val = ws[a * SB + b];
      }
      W_in[q] = val;
      W_bo[q] = val;
    }
  }
  // atom case into the self block: <i|rho_shell(j)|i> rotated with (in1, in1)
  {
    double m[NEA];
#pragma unroll
    for (int q = 0; q < NEA; q++) m[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      const Cell2cDev &ca = fd.c2rho[in1][in2][2][isorp];
      weights(ca);
      interp2c<NEA>(c.table2c, ca, i0, w, t);
#pragma unroll
      for (int q = 0; q < NEA; q++) m[q] = fma(t[q], qj[isorp], m[q]);
    }
    double XA[NA * NA];
    rotate_plan<PA, PA, K2C>(R, m, XA);
#pragma unroll
    for (int q = 0; q < NA * NA; q++) Xatom[q] += XA[q];
    double ws[SA * SA];
#pragma unroll
    for (int q = 0; q < SA * SA; q++) ws[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      const Cell2cDev &ca = fd.c2rho[in1][in2][5][isorp];
      weights(ca);
      interp2c<SA * SA>(c.table2c, ca, i0, w, t);
#pragma unroll
      for (int q = 0; q < SA * SA; q++) ws[q] = fma(t[q], qj[isorp], ws[q]);
    }
#pragma unroll
    for (int q = 0; q < SA * SA; q++) Watom[q] += ws[(q % SA) * SA + q / SA];
    if (self) {
      // rho_bond of the self block takes only the atom's own term
      long long o = c.blk_off[p];
#pragma unroll
      for (int q = 0; q < NA * NA; q++) v.rho_bond[o + q] = XA[q];
#pragma unroll
      for (int q = 0; q < VXC_WSH; q++) W_bo[q] = q < SA * SA ? ws[(q % SA) * SA + q / SA] : 0.0;
    }
  }
}

template <int PA, bool HASD>
__device__ void atom_rho2c(const Ctx2c &c, const VxcArgs &v, int i, int lane) {
  constexpr int NA = pat_norb(PA), SA = pat_nssh(PA);
  double Xatom[NA * NA], Watom[SA * SA];
#pragma unroll
  for (int q = 0; q < NA * NA; q++) Xatom[q] = 0.0;
#pragma unroll
  for (int q = 0; q < SA * SA; q++) Watom[q] = 0.0;
  int p0 = c.pair_off[i], p1 = c.pair_off[i + 1];
  for (int p = p0 + lane; p < p1; p += 32) {
    int pb = c.fd->sp[c.isp[c.neigh_j[p]]].pattern;
    if (pb == PAT_SP) pair_rho2c<PA, PAT_SP, HASD>(c, v, i, p, Xatom, Watom);
    else if (pb == PAT_S) pair_rho2c<PA, PAT_S, HASD>(c, v, i, p, Xatom, Watom);
    else if constexpr (HASD) pair_rho2c<PA, PAT_SPD, HASD>(c, v, i, p, Xatom, Watom);
  }
#pragma unroll
  for (int q = 0; q < NA * NA; q++)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) Xatom[q] += __shfl_xor_sync(0xffffffffu, Xatom[q], off);
#pragma unroll
  for (int q = 0; q < SA * SA; q++)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) Watom[q] += __shfl_xor_sync(0xffffffffu, Watom[q], off);
  if (lane == 0) {
    int ps = p0 + c.neigh_self[i];
    long long os = c.blk_off[ps];
#pragma unroll
    for (int q = 0; q < NA * NA; q++) v.rho_in[os + q] = Xatom[q];
#pragma unroll
    for (int q = 0; q < VXC_WSH; q++) v.wrho_in[(long long)VXC_WSH * ps + q] = q < SA * SA ? Watom[q] : 0.0;
  }
}

template <bool HASD>
__global__ void __launch_bounds__(128) k_rho_2c(Ctx2c c, VxcArgs v) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= c.N) return;
  int pa = c.fd->sp[c.isp[i]].pattern;
  if (pa == PAT_SP) atom_rho2c<PAT_SP, HASD>(c, v, i, lane);
  else if (pa == PAT_S) atom_rho2c<PAT_S, HASD>(c, v, i, lane);
  else if constexpr (HASD) atom_rho2c<PAT_SPD, HASD>(c, v, i, lane);
}

// ---------------------------------------------------------------------------
// rho 3c: one thread per triplet, FP64 atomics into the pair (iatom, mneigh)
// ---------------------------------------------------------------------------
// true when the triplet's Qneutral-summed density cells exist and its
// stencil node (the one interp3c takes the gradient switch from) has one
// switch for every sub-cell
__device__ __forceinline__ bool qsum_node_ok(const unsigned char *lin, const Cell3cDev &cell, double x, double y) {
  if (cell.off < 0) return false;
  int ix = (int)(x / cell.dx) + 1, iy = (int)(y / cell.dy) + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > cell.nx - 2) ix = cell.nx - 2;
  if (iy > cell.ny - 2) iy = cell.ny - 2;
  return lin[cell.node_off + (long long)(iy - 1) * cell.nx + (ix - 1)] != 2;
}
__device__ __forceinline__ bool qsum_fast(const Ctx3c &c, int in1, int in2, int in3, double x, double y) {
  const FdataDev &fd = *c.fd;
  return qsum_node_ok(c.lin, fd.c3rhoq[in1][in2][in3][0], x, y) &&
         qsum_node_ok(c.lin, fd.c3rhoq[in1][in2][in3][1], x, y);
}

template <int PA, int PB, bool HASD, bool QSUM>
__device__ __forceinline__ void trip_rho3c(const Ctx3c &c, const VxcArgs &v, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB);
  int ia, iat, jat;
  TripGeom g;
  trip_geom(c, t, ia, iat, jat, g);
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
  if (qsum_fast(c, in1, in2, indna, g.x, g.z) != QSUM) return;
  int nk = fd.sp[indna].nssh;
  const double *qk = fd.sp[indna].qn;
  double m[NE];
  if constexpr (QSUM) {
    interp3c<NE, false>(c, fd.c3rhoq[in1][in2][indna][0], g.x, g.z, g.cost, m, nullptr, nullptr, nullptr);
  } else {
    double F[NE];
#pragma unroll
    for (int q = 0; q < NE; q++) m[q] = 0.0;
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c<NE, false>(c, fd.c3rho[in1][in2][indna][0][isorp], g.x, g.z, g.cost, F, nullptr, nullptr, nullptr);
#pragma unroll
      for (int q = 0; q < NE; q++) m[q] = fma(F[q], qk[isorp], m[q]);
    }
  }
  double sint = sqrt(fmax(1.0e-5, 1.0 - g.cost * g.cost));
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    if constexpr (PL::m.mv[e] == 1) m[e] = m[e] * sint;
  });
  RotM R;
  twister<HASD>(g.e, R);
  double X[NA * NB];
  rotate_plan<PA, PB, K3C>(R, m, X);
  int p = c.tdst[t];
  double *dst = v.rho_in + c.blk_off[p];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) atomicAdd(dst + q, X[q]);
  double ws[SA * SB];
  if constexpr (QSUM) {
    interp3c<SA * SB, false>(c, fd.c3rhoq[in1][in2][indna][1], g.x, g.z, g.cost, ws, nullptr, nullptr, nullptr);
  } else {
    double Fs[SA * SB];
#pragma unroll
    for (int q = 0; q < SA * SB; q++) ws[q] = 0.0;
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c<SA * SB, false>(c, fd.c3rho[in1][in2][indna][1][isorp], g.x, g.z, g.cost, Fs, nullptr, nullptr,
                               nullptr);
#pragma unroll
      for (int q = 0; q < SA * SB; q++) ws[q] = fma(Fs[q], qk[isorp], ws[q]);
    }
  }
  double *wd = v.wrho_in + (long long)VXC_WSH * p;
#pragma unroll
  for (int q = 0; q < SA * SB; q++) atomicAdd(wd + (q / SB) + SA * (q % SB), ws[q]);
}

// triplets in the binned order (tperm) for table locality; QSUM: the
// triplets the summed cells serve (qsum_fast), else the others
template <bool HASD, bool QSUM>
__global__ void __launch_bounds__(128) k_rho_3c(Ctx3c c, VxcArgs v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.T; i += gridDim.x * blockDim.x) {
    int t = c.tperm ? c.tperm[i] : i;
    int in1 = c.isp[c.ci_j[t]], in2 = c.isp[c.cj_j[t]];
    int pa = c.fd->sp[in1].pattern, pb = c.fd->sp[in2].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_rho3c<PAT_SP, PAT_SP, HASD, QSUM>(c, v, t); break;
      case PAT_SP * 3 + PAT_S: trip_rho3c<PAT_SP, PAT_S, HASD, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_SP: trip_rho3c<PAT_S, PAT_SP, HASD, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_S: trip_rho3c<PAT_S, PAT_S, HASD, QSUM>(c, v, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_rho3c<PAT_SPD, PAT_SPD, HASD, QSUM>(c, v, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_rho3c<PAT_SPD, PAT_SP, HASD, QSUM>(c, v, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_rho3c<PAT_SP, PAT_SPD, HASD, QSUM>(c, v, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_rho3c<PAT_SPD, PAT_S, HASD, QSUM>(c, v, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_rho3c<PAT_S, PAT_SPD, HASD, QSUM>(c, v, t);
        }
    }
  }
}

// ---------------------------------------------------------------------------
// vxc: one warp per atom, one lane per pair
// ---------------------------------------------------------------------------
template <int PA, int PB, bool HASD>
__device__ __forceinline__ void pair_vxc(const Ctx2c &c, const VxcArgs &v, int i, int p) {
  using PL = Plan<PA, PB, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB);
  const FdataDev &fd = *c.fd;
  int j = c.neigh_j[p];
  long long o = c.blk_off[p];
  const double *Wi = v.wrho_in + (long long)VXC_WSH * p, *Wb = v.wrho_bond + (long long)VXC_WSH * p;
  const double *S = c.S + o, *ri = v.rho_in + o, *rb = v.rho_bond + o;
  double sn[NA * NB], snb[NA * NB], bond[NA * NB];
  bool self = (i == j && c.neigh_b[p] == 0);
  if (!self) {
    // off-site generalized Sankey-Niklewski (vxc_SN :286-357)
#pragma unroll
    for (int a = 0; a < SA; a++)
#pragma unroll
      for (int b = 0; b < SB; b++) {
        double wi = Wi[a + SA * b], wb = Wb[a + SA * b];
        Lda li = lda_ca(wi), lb = lda_ca(wb);
#pragma unroll
        for (int imu = shell_off(a); imu < shell_off(a) + 2 * a + 1; imu++)
#pragma unroll
          for (int inu = shell_off(b); inu < shell_off(b) + 2 * b + 1; inu++) {
            int q = imu + NA * inu;
            double ov = S[q];
            sn[q] = li.muxc * ov + li.dmuxc * (ri[q] - wi * ov);
            snb[q] = lb.muxc * ov + lb.dmuxc * (rb[q] - wb * ov);
          }
      }
    // vxc_bond: the rotated vxc_ontop table (:612-627)
    double r1[3], r2[3], z, e[3][3];
    pair_geom(c, i, p, r1, r2, z, e);
    RotM R;
    twister<HASD>(e, R);
    const Cell2cDev &cell = fd.c2vxc[c.isp[i]][c.isp[j]];
    if (z > cell.xmax * (1.0 + 1.0e-5)) atomicOr(c.status, DEVERR_XLARGE);
    double w[7], m[NE];
    int i0 = 0;
    lagrange7(z, cell, i0, w, nullptr);
    interp2c<NE>(c.table2c, cell, i0, w, m);
    rotate_plan<PA, PB, K2C>(R, m, bond);
  } else if constexpr (PA == PB) {
    // on-site SN (:365-480): diagonal, then the off-diagonal imu != inu
#pragma unroll
    for (int q = 0; q < NA * NA; q++) sn[q] = snb[q] = bond[q] = 0.0;
#pragma unroll
    for (int a = 0; a < SA; a++) {
      {
        double wi = Wi[a + SA * a], wb = Wb[a + SA * a];
        Lda li = lda_ca(wi), lb = lda_ca(wb);
#pragma unroll
        for (int imu = shell_off(a); imu < shell_off(a) + 2 * a + 1; imu++) {
          int q = imu + NA * imu;
          sn[q] = li.muxc + li.dmuxc * (ri[q] - wi);
          snb[q] = lb.muxc + lb.dmuxc * (rb[q] - wb);
        }
      }
#pragma unroll
      for (int b = 0; b < SA; b++) {
        Lda li = lda_ca(Wi[a + SA * b]), lb = lda_ca(Wb[a + SA * b]);
#pragma unroll
        for (int imu = shell_off(a); imu < shell_off(a) + 2 * a + 1; imu++)
#pragma unroll
          for (int inu = shell_off(b); inu < shell_off(b) + 2 * b + 1; inu++)
            if (imu != inu) {
              int q = imu + NA * inu;
              sn[q] = li.dmuxc * ri[q];
              snb[q] = lb.dmuxc * rb[q];
            }
      }
    }
    // vxc_bond on-site: V(issh, jssh) where l and m agree (:590-605); with
    // one shell per l in these bases that is the diagonal, V(issh, issh)
    const double *V = fd.vxc1c[c.isp[i]];
#pragma unroll
    for (int imu = 0; imu < NA; imu++) {
      int sa = orb_shell(imu);
      bond[imu + NA * imu] = V[sa * MAXSUB + sa];
    }
  }
#pragma unroll
  for (int q = 0; q < NA * NB; q++) v.vxc[o + q] = bond[q] + sn[q] - snb[q];
}

template <int PA, bool HASD>
__device__ void atom_vxc(const Ctx2c &c, const VxcArgs &v, int i, int lane) {
  for (int p = c.pair_off[i] + lane; p < c.pair_off[i + 1]; p += 32) {
    int pb = c.fd->sp[c.isp[c.neigh_j[p]]].pattern;
    if (pb == PAT_SP) pair_vxc<PA, PAT_SP, HASD>(c, v, i, p);
    else if (pb == PAT_S) pair_vxc<PA, PAT_S, HASD>(c, v, i, p);
    else if constexpr (HASD) pair_vxc<PA, PAT_SPD, HASD>(c, v, i, p);
  }
}

template <bool HASD>
__global__ void __launch_bounds__(128) k_vxc(Ctx2c c, VxcArgs v) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= c.N) return;
  int pa = c.fd->sp[c.isp[i]].pattern;
  if (pa == PAT_SP) atom_vxc<PAT_SP, HASD>(c, v, i, lane);
  else if (pa == PAT_S) atom_vxc<PAT_S, HASD>(c, v, i, lane);
  else if constexpr (HASD) atom_vxc<PAT_SPD, HASD>(c, v, i, lane);
}

// ===========================================================================
// force pass (k.DASSEMBLERS/M_Dassemble_vxc_McWEDA_Harris.f90,
// M_Dassemble_rho_McWEDA_Harris.f90, M_Dassemble_vxc_3c_McWEDA_Harris.f90)
// ===========================================================================
// The reference accumulates rho(mu, nu) times per-element combinations of
// the Dblocks of S, rho_in / rho_bond (ontop and atom case) and of the
// weighted densities.  Each Dblock enters linearly, so the per-element
// factors are gathered first into one weight block per Dblock, and every
// weight block is contracted with its table's derivative rotation in the
// molecular frame (contract), the same sums in a different order:
//   off site   wS = rho ((muxc_b - dmuxc_b Wb) - (muxc_in - dmuxc_in Wi))  on dS
//              wR = rho (dmuxc_b - dmuxc_in)                                on drho ontop
//              gW(a,b) = sum rho (d2muxc_b (rho_b - Wb S) - d2muxc_in (rho_in - Wi S))
//                                                                   on dW ontop
//              - rho                                                on dvxc_ontop
//   on site    wA(mu,mu) = -rho_s dmuxc_in(Wi_s(a,a)),
//              wA(mu,nu) = rho_s (dmuxc_b - dmuxc_in)(W_s(a,b)), mu != nu  on drho atom
//              gA(a,b) = sum_{mu != nu} rho_s (d2muxc_b rho_b_s - d2muxc_in rho_in_s)
//                                                                   on dW atom
// with the self block's Dblocko (the diagonal shell-density derivative of
// :498-509, never assembled for the self pair) zero, and rho_bond's
// off-diagonal derivatives taken as rho_in's (:566, :582), as the reference
// does.  The three-center pass contracts rho dmuxc_in and the shell sums
// of rho d2muxc_in (rho_in - Wi S) left here per pair.
template <int PA, int PB, bool HASD>
__device__ __forceinline__ void pair_dvxc(const Ctx2c &c, const VxcArgs &v, int i, int p, const double *wA,
                                          const double *gA) {
  using PL = Plan<PA, PB, K2C>;
  using PLA = Plan<PA, PA, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n, NEA = PLA::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB);
  const FdataDev &fd = *c.fd;
  int j = c.neigh_j[p];
  int in1 = c.isp[i], in2 = c.isp[j];
  long long o = c.blk_off[p];
  double *gdp = v.gd + (long long)VXC_WSH * p;
  if (i == j && c.neigh_b[p] == 0) {
#pragma unroll
    for (int q = 0; q < 3; q++) v.off[3 * p + q] = v.on[3 * p + q] = 0.0;
#pragma unroll
    for (int q = 0; q < NA * NB; q++) v.wd[o + q] = 0.0;
#pragma unroll
    for (int q = 0; q < VXC_WSH; q++) gdp[q] = 0.0;
    return;
  }
  double r1[3], r2[3], z, e[3][3];
  pair_geom(c, i, p, r1, r2, z, e);
  double dd[3][3][3];
  depsilon_2c(r1, r2, z, e, dd);
  RotM R;
  DRotM D;
  twister<HASD>(e, R);
  dtwister<HASD>(e, dd, D);
  double eta[3] = {e[0][2], e[1][2], e[2][2]};
  bool tiny = z < 1.0e-5;
  bool on_eta = z > 1.0e-3;
  // weights of the off-site terms and of the three-center pass
  const double *rho = v.a.rho + o, *S = c.S + o, *ri = v.rho_in + o, *rb = v.rho_bond + o;
  const double *Wi = v.wrho_in + (long long)VXC_WSH * p, *Wb = v.wrho_bond + (long long)VXC_WSH * p;
  double wS[NA * NB], wR[NA * NB], gW[SA * SB];
#pragma unroll
  for (int a = 0; a < SA; a++)
#pragma unroll
    for (int b = 0; b < SB; b++) {
      double wi = Wi[a + SA * b], wb = Wb[a + SA * b];
      Lda li = lda_ca(wi), lb = lda_ca(wb);
      double g = 0.0, gd = 0.0;
#pragma unroll
      for (int mu = shell_off(a); mu < shell_off(a) + 2 * a + 1; mu++)
#pragma unroll
        for (int nu = shell_off(b); nu < shell_off(b) + 2 * b + 1; nu++) {
          int q = mu + NA * nu;
          double r = rho[q], ov = S[q];
          wS[q] = r * ((lb.muxc - lb.dmuxc * wb) - (li.muxc - li.dmuxc * wi));
          wR[q] = r * (lb.dmuxc - li.dmuxc);
          g += r * (lb.d2muxc * (rb[q] - wb * ov) - li.d2muxc * (ri[q] - wi * ov));
          v.wd[o + q] = r * li.dmuxc;
          gd += r * li.d2muxc * (ri[q] - wi * ov);
        }
      gW[a + SA * b] = g;
      gdp[a + SA * b] = gd;
    }
#pragma unroll
  for (int q = SA * SB; q < VXC_WSH; q++) gdp[q] = 0.0;
  double f[3], out[3];
  double val[NE > NEA ? NE : NEA], dv[NE > NEA ? NE : NEA], vd[3 * (NE > NEA ? NE : NEA)];
  // d overlap
  interp2c_d<NE>(c.table2c, fd.c2[in1][in2][0], z, tiny, val, dv, c.status);
  vec2c<NE>(z, eta, dv, vd);
  contract<PA, PB, K2C, HASD>(R, D, wS, val, vd, f);
  // d rho ontop: the shells of i (left) and of j (right), Qneutral weighted
  {
    double m[NE], dm[NE], t[NE], dt[NE];
#pragma unroll
    for (int q = 0; q < NE; q++) m[q] = dm[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SA; isorp++) {
      interp2c_d<NE>(c.table2c, fd.c2rho[in1][in2][0][isorp], z, tiny, t, dt, c.status);
      double Q = fd.sp[in1].qn[isorp];
#pragma unroll
      for (int q = 0; q < NE; q++) m[q] = fma(t[q], Q, m[q]), dm[q] = fma(dt[q], Q, dm[q]);
    }
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      interp2c_d<NE>(c.table2c, fd.c2rho[in1][in2][1][isorp], z, tiny, t, dt, c.status);
      double Q = fd.sp[in2].qn[isorp];
#pragma unroll
      for (int q = 0; q < NE; q++) m[q] = fma(t[q], Q, m[q]), dm[q] = fma(dt[q], Q, dm[q]);
    }
    vec2c<NE>(z, eta, dm, vd);
    contract<PA, PB, K2C, HASD>(R, D, wR, m, vd, out);
#pragma unroll
    for (int q = 0; q < 3; q++) f[q] += out[q];
  }
  // d W ontop (shell level, no rotation)
  {
    double dw[SA * SB], t[SA * SB], dt[SA * SB];
#pragma unroll
    for (int q = 0; q < SA * SB; q++) dw[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SA; isorp++) {
      interp2c_d<SA * SB>(c.table2c, fd.c2rho[in1][in2][3][isorp], z, tiny, t, dt, c.status);
      double Q = fd.sp[in1].qn[isorp];
#pragma unroll
      for (int q = 0; q < SA * SB; q++) dw[q] = fma(dt[q], Q, dw[q]);
    }
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      interp2c_d<SA * SB>(c.table2c, fd.c2rho[in1][in2][4][isorp], z, tiny, t, dt, c.status);
      double Q = fd.sp[in2].qn[isorp];
#pragma unroll
      for (int q = 0; q < SA * SB; q++) dw[q] = fma(dt[q], Q, dw[q]);
    }
    if (on_eta) {
#pragma unroll
      for (int a = 0; a < SA; a++)
#pragma unroll
        for (int b = 0; b < SB; b++)
#pragma unroll
          for (int k = 0; k < 3; k++) f[k] += gW[a + SA * b] * (-eta[k] * dw[a * SB + b]);
    }
  }
  // - rho . d vxc_ontop (Dassemble_vxc_bond)
  interp2c_d<NE>(c.table2c, fd.c2vxc[in1][in2], z, tiny, val, dv, c.status);
  vec2c<NE>(z, eta, dv, vd);
  contract<PA, PB, K2C, HASD>(R, D, rho, val, vd, out);
#pragma unroll
  for (int q = 0; q < 3; q++) v.off[3 * p + q] = f[q] - out[q];
  // on site: d rho atom and d W atom of this neighbor
  {
    double m[NEA], dm[NEA], t[NEA], dt[NEA];
#pragma unroll
    for (int q = 0; q < NEA; q++) m[q] = dm[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      interp2c_d<NEA>(c.table2c, fd.c2rho[in1][in2][2][isorp], z, tiny, t, dt, c.status);
      double Q = fd.sp[in2].qn[isorp];
#pragma unroll
      for (int q = 0; q < NEA; q++) m[q] = fma(t[q], Q, m[q]), dm[q] = fma(dt[q], Q, dm[q]);
    }
    vec2c<NEA>(z, eta, dm, vd);
    contract<PA, PA, K2C, HASD>(R, D, wA, m, vd, f);
    double dw[SA * SA], ts[SA * SA], dts[SA * SA];
#pragma unroll
    for (int q = 0; q < SA * SA; q++) dw[q] = 0.0;
#pragma unroll
    for (int isorp = 0; isorp < SB; isorp++) {
      interp2c_d<SA * SA>(c.table2c, fd.c2rho[in1][in2][5][isorp], z, tiny, ts, dts, c.status);
      double Q = fd.sp[in2].qn[isorp];
#pragma unroll
      for (int q = 0; q < SA * SA; q++) dw[q] = fma(dts[q], Q, dw[q]);
    }
    if (on_eta) {
#pragma unroll
      for (int a = 0; a < SA; a++)
#pragma unroll
        for (int b = 0; b < SA; b++)
#pragma unroll
          for (int k = 0; k < 3; k++) f[k] += gA[a + SA * b] * (-eta[k] * dw[a * SA + b]);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) v.on[3 * p + q] = f[q];
  }
}

template <int PA, bool HASD>
__device__ void atom_dvxc(const Ctx2c &c, const VxcArgs &v, int i, int lane) {
  constexpr int NA = pat_norb(PA), SA = pat_nssh(PA);
  int p0 = c.pair_off[i], ps = p0 + c.neigh_self[i];
  long long os = c.blk_off[ps];
  // on-site weights from the self block (the same for every neighbor of i)
  double wA[NA * NA], gA[SA * SA];
  {
    const double *Wi = v.wrho_in + (long long)VXC_WSH * ps, *Wb = v.wrho_bond + (long long)VXC_WSH * ps;
    const double *rs = v.a.rho + os, *ri = v.rho_in + os, *rb = v.rho_bond + os;
#pragma unroll
    for (int a = 0; a < SA; a++) {
      Lda ld = lda_ca(Wi[a + SA * a]);
#pragma unroll
      for (int b = 0; b < SA; b++) {
        Lda li = lda_ca(Wi[a + SA * b]), lb = lda_ca(Wb[a + SA * b]);
        double g = 0.0;
#pragma unroll
        for (int mu = shell_off(a); mu < shell_off(a) + 2 * a + 1; mu++)
#pragma unroll
          for (int nu = shell_off(b); nu < shell_off(b) + 2 * b + 1; nu++) {
            int q = mu + NA * nu;
            double r = rs[q];
            if (mu == nu) {
              wA[q] = -r * ld.dmuxc;
            } else {
              wA[q] = r * (lb.dmuxc - li.dmuxc);
              g += r * (lb.d2muxc * rb[q] - li.d2muxc * ri[q]);
            }
          }
        gA[a + SA * b] = g;
      }
    }
  }
  for (int p = p0 + lane; p < c.pair_off[i + 1]; p += 32) {
    int pb = c.fd->sp[c.isp[c.neigh_j[p]]].pattern;
    if (pb == PAT_SP) pair_dvxc<PA, PAT_SP, HASD>(c, v, i, p, wA, gA);
    else if (pb == PAT_S) pair_dvxc<PA, PAT_S, HASD>(c, v, i, p, wA, gA);
    else if constexpr (HASD) pair_dvxc<PA, PAT_SPD, HASD>(c, v, i, p, wA, gA);
  }
}

template <bool HASD>
__global__ void __launch_bounds__(128) k_dvxc_2c(Ctx2c c, VxcArgs v) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= c.N) return;
  int pa = c.fd->sp[c.isp[i]].pattern;
  if (pa == PAT_SP) atom_dvxc<PAT_SP, HASD>(c, v, i, lane);
  else if (pa == PAT_S) atom_dvxc<PAT_S, HASD>(c, v, i, lane);
  else if constexpr (HASD) atom_dvxc<PAT_SPD, HASD>(c, v, i, lane);
}

// Dassemble_vxc_3c: rhoxa/b = the Qneutral-weighted derivative rotations of
// den3, rhoma/b the shell-level denS3 derivatives; mxca = dmuxc rhoxa +
// rhoma d2muxc (rho_in - W S) (:371-402), contracted with rho of the pair:
// sum rho mxca = contract(rho dmuxc, rhoxa) + sum_ab gd(a,b) rhoma(a,b).
template <int PA, int PB, bool HASD, bool QSUM>
__device__ void trip_dvxc(const Ctx3c &c, const VxcArgs &v, int t) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  constexpr int SA = pat_nssh(PA), SB = pat_nssh(PB);
  int ia, iat, jat;
  TripGeom g;
  trip_geom(c, t, ia, iat, jat, g);
  const FdataDev &fd = *c.fd;
  int in1 = c.isp[iat], in2 = c.isp[jat], indna = c.isp[ia];
  if (qsum_fast(c, in1, in2, indna, g.x, g.z) != QSUM) return;
  int nk = fd.sp[indna].nssh;
  const double *qk = fd.sp[indna].qn;
  int p = c.tdst[t];
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
  // shell level first (denS3, no rotation, mvalue 0): with rhoma = rhat dx +
  // amt dp and rhomb = -sighat dy + bmt dp - rhoma / 2, only the gd-weighted
  // sums of dp, dx, dy enter
  double gp = 0.0, gx = 0.0, gy = 0.0;
  {
    constexpr int NS = SA * SB;
    double Dp[NS], Dx[NS], Dy[NS], s0[NS];
    if constexpr (QSUM) {
      interp3c<NS, true>(c, fd.c3rhoq[in1][in2][indna][1], g.x, g.z, g.cost, s0, Dp, Dx, Dy);
    } else {
      double s1[NS], s2[NS], s3[NS];
#pragma unroll
      for (int e = 0; e < NS; e++) Dp[e] = Dx[e] = Dy[e] = 0.0;
#pragma unroll 1
      for (int isorp = 0; isorp < nk; isorp++) {
        interp3c<NS, true>(c, fd.c3rho[in1][in2][indna][1][isorp], g.x, g.z, g.cost, s0, s1, s2, s3);
        double Q = qk[isorp];
#pragma unroll
        for (int e = 0; e < NS; e++) {
          Dp[e] = fma(s1[e], Q, Dp[e]);
          Dx[e] = fma(s2[e], Q, Dx[e]);
          Dy[e] = fma(s3[e], Q, Dy[e]);
        }
      }
    }
    const double *gd = v.gd + (long long)VXC_WSH * p;
#pragma unroll
    for (int a = 0; a < SA; a++)
#pragma unroll
      for (int b = 0; b < SB; b++) {
        int e = a * SB + b;
        double w = gd[a + SA * b];
        gp = fma(w, Dp[e], gp);
        gx = fma(w, Dx[e], gx);
        gy = fma(w, Dy[e], gy);
      }
  }
  // orbital level (den3): value and derivatives, Qneutral-summed
  double F[NE], DpF[NE], DxF[NE], DyF[NE];
  if constexpr (QSUM) {
    interp3c<NE, true>(c, fd.c3rhoq[in1][in2][indna][0], g.x, g.z, g.cost, F, DpF, DxF, DyF);
  } else {
    double t0[NE], t1[NE], t2[NE], t3[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) F[e] = DpF[e] = DxF[e] = DyF[e] = 0.0;
#pragma unroll 1
    for (int isorp = 0; isorp < nk; isorp++) {
      interp3c<NE, true>(c, fd.c3rho[in1][in2][indna][0][isorp], g.x, g.z, g.cost, t0, t1, t2, t3);
      double Q = qk[isorp];
#pragma unroll
      for (int e = 0; e < NE; e++) {
        F[e] = fma(t0[e], Q, F[e]);
        DpF[e] = fma(t1[e], Q, DpF[e]);
        DxF[e] = fma(t2[e], Q, DxF[e]);
        DyF[e] = fma(t3[e], Q, DyF[e]);
      }
    }
  }
  // the sin(theta) factor of the mvalue = 1 channels (getDMEs_Fdata_3c
  // :827-832), in place
  double sint = sqrt(fmax(1.0e-5, 1.0 - g.cost * g.cost));
  sfor<NE>([&](auto E) {
    constexpr int e = decltype(E)::value;
    if constexpr (PL::m.mv[e] == 1) {
      DpF[e] = DpF[e] * sint - g.cost * F[e] / sint;
      F[e] = F[e] * sint;
      DxF[e] = DxF[e] * sint;
      DyF[e] = DyF[e] * sint;
    }
  });
  // vdxcMa = rhat dx + amt dp, vdxcMb = -sighat dy + bmt dp - vdxcMa / 2
  // (:285-301): contracted with the molecular-frame weights G only through
  // the sums of dx G, dp G, dy G
  RotM R;
  twister<HASD>(g.e, R);
  const double *wdp = v.wd + c.blk_off[p];
  double wb[NA * NB];
#pragma unroll
  for (int q = 0; q < NA * NB; q++) wb[q] = __ldg(wdp + q);
  double fa[3], fb[3];
  if constexpr (NA <= 4 && NB <= 4) {
    // frame-derivative terms through the rotation rates of the frame
    // (frame_terms_3c); G(e) from the whole molecular-frame block
    double Gf[NA * NB], Ge[NE], hA[3], hB[3];
    mol_G_full<PA, PB>(R, wb, Gf);
    sfor<NE>([&](auto E) {
      constexpr int e = decltype(E)::value;
      constexpr int at = PL::m.mu[e] + NA * PL::m.nu[e];
      Ge[e] = Gf[at];
    });
    frame_terms_3c<PA, PB>(g, Gf, F, hA, hB);
    double sx = 0.0, sp = 0.0, sy = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
      sx = fma(DxF[e], Ge[e], sx);
      sp = fma(DpF[e], Ge[e], sp);
      sy = fma(DyF[e], Ge[e], sy);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double ga = g.rhat[q] * (sx + gx) + amt[q] * (sp + gp);
      fa[q] = hA[q] + ga;
      fb[q] = hB[q] - g.sighat[q] * (sy + gy) + bmt[q] * (sp + gp) - 0.5 * ga;
    }
  } else {
    double dA[3][3][3], dB[3][3][3];
    depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.e, dA, dB);
    DRotM DA;
    dtwister<HASD>(g.e, dA, DA);
    MolRho<PA, PB, K3C> G;
    mol_rho<PA, PB, K3C>(R, DA, wb, G);
    double sx = 0.0, sp = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) sx = fma(DxF[e], G.G[e], sx), sp = fma(DpF[e], G.G[e], sp);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double h = 0.0;
#pragma unroll
      for (int e = 0; e < NE; e++) h = fma(F[e], G.H[q][e], h);
      fa[q] = h + g.rhat[q] * (sx + gx) + amt[q] * (sp + gp);
    }
    DRotM DB;
    dtwister<HASD>(g.e, dB, DB);
    mol_rho<PA, PB, K3C>(R, DB, wb, G);
    double tx = 0.0, tp = 0.0, ty = 0.0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
      tx = fma(DxF[e], G.G[e], tx);
      tp = fma(DpF[e], G.G[e], tp);
      ty = fma(DyF[e], G.G[e], ty);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
      double h = 0.0;
#pragma unroll
      for (int e = 0; e < NE; e++) h = fma(F[e], G.H[q][e], h);
      fb[q] = h - g.sighat[q] * (ty + gy) + bmt[q] * (tp + gp) - 0.5 * (g.rhat[q] * (tx + gx) + amt[q] * (tp + gp));
    }
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    atomicAdd(v.f3a + 3 * ia + q, -fa[q]);
    atomicAdd(v.f3b + 3 * iat + q, -fb[q]);
    atomicAdd(v.f3c + 3 * jat + q, fa[q] + fb[q]);
  }
}

template <bool HASD, bool QSUM>
__global__ void __launch_bounds__(128) k_dvxc_3c(Ctx3c c, VxcArgs v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.T; i += gridDim.x * blockDim.x) {
    int t = c.tperm ? c.tperm[i] : i;
    int in1 = c.isp[c.ci_j[t]], in2 = c.isp[c.cj_j[t]];
    int pa = c.fd->sp[in1].pattern, pb = c.fd->sp[in2].pattern;
    int key = pa * 3 + pb;
    switch (key) {
      case PAT_SP * 3 + PAT_SP: trip_dvxc<PAT_SP, PAT_SP, HASD, QSUM>(c, v, t); break;
      case PAT_SP * 3 + PAT_S: trip_dvxc<PAT_SP, PAT_S, HASD, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_SP: trip_dvxc<PAT_S, PAT_SP, HASD, QSUM>(c, v, t); break;
      case PAT_S * 3 + PAT_S: trip_dvxc<PAT_S, PAT_S, HASD, QSUM>(c, v, t); break;
      default:
        if constexpr (HASD) {
          if (key == PAT_SPD * 3 + PAT_SPD) trip_dvxc<PAT_SPD, PAT_SPD, HASD, QSUM>(c, v, t);
          else if (key == PAT_SPD * 3 + PAT_SP) trip_dvxc<PAT_SPD, PAT_SP, HASD, QSUM>(c, v, t);
          else if (key == PAT_SP * 3 + PAT_SPD) trip_dvxc<PAT_SP, PAT_SPD, HASD, QSUM>(c, v, t);
          else if (key == PAT_SPD * 3 + PAT_S) trip_dvxc<PAT_SPD, PAT_S, HASD, QSUM>(c, v, t);
          else if (key == PAT_S * 3 + PAT_SPD) trip_dvxc<PAT_S, PAT_SPD, HASD, QSUM>(c, v, t);
        }
    }
  }
}

#if FB_IN_PART(0)
// build_forces vxc terms (c.SYSTEM/M_build_forces.f90:345-365, :453-455):
// f_i += off + on of i's pairs, f_j -= them, gathered by atom j through
// neigh_back (one warp per atom); ftot += that + f3xca + f3xcb + f3xcc.
__global__ void k_vxc_forces(int N, const int *__restrict__ pair_off, const int *__restrict__ neigh_j,
                             const int *__restrict__ neigh_back, const double *__restrict__ off,
                             const double *__restrict__ on, const double *__restrict__ f3a,
                             const double *__restrict__ f3b, const double *__restrict__ f3c,
                             double *__restrict__ fvxc, double *__restrict__ ftot) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= N) return;
  double f[3] = {0.0, 0.0, 0.0};
  for (int p = pair_off[i] + lane; p < pair_off[i + 1]; p += 32) {
    int pb = pair_off[neigh_j[p]] + neigh_back[p];  // pair (j -> i)
#pragma unroll
    for (int q = 0; q < 3; q++) f[q] += off[3 * p + q] + on[3 * p + q] - off[3 * pb + q] - on[3 * pb + q];
  }
#pragma unroll
  for (int q = 0; q < 3; q++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) f[q] += __shfl_xor_sync(0xffffffffu, f[q], o);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 3; q++) {
      fvxc[3 * i + q] = f[q];
      ftot[3 * i + q] += f[q] + f3a[3 * i + q] + f3b[3 * i + q] + f3c[3 * i + q];
    }
  }
}
#endif

}  // namespace

// The launchers are split over eight parts of this source (FB_IN_PART): the
// d-shell (HASD) instantiations build apart from the s/p ones.
int launch_dvxc_3c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s);
int launch_dvxc_3c_d_split(const VxcArgs &v, int blocks, int threads, cudaStream_t s);
int launch_rho_3c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s);
int launch_dvxc_2c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s);

#if FB_IN_PART(0)
int launch_rho_2c(const VxcArgs &v, cudaStream_t s) {
  if (v.a.N == 0) return 0;
  Ctx2c c = make2c(v.a);
  int threads = 128, blocks = (int)(((long long)v.a.N * 32 + threads - 1) / threads);
  if (v.a.have_d) k_rho_2c<true><<<blocks, threads, 0, s>>>(c, v);
  else k_rho_2c<false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_vxc(const VxcArgs &v, cudaStream_t s) {
  if (v.a.N == 0) return 0;
  Ctx2c c = make2c(v.a);
  int threads = 128, blocks = (int)(((long long)v.a.N * 32 + threads - 1) / threads);
  if (v.a.have_d) k_vxc<true><<<blocks, threads, 0, s>>>(c, v);
  else k_vxc<false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_vxc_forces(const VxcArgs &v, cudaStream_t s) {
  if (v.a.N == 0) return 0;
  int threads = 128, blocks = (int)(((long long)v.a.N * 32 + threads - 1) / threads);
  k_vxc_forces<<<blocks, threads, 0, s>>>(v.a.N, v.a.pair_off, v.a.neigh_j, v.a.neigh_back, v.off, v.on, v.f3a,
                                          v.f3b, v.f3c, v.fvxc, v.a.ftot);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(1)
int launch_rho_3c(const VxcArgs &v, cudaStream_t s) {
  if (v.a.ntrip == 0) return 0;
  int threads = 128;
  long long need = ((long long)v.a.ntrip + threads - 1) / threads;
  int blocks = (int)(need < 152LL * 64 ? need : 152LL * 64);
  if (v.a.have_d) return launch_rho_3c_d(v, blocks, threads, s);
  Ctx3c c = make3c(v.a);
  k_rho_3c<false, true><<<blocks, threads, 0, s>>>(c, v);
  if (!v.qsum_all) k_rho_3c<false, false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(2)
int launch_rho_3c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s) {
  Ctx3c c = make3c(v.a);
  k_rho_3c<true, true><<<blocks, threads, 0, s>>>(c, v);
  if (!v.qsum_all) k_rho_3c<true, false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}

#endif

#if FB_IN_PART(3)
int launch_dvxc_2c(const VxcArgs &v, cudaStream_t s) {
  if (v.a.N == 0) return 0;
  int threads = 128, blocks = (int)(((long long)v.a.N * 32 + threads - 1) / threads);
  if (v.a.have_d) return launch_dvxc_2c_d(v, blocks, threads, s);
  Ctx2c c = make2c(v.a);
  k_dvxc_2c<false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(4)
int launch_dvxc_2c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s) {
  Ctx2c c = make2c(v.a);
  k_dvxc_2c<true><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(5)
int launch_dvxc_3c(const VxcArgs &v, cudaStream_t s) {
  if (v.a.ntrip == 0) return 0;
  int threads = 128;
  long long need = ((long long)v.a.ntrip + threads - 1) / threads;
  int blocks = (int)(need < 152LL * 64 ? need : 152LL * 64);
  if (v.a.have_d) return launch_dvxc_3c_d(v, blocks, threads, s);
  Ctx3c c = make3c(v.a);
  k_dvxc_3c<false, true><<<blocks, threads, 0, s>>>(c, v);
  if (!v.qsum_all) k_dvxc_3c<false, false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

#if FB_IN_PART(6)
int launch_dvxc_3c_d(const VxcArgs &v, int blocks, int threads, cudaStream_t s) {
  Ctx3c c = make3c(v.a);
  k_dvxc_3c<true, true><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  if (!v.qsum_all) return launch_dvxc_3c_d_split(v, blocks, threads, s);
  return 0;
}
#endif

#if FB_IN_PART(7)
int launch_dvxc_3c_d_split(const VxcArgs &v, int blocks, int threads, cudaStream_t s) {
  Ctx3c c = make3c(v.a);
  k_dvxc_3c<true, false><<<blocks, threads, 0, s>>>(c, v);
  FB_LAUNCH_CHECK();
  return 0;
}
#endif

}  // namespace fb
