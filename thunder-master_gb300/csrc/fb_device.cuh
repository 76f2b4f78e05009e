// fb_device.cuh -- device math of libfbgpu: local frames, Slater-Koster
// rotations and their derivatives, and table interpolation weights.
// Every routine names the reference routine whose mathematics it computes.
#pragma once
#include <utility>
#include <type_traits>
#include "fb_internal.h"

namespace fb {

// ---------------------------------------------------------------------------
// compile-time loops
// ---------------------------------------------------------------------------
template <class F, int... I>
__device__ __forceinline__ void sfor_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sfor(F &&f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

enum { K2C = 0, K3C = 1 };
template <int PA, int PB, int K>
struct Plan {
  static constexpr MEMap m = (K == K3C) ? make_munu_3c(PA, PB) : make_munu(PA, PB);
  static constexpr int NA = pat_norb(PA);
  static constexpr int NB = pat_norb(PB);
  // is ME e the first one feeding row mu of Y, block column shell sb?
  static constexpr bool first_y(int e) {
    for (int q = 0; q < e; q++)
      if (m.mu[q] == m.mu[e] && orb_shell(m.nu[q]) == orb_shell(m.nu[e])) return false;
    return true;
  }
  // is Y(mu, k2) structurally nonzero?
  static constexpr bool ynz(int mu, int k2) {
    for (int q = 0; q < m.n; q++)
      if (m.mu[q] == mu && orb_shell(m.nu[q]) == orb_shell(k2)) return true;
    return false;
  }
  // is X(k1, k2) structurally nonzero?
  static constexpr bool xnz(int k1, int k2) {
    int s1 = orb_shell(k1);
    for (int mu = shell_off(s1); mu < shell_off(s1) + 2 * s1 + 1; mu++)
      if (ynz(mu, k2)) return true;
    return false;
  }
};

// ---------------------------------------------------------------------------
// exact (uncontracted) FP64 helpers for integer-valued decisions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dist_rn(const double *a, const double *b) {
  double d0 = __dsub_rn(b[0], a[0]), d1 = __dsub_rn(b[1], a[1]), d2 = __dsub_rn(b[2], a[2]);
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

// ---------------------------------------------------------------------------
// epsilon_function (b.FUNCTIONS/epsilon.f90:73-202): e[i][j] = spe(i+1,j+1)
// ---------------------------------------------------------------------------
// Returns true when the y axis is r2 x r1 normalised (the standard frame),
// false for the identity or the fallback y axis of a collinear pair.
__device__ __forceinline__ bool epsilon_fn(const double *r1, const double *r2, double e[3][3]) {
  double r1m = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  double r2m = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  if (r2m < 1.0e-4) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) e[i][j] = (i == j) ? 1.0 : 0.0;
    return false;
  }
  double inv2 = 1.0 / r2m;
  double zp[3] = {r2[0] * inv2, r2[1] * inv2, r2[2] * inv2};
  double yp[3] = {0.0, 0.0, 0.0}, ypm = 0.0;
  if (r1m > 1.0e-4) {
    double inv1 = 1.0 / r1m;
    double h0 = r1[0] * inv1, h1 = r1[1] * inv1, h2 = r1[2] * inv1;
    yp[0] = zp[1] * h2 - zp[2] * h1;
    yp[1] = zp[2] * h0 - zp[0] * h2;
    yp[2] = zp[0] * h1 - zp[1] * h0;
    ypm = sqrt(yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]);
  }
  const bool standard = !(ypm < 1.0e-4);
  if (!standard) {
    if (fabs(zp[0]) > 1.0e-4) {
      yp[0] = -(zp[1] + zp[2]) / zp[0];
      yp[1] = 1.0;
      yp[2] = 1.0;
    } else if (fabs(zp[1]) > 1.0e-4) {
      yp[0] = 1.0;
      yp[1] = -(zp[0] + zp[2]) / zp[1];
      yp[2] = 1.0;
    } else {
      yp[0] = 1.0;
      yp[1] = 1.0;
      yp[2] = -(zp[0] + zp[1]) / zp[2];
    }
    ypm = sqrt(yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]);
  }
  double iy = 1.0 / ypm;
  yp[0] *= iy;
  yp[1] *= iy;
  yp[2] *= iy;
  double xp[3] = {yp[1] * zp[2] - yp[2] * zp[1], yp[2] * zp[0] - yp[0] * zp[2], yp[0] * zp[1] - yp[1] * zp[0]};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    e[k][0] = xp[k];
    e[k][1] = yp[k];
    e[k][2] = zp[k];
  }
  return standard;
}

// epsilon_fn for arguments that are unit vectors already (or r1 = 0): the
// three-center frame epsilon(rhat, sighat).  The normalisations of r1 and r2
// are the identity to within an ulp and are skipped; the decisions are the
// same (r1 = 0 or |r2 x r1| < 1e-4 takes the fallback y axis).
__device__ __forceinline__ bool epsilon_unit(const double *r1, const double *r2, double e[3][3]) {
  const double zp[3] = {r2[0], r2[1], r2[2]};
  double yp[3] = {0.0, 0.0, 0.0}, ypm = 0.0;
  if (r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2] > 1.0e-8) {
    yp[0] = zp[1] * r1[2] - zp[2] * r1[1];
    yp[1] = zp[2] * r1[0] - zp[0] * r1[2];
    yp[2] = zp[0] * r1[1] - zp[1] * r1[0];
    ypm = sqrt(yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]);
  }
  const bool standard = !(ypm < 1.0e-4);
  if (!standard) {
    if (fabs(zp[0]) > 1.0e-4) {
      yp[0] = -(zp[1] + zp[2]) / zp[0];
      yp[1] = 1.0;
      yp[2] = 1.0;
    } else if (fabs(zp[1]) > 1.0e-4) {
      yp[0] = 1.0;
      yp[1] = -(zp[0] + zp[2]) / zp[1];
      yp[2] = 1.0;
    } else {
      yp[0] = 1.0;
      yp[1] = 1.0;
      yp[2] = -(zp[0] + zp[1]) / zp[2];
    }
    ypm = sqrt(yp[0] * yp[0] + yp[1] * yp[1] + yp[2] * yp[2]);
  }
  double iy = 1.0 / ypm;
  yp[0] *= iy;
  yp[1] *= iy;
  yp[2] *= iy;
  double xp[3] = {yp[1] * zp[2] - yp[2] * zp[1], yp[2] * zp[0] - yp[0] * zp[2], yp[0] * zp[1] - yp[1] * zp[0]};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    e[k][0] = xp[k];
    e[k][1] = yp[k];
    e[k][2] = zp[k];
  }
  return standard;
}

__device__ __forceinline__ constexpr double levi(int i, int j, int k) {
  return (i == j || j == k || i == k) ? 0.0
         : ((i == 0 && j == 1) || (i == 1 && j == 2) || (i == 2 && j == 0)) ? 1.0
                                                                            : -1.0;
}

// Depsilon_2c (b.FUNCTIONS/Depsilon_2c.f90:46-140): d[ix][imu][k]
__device__ __forceinline__ void depsilon_2c(const double *r1, const double *r2, double z, const double e[3][3],
                                            double d[3][3][3]) {
#pragma unroll
  for (int a = 0; a < 27; a++) (&d[0][0][0])[a] = 0.0;
  if (z < 1.0e-5) return;
  double c0 = r2[1] * r1[2] - r2[2] * r1[1];
  double c1 = r2[2] * r1[0] - r2[0] * r1[2];
  double c2 = r2[0] * r1[1] - r2[1] * r1[0];
  double cm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  if (fabs(cm) < 1.0e-3) return;
  double r2m2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
  double r12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  double iz = 1.0 / z, ic = 1.0 / cm;
#pragma unroll
  for (int ix = 0; ix < 3; ix++)
#pragma unroll
    for (int imu = 0; imu < 3; imu++) {
      double sum = levi(ix, imu, 0) * r2[0] + levi(ix, imu, 1) * r2[1] + levi(ix, imu, 2) * r2[2];
      double dk = (ix == imu) ? 1.0 : 0.0;
      d[ix][imu][0] = e[imu][0] * e[ix][2] * iz - e[imu][0] * ic * ic * (r2m2 * r1[ix] - r12 * r2[ix]) +
                      iz * ic * (dk * (r2m2 - r12) - r1[imu] * r2[ix] - r2[imu] * r2[ix] + 2.0 * r1[ix] * r2[imu]);
      d[ix][imu][1] = ic * (sum + e[imu][1] * ic * (r12 * r2[ix] - r2m2 * r1[ix]));
      d[ix][imu][2] = -(dk - e[imu][2] * e[ix][2]) * iz;
    }
}

// Depsilon_3c (b.FUNCTIONS/Depsilon_3c.f90:49-189): dA = deps/dratm,
// dB = deps/dr1
__device__ __forceinline__ void depsilon_3c(const double *r1, const double *r2, const double *r21, double z,
                                            const double *ratm, const double *rnabc, const double e[3][3],
                                            double dA[3][3][3], double dB[3][3][3]) {
#pragma unroll
  for (int a = 0; a < 27; a++) (&dA[0][0][0])[a] = 0.0, (&dB[0][0][0])[a] = 0.0;
  double c0 = r21[1] * rnabc[2] - r21[2] * rnabc[1];
  double c1 = r21[2] * rnabc[0] - r21[0] * rnabc[2];
  double c2 = r21[0] * rnabc[1] - r21[1] * rnabc[0];
  double cm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  if (fabs(cm) < 1.0e-3) return;
  double r2m2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
  double r1m2 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
  double ram2 = ratm[0] * ratm[0] + ratm[1] * ratm[1] + ratm[2] * ratm[2];
  double r12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  double r2a = r2[0] * ratm[0] + r2[1] * ratm[1] + r2[2] * ratm[2];
  double r1a = r1[0] * ratm[0] + r1[1] * ratm[1] + r1[2] * ratm[2];
  double ic = 1.0 / cm, iz = 1.0 / z;
  double A1 = r1m2 + r2m2 - 2.0 * r12, A2 = r12 - r1m2 - r2a + r1a, A3 = r12 - r2m2 + r2a - r1a;
  double B1 = r2a - r1a + r12 - r2m2, B2 = r2a + r1a - r12 - ram2, B3 = ram2 - 2.0 * r2a + r2m2;
#pragma unroll
  for (int ix = 0; ix < 3; ix++)
#pragma unroll
    for (int imu = 0; imu < 3; imu++) {
      double sum = levi(ix, imu, 0) * (r2[0] - r1[0]) + levi(ix, imu, 1) * (r2[1] - r1[1]) +
                   levi(ix, imu, 2) * (r2[2] - r1[2]);
      dA[ix][imu][1] = ic * (sum - (e[imu][1] * ic) * (A1 * ratm[ix] + A2 * r2[ix] + A3 * r1[ix]));
      double dk = (ix == imu) ? 1.0 : 0.0;
      dB[ix][imu][2] = iz * (e[imu][2] * e[ix][2] - dk);
      double sb = levi(ix, imu, 0) * (ratm[0] - r2[0]) + levi(ix, imu, 1) * (ratm[1] - r2[1]) +
                  levi(ix, imu, 2) * (ratm[2] - r2[2]);
      dB[ix][imu][1] = ic * (sb - (e[imu][1] * ic) * (B1 * ratm[ix] + B2 * r2[ix] + B3 * r1[ix]));
    }
#pragma unroll
  for (int a = 0; a < 3; a++) {
    dA[a][0][0] = e[2][2] * dA[a][1][1] - e[1][2] * dA[a][2][1];
    dA[a][1][0] = e[0][2] * dA[a][2][1] - e[2][2] * dA[a][0][1];
    dA[a][2][0] = e[1][2] * dA[a][0][1] - e[0][2] * dA[a][1][1];
    dB[a][0][0] = e[2][2] * dB[a][1][1] - e[2][1] * dB[a][1][2] - e[1][2] * dB[a][2][1] + e[1][1] * dB[a][2][2];
    dB[a][1][0] = e[0][2] * dB[a][2][1] - e[0][1] * dB[a][2][2] - e[2][2] * dB[a][0][1] + e[2][1] * dB[a][0][2];
    dB[a][2][0] = e[1][2] * dB[a][0][1] - e[1][1] * dB[a][0][2] - e[0][2] * dB[a][1][1] + e[0][1] * dB[a][1][2];
  }
}

// ---------------------------------------------------------------------------
// twister / Dtwister (c.SYSTEM/M_rotations.f90:221-313,
// M_Drotations.f90:203-298).  p-orbital order (y, z, x).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr double amat_v(int ix, int jx, int imu) {
  // include/constants.h:30-38 (symmetric in ix, jx)
  return imu == 0   ? (((ix == 0 && jx == 1) || (ix == 1 && jx == 0)) ? 0.5 : 0.0)
         : imu == 1 ? (((ix == 1 && jx == 2) || (ix == 2 && jx == 1)) ? 0.5 : 0.0)
         : imu == 2 ? ((ix == jx) ? (ix == 2 ? 0.57735026918962573 : -0.28867513459481287) : 0.0)
         : imu == 3 ? (((ix == 0 && jx == 2) || (ix == 2 && jx == 0)) ? 0.5 : 0.0)
                    : ((ix == jx && ix < 2) ? (ix == 0 ? 0.5 : -0.5) : 0.0);
}
__host__ __device__ constexpr int pperm(int a) { return a == 0 ? 1 : (a == 1 ? 2 : 0); }

struct RotM {
  double p[3][3];
  double d[5][5];
};
struct DRotM {
  double p[3][3][3];  // [c][a][b]
  double d[3][5][5];
};

template <bool HASD>
__device__ __forceinline__ void twister(const double e[3][3], RotM &R) {
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = e[pperm(a)][pperm(b)];
  if constexpr (HASD) {
#pragma unroll
    for (int imu = 0; imu < 5; imu++) {
      double l11 = 0, l12 = 0, l13 = 0, l32 = 0, l33 = 0;
#pragma unroll
      for (int jx = 0; jx < 3; jx++)
#pragma unroll
        for (int ix = 0; ix < 3; ix++) {
          constexpr double dummy = 0.0;
          (void)dummy;
          double a = amat_v(ix, jx, imu);
          if (a != 0.0) {
            l11 += a * e[jx][0] * e[ix][0];
            l12 += a * e[jx][0] * e[ix][1];
            l13 += a * e[jx][0] * e[ix][2];
            l32 += a * e[jx][2] * e[ix][1];
            l33 += a * e[jx][2] * e[ix][2];
          }
        }
      R.d[imu][0] = 2.0 * l12;
      R.d[imu][1] = 2.0 * l32;
      R.d[imu][2] = 1.7320508075688772 * l33;
      R.d[imu][3] = 2.0 * l13;
      R.d[imu][4] = 2.0 * l11 + l33;
    }
  }
}

template <bool HASD>
__device__ __forceinline__ void dtwister(const double e[3][3], const double dd[3][3][3], DRotM &D) {
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) D.p[c][a][b] = dd[c][pperm(a)][pperm(b)];
  if constexpr (HASD) {
#pragma unroll
    for (int imu = 0; imu < 5; imu++)
#pragma unroll
      for (int kx = 0; kx < 3; kx++) {
        double a12 = 0, a32 = 0, a33 = 0, a13 = 0, a11 = 0;
#pragma unroll
        for (int ix = 0; ix < 3; ix++)
#pragma unroll
          for (int jx = 0; jx < 3; jx++) {
            double a = amat_v(jx, ix, imu);
            if (a != 0.0) {
              a12 += a * (dd[kx][ix][0] * e[jx][1] + e[ix][0] * dd[kx][jx][1]);
              a32 += a * (dd[kx][ix][2] * e[jx][1] + e[ix][2] * dd[kx][jx][1]);
              a33 += a * (dd[kx][ix][2] * e[jx][2] + e[ix][2] * dd[kx][jx][2]);
              a13 += a * (dd[kx][ix][0] * e[jx][2] + e[ix][0] * dd[kx][jx][2]);
              a11 += a * (dd[kx][ix][0] * e[jx][0] + e[ix][0] * dd[kx][jx][0]);
            }
          }
        D.d[kx][imu][0] = 2.0 * a12;
        D.d[kx][imu][1] = 2.0 * a32;
        D.d[kx][imu][2] = 1.7320508075688772 * a33;
        D.d[kx][imu][3] = 2.0 * a13;
        D.d[kx][imu][4] = 2.0 * a11 + a33;
      }
  }
}

// element (k, m) of the rotation block of shell s (chooser,
// M_rotations.f90:341-382); s = 0 gives the literal 1
template <int S>
__device__ __forceinline__ double Lrot(const RotM &R, int k, int m) {
  if constexpr (S == 0) return 1.0;
  else if constexpr (S == 1) return R.p[k][m];
  else return R.d[k][m];
}
template <int S>
__device__ __forceinline__ double DLrot(const DRotM &D, int c, int k, int m) {
  if constexpr (S == 0) return 0.0;
  else if constexpr (S == 1) return D.p[c][k][m];
  else return D.d[c][k][m];
}

// rotate (M_rotations.f90:98-177): X = L M R^T with M given only at the ME
// positions of the plan (v[e]), computed as Y = M R^T then X = L Y while
// skipping every structurally zero product.
template <int PA, int PB, int K>
__device__ __forceinline__ void rotate_plan(const RotM &R, const double *v, double *X) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  double Y[NA * NB];
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int mu = PL::m.mu[e], nu = PL::m.nu[e];
    constexpr int sb = orb_shell(nu), mb = orb_m(nu), ob = shell_off(sb);
    constexpr bool first = PL::first_y(e);
    sfor<2 * sb + 1>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      double r = Lrot<sb>(R, k, mb);
      if constexpr (first) Y[mu * NB + ob + k] = v[e] * r;
      else Y[mu * NB + ob + k] = fma(v[e], r, Y[mu * NB + ob + k]);
    });
  });
  sfor<NA>([&](auto K1) {
    constexpr int k1 = decltype(K1)::value;
    constexpr int s1 = orb_shell(k1), m1 = orb_m(k1), o1 = shell_off(s1);
    sfor<NB>([&](auto K2) {
      constexpr int k2 = decltype(K2)::value;
      if constexpr (!PL::xnz(k1, k2)) {
        X[k1 + NA * k2] = 0.0;
      } else {
        double acc = 0.0;
        bool have = false;
        sfor<2 * s1 + 1>([&](auto MM) {
          constexpr int mm = decltype(MM)::value;
          if constexpr (PL::ynz(o1 + mm, k2)) {
            double l = Lrot<s1>(R, m1, mm);
            if (!have) acc = l * Y[(o1 + mm) * NB + k2];
            else acc = fma(l, Y[(o1 + mm) * NB + k2], acc);
            have = true;
          }
        });
        X[k1 + NA * k2] = acc;
      }
    });
  });
}

// ---------------------------------------------------------------------------
// Contraction of a rotated derivative with a density block, in the molecular
// frame.  For X_c = dL_c M R^T + L M dR_c^T + L Md_c R^T (Dmatrix,
// M_Drotations.f90:389-482), sum_{mu,nu} rho(mu,nu) X_c(mu,nu) equals
//   sum_e [ M_e H_c(e) + Md_c(e) G(e) ]
// with G = L^T rho R and H_c = dL_c^T rho R + L^T rho dR_c evaluated at the
// ME positions e only.  This is the same sum in a different order.
// ---------------------------------------------------------------------------
template <int PA, int PB, int K>
struct MolRho {
  static constexpr int NA = pat_norb(PA), NB = pat_norb(PB), NE = Plan<PA, PB, K>::m.n;
  double G[NE];
  double H[3][NE];
};

template <int PA, int PB, int K>
__device__ __forceinline__ void mol_rho(const RotM &R, const DRotM &D, const double *rho, MolRho<PA, PB, K> &out) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  // rhoR(mu, b) = sum_nu rho(mu, nu) R(nu, b) over the shell of b
  double rR[NA * NB];
  sfor<NA>([&](auto MU) {
    constexpr int mu = decltype(MU)::value;
    sfor<NB>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
      double acc = 0.0;
      sfor<2 * sb + 1>([&](auto NU) {
        constexpr int k = decltype(NU)::value;
        double t = rho[mu + NA * (ob + k)] * Lrot<sb>(R, k, mb);
        acc = (k == 0) ? t : acc + t;
      });
      rR[mu + NA * b] = acc;
    });
  });
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
    double g = 0.0;
    sfor<2 * sa + 1>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      g = fma(Lrot<sa>(R, k, ma), rR[(oa + k) + NA * b], g);
    });
    out.G[e] = g;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double h = 0.0;
      if constexpr (sa > 0) {
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          h = fma(DLrot<sa>(D, c, k, ma), rR[(oa + k) + NA * b], h);
        });
      }
      if constexpr (sb > 0) {
        // L^T rho dR at (a, b): sum_k L(k, ma) sum_nu rho(oa+k, nu) dR(nu, mb)
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          double t = 0.0;
          sfor<2 * sb + 1>([&](auto NU) {
            constexpr int q = decltype(NU)::value;
            t = fma(rho[(oa + k) + NA * (ob + q)], DLrot<sb>(D, c, q, mb), t);
          });
          h = fma(Lrot<sa>(R, k, ma), t, h);
        });
      }
      out.H[c][e] = h;
    }
  });
}

// mol_rho for the two frame derivatives of a triplet (the neutral atom's and
// atom 1's) at once: rho R and G are computed once, and rho dR_c is formed
// once per column and component, then contracted with L^T.  The same sums as
// two mol_rho calls, with the shared terms taken once.
template <int PA, int PB, int K>
__device__ __forceinline__ void mol_rho_ab(const RotM &R, const DRotM &DA, const DRotM &DB, const double *rho,
                                           MolRho<PA, PB, K> &A, MolRho<PA, PB, K> &Bo) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  double rR[NA * NB], rdA[3][NA * NB], rdB[3][NA * NB];
  sfor<NA>([&](auto MU) {
    constexpr int mu = decltype(MU)::value;
    sfor<NB>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
      double acc = 0.0;
      sfor<2 * sb + 1>([&](auto NU) {
        constexpr int k = decltype(NU)::value;
        double t = rho[mu + NA * (ob + k)] * Lrot<sb>(R, k, mb);
        acc = (k == 0) ? t : acc + t;
      });
      rR[mu + NA * b] = acc;
      if constexpr (sb > 0) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          double ta = 0.0, tb = 0.0;
          sfor<2 * sb + 1>([&](auto NU) {
            constexpr int q = decltype(NU)::value;
            ta = fma(rho[mu + NA * (ob + q)], DLrot<sb>(DA, c, q, mb), ta);
            tb = fma(rho[mu + NA * (ob + q)], DLrot<sb>(DB, c, q, mb), tb);
          });
          rdA[c][mu + NA * b] = ta;
          rdB[c][mu + NA * b] = tb;
        }
      }
    });
  });
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    constexpr int sb = orb_shell(b);
    double g = 0.0;
    sfor<2 * sa + 1>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      g = fma(Lrot<sa>(R, k, ma), rR[(oa + k) + NA * b], g);
    });
    A.G[e] = g;
    Bo.G[e] = g;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double ha = 0.0, hb = 0.0;
      if constexpr (sa > 0) {
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          ha = fma(DLrot<sa>(DA, c, k, ma), rR[(oa + k) + NA * b], ha);
          hb = fma(DLrot<sa>(DB, c, k, ma), rR[(oa + k) + NA * b], hb);
        });
      }
      if constexpr (sb > 0) {
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          ha = fma(Lrot<sa>(R, k, ma), rdA[c][(oa + k) + NA * b], ha);
          hb = fma(Lrot<sa>(R, k, ma), rdB[c][(oa + k) + NA * b], hb);
        });
      }
      A.H[c][e] = ha;
      Bo.H[c][e] = hb;
    }
  });
}

// ---------------------------------------------------------------------------
// Frame-derivative terms through rotation rates (s and p shells).
//
// The three-center frame e (columns x, y, z) is orthonormal, so its
// derivative along any coordinate is de = e W with W = e^T de skew: three
// rates W^xy, W^yz, W^xz.  The p block of the rotation is L_p = P e P^T (p
// order y, z, x), so dL = L Omega with Omega the same rates in p order, and
// for X = L M L^T
//   sum rho (dL M L^T + L M dL^T) = sum_e M_e [G, Omega](e),   G = L^T rho L,
// which is W^xy tau^xy + W^yz tau^yz + W^xz tau^xz with
// tau^ij = sum_e M_e [G, J^ij](e), J^ij = E(p_i, p_j) - E(p_j, p_i).  This is
// the same sum as contracting Dtwister's dL (M_Drotations.f90:456-471) with
// rho, without forming dL: the rates come from Depsilon_3c in closed form
// (frame_rates_3c).
// ---------------------------------------------------------------------------
// p orbital of frame axis i (x, y, z) in the order (y, z, x)
__host__ __device__ constexpr int p_of_axis(int i) { return 1 + (i == 0 ? 2 : i - 1); }

// G = L^T rho L over the whole block (rho and G column-major, NA rows)
template <int PA, int PB>
__device__ __forceinline__ void mol_G_full(const RotM &R, const double *rho, double *G) {
  constexpr int NA = pat_norb(PA), NB = pat_norb(PB);
  static_assert(NA <= 4 && NB <= 4, "s and p shells only");
  double rR[NA * NB];
  sfor<NA>([&](auto MU) {
    constexpr int mu = decltype(MU)::value;
    sfor<NB>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
      if constexpr (sb == 0) {
        rR[mu + NA * b] = rho[mu + NA * b];
      } else {
        double acc = rho[mu + NA * ob] * R.p[0][mb];
        acc = fma(rho[mu + NA * (ob + 1)], R.p[1][mb], acc);
        rR[mu + NA * b] = fma(rho[mu + NA * (ob + 2)], R.p[2][mb], acc);
      }
    });
  });
  sfor<NB>([&](auto B) {
    constexpr int b = decltype(B)::value;
    sfor<NA>([&](auto A) {
      constexpr int a = decltype(A)::value;
      constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
      if constexpr (sa == 0) {
        G[a + NA * b] = rR[a + NA * b];
      } else {
        double acc = R.p[0][ma] * rR[oa + NA * b];
        acc = fma(R.p[1][ma], rR[(oa + 1) + NA * b], acc);
        G[a + NA * b] = fma(R.p[2][ma], rR[(oa + 2) + NA * b], acc);
      }
    });
  });
}

// tau^xy, tau^yz, tau^xz of the molecular-frame block M (values at the ME
// positions of the plan) against the full molecular-frame density G
template <int PA, int PB, int K = K3C>
__device__ __forceinline__ void mol_tau(const double *G, const double *M, double tau[3]) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  constexpr bool pa = NA >= 4, pb = NB >= 4;
  sfor<3>([&](auto PR) {
    constexpr int pr = decltype(PR)::value;
    constexpr int ai = pr == 1 ? 1 : 0, aj = pr == 0 ? 1 : 2;  // (x,y), (y,z), (x,z)
    constexpr int Pi = p_of_axis(ai), Pj = p_of_axis(aj);
    double acc = 0.0;
    sfor<PL::m.n>([&](auto E) {
      constexpr int e = decltype(E)::value;
      constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
      // [G, J]_ab = G(a,Pi)[b=Pj] - G(a,Pj)[b=Pi] - [a=Pi] G(Pj,b) + [a=Pj] G(Pi,b)
      if constexpr (pb && b == Pj) acc = fma(M[e], G[a + NA * Pi], acc);
      if constexpr (pb && b == Pi) acc = fma(-M[e], G[a + NA * Pj], acc);
      if constexpr (pa && a == Pi) acc = fma(-M[e], G[Pj + NA * b], acc);
      if constexpr (pa && a == Pj) acc = fma(M[e], G[Pi + NA * b], acc);
    });
    tau[pr] = acc;
  });
}

// Rotation rates of the three-center frame, component c of d/dratm (a*) and
// d/dr1 (b*).  Depsilon_3c (b.FUNCTIONS/Depsilon_3c.f90:49-189) gives, with
// u = r21, ic = 1 / |r21 x rnabc| and iz = 1 / z,
//   e_x . de_y/dratm_c = ic (e_x x u)_c             (de_z/dratm = 0)
//   e_x . de_y/dr1_c   = ic (e_x x (ratm - r2))_c
//   e_y . de_z/dr1_c   = -iz e_y,c,   e_x . de_z/dr1_c = -iz e_x,c
// (its terms along e_x . e_y and e_y . e_z vanish).  Valid for the standard
// frame (y along r21 x rnabc); every rate is zero where Depsilon_3c returns
// zeros (|r21 x rnabc| < 1e-3).
struct FrameRates3c {
  double axy[3];
  double bxy[3], byz[3], bxz[3];
};

__device__ __forceinline__ void frame_rates_3c(const double *r2, const double *r21, double z, const double *ratm,
                                               const double *rnabc, const double e[3][3], FrameRates3c &w) {
  double c0 = r21[1] * rnabc[2] - r21[2] * rnabc[1];
  double c1 = r21[2] * rnabc[0] - r21[0] * rnabc[2];
  double c2 = r21[0] * rnabc[1] - r21[1] * rnabc[0];
  double cm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  bool zero = fabs(cm) < 1.0e-3;
  double ic = zero ? 0.0 : 1.0 / cm, iz = zero ? 0.0 : 1.0 / z;
  double ex[3] = {e[0][0], e[1][0], e[2][0]}, ey[3] = {e[0][1], e[1][1], e[2][1]};
  double s[3] = {ratm[0] - r2[0], ratm[1] - r2[1], ratm[2] - r2[2]};
  w.axy[0] = ic * (ex[1] * r21[2] - ex[2] * r21[1]);
  w.axy[1] = ic * (ex[2] * r21[0] - ex[0] * r21[2]);
  w.axy[2] = ic * (ex[0] * r21[1] - ex[1] * r21[0]);
  w.bxy[0] = ic * (ex[1] * s[2] - ex[2] * s[1]);
  w.bxy[1] = ic * (ex[2] * s[0] - ex[0] * s[2]);
  w.bxy[2] = ic * (ex[0] * s[1] - ex[1] * s[0]);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    w.byz[k] = -iz * ey[k];
    w.bxz[k] = -iz * ex[k];
  }
}

// Rotation rates of the two-center frame epsilon(r2, sighat), component q of
// d/dr1 (Depsilon_2c, b.FUNCTIONS/Depsilon_2c.f90:46-140, with
// ic = 1 / |r2 x r1| and iz = 1 / z):
//   W^xy = e_x . de_y = ic (e_x x r2)_q,  W^yz = e_y . de_z = -iz e_y,q,
//   W^xz = e_x . de_z = -iz e_x,q
// (its terms along e_x . e_y vanish).  Valid for the standard frame; all zero
// where Depsilon_2c returns zeros (z < 1e-5 or |r2 x r1| < 1e-3).  W[pair][q],
// pairs (x,y), (y,z), (x,z).
__device__ __forceinline__ bool frame2c_degenerate(const double *r1, const double *r2, double z, double &cm) {
  double c0 = r2[1] * r1[2] - r2[2] * r1[1];
  double c1 = r2[2] * r1[0] - r2[0] * r1[2];
  double c2 = r2[0] * r1[1] - r2[1] * r1[0];
  cm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  return z < 1.0e-5 || fabs(cm) < 1.0e-3;
}
__device__ __forceinline__ void frame_rates_2c(const double *r1, const double *r2, double z, const double e[3][3],
                                               double W[3][3]) {
  double cm;
  bool zero = frame2c_degenerate(r1, r2, z, cm);
  double ic = zero ? 0.0 : 1.0 / cm, iz = zero ? 0.0 : 1.0 / z;
  double ex[3] = {e[0][0], e[1][0], e[2][0]};
  W[0][0] = ic * (ex[1] * r2[2] - ex[2] * r2[1]);
  W[0][1] = ic * (ex[2] * r2[0] - ex[0] * r2[2]);
  W[0][2] = ic * (ex[0] * r2[1] - ex[1] * r2[0]);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    W[1][q] = -iz * e[q][1];
    W[2][q] = -iz * ex[q];
  }
}

// epsilon's collinear fallback frame (y axis not along r21 x rnabc) is not
// the frame Depsilon_3c differentiates.  Its de_y then has a component along
// e_y, psi = e_y . de_y, and e_z . de_y (chi) is no longer -e_y . de_z, so the
// rates of the literal derivatives gain psi (E_xx + E_yy) and, for d/dr1,
// (chi - e_y . de_z) E_zy.  From Depsilon_3c's expressions, with
// V = A1 ratm + A2 r2 + A3 r1 and V' = B1 ratm + B2 r2 + B3 r1 as there:
//   psiA = ic ((e_y x u) - ic V),  psiB = ic ((e_y x (ratm - r2)) - ic V'),
//   chiB = ic (e_z x (ratm - r2))
struct FrameExtra3c {
  double psiA[3], psiB[3], chiB[3];
};

__device__ __forceinline__ void frame_extra_3c(const double *r1, const double *r2, const double *r21,
                                               const double *ratm, const double *rnabc, const double e[3][3],
                                               FrameExtra3c &x) {
  double c0 = r21[1] * rnabc[2] - r21[2] * rnabc[1];
  double c1 = r21[2] * rnabc[0] - r21[0] * rnabc[2];
  double c2 = r21[0] * rnabc[1] - r21[1] * rnabc[0];
  double cm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  double ic = fabs(cm) < 1.0e-3 ? 0.0 : 1.0 / cm;
  double r2m2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
  double r1m2 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
  double ram2 = ratm[0] * ratm[0] + ratm[1] * ratm[1] + ratm[2] * ratm[2];
  double r12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  double r2a = r2[0] * ratm[0] + r2[1] * ratm[1] + r2[2] * ratm[2];
  double r1a = r1[0] * ratm[0] + r1[1] * ratm[1] + r1[2] * ratm[2];
  double A1 = r1m2 + r2m2 - 2.0 * r12, A2 = r12 - r1m2 - r2a + r1a, A3 = r12 - r2m2 + r2a - r1a;
  double B1 = r2a - r1a + r12 - r2m2, B2 = r2a + r1a - r12 - ram2, B3 = ram2 - 2.0 * r2a + r2m2;
  double ey[3] = {e[0][1], e[1][1], e[2][1]}, ez[3] = {e[0][2], e[1][2], e[2][2]};
  double s[3] = {ratm[0] - r2[0], ratm[1] - r2[1], ratm[2] - r2[2]};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int c1i = (c + 1) % 3, c2i = (c + 2) % 3;
    double V = A1 * ratm[c] + A2 * r2[c] + A3 * r1[c];
    double Vb = B1 * ratm[c] + B2 * r2[c] + B3 * r1[c];
    x.psiA[c] = ic * ((ey[c1i] * r21[c2i] - ey[c2i] * r21[c1i]) - ic * V);
    x.psiB[c] = ic * ((ey[c1i] * s[c2i] - ey[c2i] * s[c1i]) - ic * Vb);
    x.chiB[c] = ic * (ez[c1i] * s[c2i] - ez[c2i] * s[c1i]);
  }
}

// kappa_ij = sum_e M_e ([a = p_j] G(p_i, b) + [b = p_j] G(a, p_i)), the
// coefficient of Omega_ij; returns kappa_xx + kappa_yy and kappa_zy
template <int PA, int PB>
__device__ __forceinline__ void mol_kappa_extra(const double *G, const double *M, double &kd, double &kzy) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB;
  constexpr bool pa = NA >= 4, pb = NB >= 4;
  constexpr int Px = p_of_axis(0), Py = p_of_axis(1), Pz = p_of_axis(2);
  double d = 0.0, zy = 0.0;
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    if constexpr (pa && a == Px) d = fma(M[e], G[Px + NA * b], d);
    if constexpr (pa && a == Py) d = fma(M[e], G[Py + NA * b], d);
    if constexpr (pb && b == Px) d = fma(M[e], G[a + NA * Px], d);
    if constexpr (pb && b == Py) d = fma(M[e], G[a + NA * Py], d);
    if constexpr (pa && a == Py) zy = fma(M[e], G[Pz + NA * b], zy);
    if constexpr (pb && b == Py) zy = fma(M[e], G[a + NA * Pz], zy);
  });
  kd = d;
  kzy = zy;
}

// Explicit Drotate (M_Drotations.f90:102-153, Dmatrix :389-482):
// Xd[c + 3*(mu + NA*nu)]
template <int PA, int PB, int K>
__device__ __forceinline__ void drotate_plan(const RotM &R, const DRotM &D, const double *v, const double *vd,
                                             double *Xd) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
#pragma unroll
  for (int q = 0; q < 3 * NA * NB; q++) Xd[q] = 0.0;
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
    sfor<2 * sa + 1>([&](auto K1) {
      constexpr int k1 = decltype(K1)::value;
      sfor<2 * sb + 1>([&](auto K2) {
        constexpr int k2 = decltype(K2)::value;
        double l = Lrot<sa>(R, k1, ma), r = Lrot<sb>(R, k2, mb);
        double lr = l * r;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          double t = lr * vd[c + 3 * e];
          if constexpr (sa > 0) t = fma(DLrot<sa>(D, c, k1, ma) * r, v[e], t);
          if constexpr (sb > 0) t = fma(l * DLrot<sb>(D, c, k2, mb), v[e], t);
          Xd[c + 3 * ((oa + k1) + NA * (ob + k2))] += t;
        }
      });
    });
  });
}

// ---------------------------------------------------------------------------
// Interpolation weights
// ---------------------------------------------------------------------------
// 7-point Lagrange weights of getMEs_Fdata_2c (e.FDATA/M_Fdata_2c.f90:366-393)
// with the stencil choice of the reference; i0 = 0-based first point.
__device__ __forceinline__ void lagrange7(double x, const Cell2cDev &c, int &i0, double w[7], double *dw) {
  int imid = (int)(x / c.dx) + 1;
  int ileft = imid - 3;
  if (ileft < 1) ileft = 1;
  else if (imid + 3 > c.nx) ileft = c.nx - 6;
  i0 = ileft - 1;
  double t[7];
#pragma unroll
  for (int p = 0; p < 7; p++) t[p] = x - (double)(ileft - 1 + p) * c.dx;
  // C_k = 1 / prod_{p != k} (k - p)
  constexpr double Ck[7] = {1.0 / 720, -1.0 / 120, 1.0 / 48, -1.0 / 36, 1.0 / 48, -1.0 / 120, 1.0 / 720};
  double pre[7], suf[7];
  pre[0] = 1.0;
#pragma unroll
  for (int p = 1; p < 7; p++) pre[p] = pre[p - 1] * t[p - 1];
  suf[6] = 1.0;
#pragma unroll
  for (int p = 5; p >= 0; p--) suf[p] = suf[p + 1] * t[p + 1];
#pragma unroll
  for (int k = 0; k < 7; k++) w[k] = pre[k] * suf[k] * (Ck[k] * c.inv_dx6);
  if (dw) {
    // derivative of prod_{p != k} t_p = pre_k suf_k (every dt_p/dx = 1):
    // the prefix and suffix products' derivatives by the product rule,
    // dpre_{k+1} = dpre_k t_k + pre_k, dsuf_{k-1} = dsuf_k t_k + suf_k
    double dpre[7], dsuf[7];
    dpre[0] = 0.0;
    dpre[1] = 1.0;
#pragma unroll
    for (int p = 2; p < 7; p++) dpre[p] = fma(dpre[p - 1], t[p - 1], pre[p - 1]);
    dsuf[6] = 0.0;
    dsuf[5] = 1.0;
#pragma unroll
    for (int p = 4; p >= 0; p--) dsuf[p] = fma(dsuf[p + 1], t[p + 1], suf[p + 1]);
#pragma unroll
    for (int k = 0; k < 7; k++) dw[k] = fma(dpre[k], suf[k], pre[k] * dsuf[k]) * (Ck[k] * c.inv_dx6);
  }
}

// 4-point Lagrange weights on nodes -1, 0, 1, 2 (Abramowitz-Stegun 25.2.13,
// the bicubic of getMEs_Fdata_3c, M_Fdata_3c.f90:425-481) and derivatives
__device__ __forceinline__ void lagrange4(double p, double w[4], double *dw) {
  double pm1 = p - 1.0, pm2 = p - 2.0, pp1 = p + 1.0;
  w[0] = -p * pm1 * pm2 * (1.0 / 6.0);
  w[1] = pp1 * pm1 * pm2 * 0.5;
  w[2] = -pp1 * p * pm2 * 0.5;
  w[3] = pp1 * p * pm1 * (1.0 / 6.0);
  if (dw) {
    double p2 = p * p;
    dw[0] = -(3.0 * p2 - 6.0 * p + 2.0) * (1.0 / 6.0);
    dw[1] = (3.0 * p2 - 4.0 * p - 1.0) * 0.5;
    dw[2] = -(3.0 * p2 - 2.0 * p - 2.0) * 0.5;
    dw[3] = (3.0 * p2 - 1.0) * (1.0 / 6.0);
  }
}

}  // namespace fb
