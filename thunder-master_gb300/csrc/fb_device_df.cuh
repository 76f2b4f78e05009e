// fb_device_df.cuh -- double-float (FP32-pipe) forms of the Slater-Koster
// rotation, the molecular-frame density and rotation-rate sums and the
// bicubic table contraction used by the three-center kernels.  Same
// mathematics and same operation structure as the FP64 forms in
// fb_device.cuh (rotate_plan, mol_G_full, mol_tau) and fb_common.cuh
// (interp3c); s and p shells only.
#pragma once
#include "fb_df.cuh"
#include "fb_device.cuh"

namespace fb {

struct RotDF {
  df p[3][3];
};
__device__ __forceinline__ df df_zero() { return df{0.0f, 0.0f}; }
__device__ __forceinline__ df df_one() { return df{1.0f, 0.0f}; }

// twister (c.SYSTEM/M_rotations.f90:256-270): pmat is eps with the (y, z, x)
// order, so only conversions are needed
__device__ __forceinline__ void twister_df(const double e[3][3], RotDF &R) {
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 3; b++) R.p[a][b] = df_from(e[pperm(a)][pperm(b)]);
}
template <int S>
__device__ __forceinline__ df Lrot_df(const RotDF &R, int k, int m) {
  if constexpr (S == 0) return df_one();
  else return R.p[k][m];
}

// rotate (M_rotations.f90:98-177) in df: X = L M R^T, structural zeros
// skipped, s-shell factors (exactly 1) not multiplied
template <int PA, int PB, int K>
__device__ __forceinline__ void rotate_plan_df(const RotDF &R, const df *v, df *X) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  df Y[NA * NB];
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int mu = PL::m.mu[e], nu = PL::m.nu[e];
    constexpr int sb = orb_shell(nu), mb = orb_m(nu), ob = shell_off(sb);
    constexpr bool first = PL::first_y(e);
    sfor<2 * sb + 1>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      df t = (sb == 0) ? v[e] : v[e] * Lrot_df<sb>(R, k, mb);
      if constexpr (first) Y[mu * NB + ob + k] = t;
      else Y[mu * NB + ob + k] = Y[mu * NB + ob + k] + t;
    });
  });
  sfor<NA>([&](auto K1) {
    constexpr int k1 = decltype(K1)::value;
    constexpr int s1 = orb_shell(k1), m1 = orb_m(k1), o1 = shell_off(s1);
    sfor<NB>([&](auto K2) {
      constexpr int k2 = decltype(K2)::value;
      if constexpr (!PL::xnz(k1, k2)) {
        X[k1 + NA * k2] = df_zero();
      } else {
        df acc = df_zero();
        bool have = false;
        sfor<2 * s1 + 1>([&](auto MM) {
          constexpr int mm = decltype(MM)::value;
          if constexpr (PL::ynz(o1 + mm, k2)) {
            df t = (s1 == 0) ? Y[(o1 + mm) * NB + k2] : Lrot_df<s1>(R, m1, mm) * Y[(o1 + mm) * NB + k2];
            acc = have ? acc + t : t;
            have = true;
          }
        });
        X[k1 + NA * k2] = acc;
      }
    });
  });
}

// G = L^T rho L over the whole block and the rotation-rate sums tau^xy,
// tau^yz, tau^xz of M against it (mol_G_full / mol_tau in fb_device.cuh)
template <int PA, int PB>
__device__ __forceinline__ void mol_G_full_df(const RotDF &R, const df *rho, df *G) {
  constexpr int NA = pat_norb(PA), NB = pat_norb(PB);
  static_assert(NA <= 4 && NB <= 4, "s and p shells only");
  df rR[NA * NB];
  sfor<NA>([&](auto MU) {
    constexpr int mu = decltype(MU)::value;
    sfor<NB>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
      if constexpr (sb == 0) {
        rR[mu + NA * b] = rho[mu + NA * b];
      } else {
        rR[mu + NA * b] = rho[mu + NA * ob] * R.p[0][mb] + rho[mu + NA * (ob + 1)] * R.p[1][mb] +
                          rho[mu + NA * (ob + 2)] * R.p[2][mb];
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
        G[a + NA * b] = R.p[0][ma] * rR[oa + NA * b] + R.p[1][ma] * rR[(oa + 1) + NA * b] +
                        R.p[2][ma] * rR[(oa + 2) + NA * b];
      }
    });
  });
}

template <int PA, int PB>
__device__ __forceinline__ void mol_tau_df(const df *G, const df *M, df tau[3]) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB;
  constexpr bool pa = NA >= 4, pb = NB >= 4;
  sfor<3>([&](auto PR) {
    constexpr int pr = decltype(PR)::value;
    constexpr int ai = pr == 1 ? 1 : 0, aj = pr == 0 ? 1 : 2;
    constexpr int Pi = p_of_axis(ai), Pj = p_of_axis(aj);
    df acc = df_zero();
    sfor<PL::m.n>([&](auto E) {
      constexpr int e = decltype(E)::value;
      constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
      if constexpr (pb && b == Pj) acc = acc + M[e] * G[a + NA * Pi];
      if constexpr (pb && b == Pi) acc = acc - M[e] * G[a + NA * Pj];
      if constexpr (pa && a == Pi) acc = acc - M[e] * G[Pj + NA * b];
      if constexpr (pa && a == Pj) acc = acc + M[e] * G[Pi + NA * b];
    });
    tau[pr] = acc;
  });
}

// kappa_xx + kappa_yy and kappa_zy (mol_kappa_extra in fb_device.cuh)
template <int PA, int PB>
__device__ __forceinline__ void mol_kappa_extra_df(const df *G, const df *M, df &kd, df &kzy) {
  using PL = Plan<PA, PB, K3C>;
  constexpr int NA = PL::NA, NB = PL::NB;
  constexpr bool pa = NA >= 4, pb = NB >= 4;
  constexpr int Px = p_of_axis(0), Py = p_of_axis(1), Pz = p_of_axis(2);
  df d = df_zero(), zy = df_zero();
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    if constexpr (pa && a == Px) d = d + M[e] * G[Px + NA * b];
    if constexpr (pa && a == Py) d = d + M[e] * G[Py + NA * b];
    if constexpr (pb && b == Px) d = d + M[e] * G[a + NA * Px];
    if constexpr (pb && b == Py) d = d + M[e] * G[a + NA * Py];
    if constexpr (pa && a == Py) zy = zy + M[e] * G[Pz + NA * b];
    if constexpr (pb && b == Py) zy = zy + M[e] * G[a + NA * Pz];
  });
  kd = d;
  kzy = zy;
}

// 4-point Lagrange weights on nodes -1, 0, 1, 2 and their derivatives in df
__device__ __forceinline__ void lagrange4_df(df p, df w[4], df *dw) {
  const df one = df_one(), two = df_make(2.0f);
  df pm1 = p - one, pm2 = p - two, pp1 = p + one;
  const df sixth = df_make(0.16666667f, -4.9670538e-09f);  // 1/6 as hi + lo
  df a = p * pm1;          // p(p-1)
  df b = pp1 * pm2;        // (p+1)(p-2)
  w[0] = -(a * pm2) * sixth;
  w[1] = (b * pm1) * 0.5f;
  w[2] = -(b * p) * 0.5f;
  w[3] = (a * pp1) * sixth;
  if (dw) {
    df p2 = p * p;
    df t3 = p2 * 3.0f;
    dw[0] = -((t3 - p * 6.0f) + two) * sixth;
    dw[1] = ((t3 - p * 4.0f) - one) * 0.5f;
    dw[2] = -((t3 - p * 2.0f) - two) * 0.5f;
    dw[3] = (t3 - one) * sixth;
  }
}

}  // namespace fb
