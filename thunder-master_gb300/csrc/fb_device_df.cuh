// fb_device_df.cuh -- double-float (FP32-pipe) forms of the Slater-Koster
// rotation, the molecular-frame density contraction and the bicubic table
// contraction used by the three-center kernels.  Same mathematics and same
// operation structure as the FP64 forms in fb_device.cuh (rotate_plan,
// mol_rho) and fb_common.cuh (interp3c); s and p shells only.
#pragma once
#include "fb_df.cuh"
#include "fb_device.cuh"

namespace fb {

struct RotDF {
  df p[3][3];
};
struct DRotDF {
  df p[3][3][3];
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
__device__ __forceinline__ void dtwister_df(const df dd[3][3][3], DRotDF &D) {
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) D.p[c][a][b] = dd[c][pperm(a)][pperm(b)];
}

template <int S>
__device__ __forceinline__ df Lrot_df(const RotDF &R, int k, int m) {
  if constexpr (S == 0) return df_one();
  else return R.p[k][m];
}
template <int S>
__device__ __forceinline__ df DLrot_df(const DRotDF &D, int c, int k, int m) {
  if constexpr (S == 0) return df_zero();
  else return D.p[c][k][m];
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

// molecular-frame density contraction (see mol_rho in fb_device.cuh):
// rR = rho R, G(e) = (L^T rho R)(e), H_c(e) = (dL_c^T rho R + L^T rho dR_c)(e)
template <int PA, int PB, int K>
__device__ __forceinline__ void mol_rR_df(const RotDF &R, const df *rho, df *rR) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA, NB = PL::NB;
  sfor<NA>([&](auto MU) {
    constexpr int mu = decltype(MU)::value;
    sfor<NB>([&](auto B) {
      constexpr int b = decltype(B)::value;
      constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
      df acc = df_zero();
      sfor<2 * sb + 1>([&](auto NU) {
        constexpr int k = decltype(NU)::value;
        df t = (sb == 0) ? rho[mu + NA * (ob + k)] : rho[mu + NA * (ob + k)] * Lrot_df<sb>(R, k, mb);
        acc = (k == 0) ? t : acc + t;
      });
      rR[mu + NA * b] = acc;
    });
  });
}

template <int PA, int PB, int K>
__device__ __forceinline__ void mol_G_df(const RotDF &R, const df *rR, df *G) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA;
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    df g = df_zero();
    sfor<2 * sa + 1>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      df t = (sa == 0) ? rR[(oa + k) + NA * b] : Lrot_df<sa>(R, k, ma) * rR[(oa + k) + NA * b];
      g = (k == 0) ? t : g + t;
    });
    G[e] = g;
  });
}

template <int PA, int PB, int K>
__device__ __forceinline__ void mol_H_df(const RotDF &R, const DRotDF &D, const df *rho, const df *rR,
                                         df (*H)[Plan<PA, PB, K>::m.n]) {
  using PL = Plan<PA, PB, K>;
  constexpr int NA = PL::NA;
  sfor<PL::m.n>([&](auto E) {
    constexpr int e = decltype(E)::value;
    constexpr int a = PL::m.mu[e], b = PL::m.nu[e];
    constexpr int sa = orb_shell(a), ma = orb_m(a), oa = shell_off(sa);
    constexpr int sb = orb_shell(b), mb = orb_m(b), ob = shell_off(sb);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      df h = df_zero();
      if constexpr (sa > 0) {
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          h = h + DLrot_df<sa>(D, c, k, ma) * rR[(oa + k) + NA * b];
        });
      }
      if constexpr (sb > 0) {
        sfor<2 * sa + 1>([&](auto KK) {
          constexpr int k = decltype(KK)::value;
          df t = df_zero();
          sfor<2 * sb + 1>([&](auto NU) {
            constexpr int q = decltype(NU)::value;
            t = t + rho[(oa + k) + NA * (ob + q)] * DLrot_df<sb>(D, c, q, mb);
          });
          h = h + ((sa == 0) ? t : Lrot_df<sa>(R, k, ma) * t);
        });
      }
      H[c][e] = h;
    }
  });
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
