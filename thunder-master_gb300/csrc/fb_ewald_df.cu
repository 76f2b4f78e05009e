// fb_ewald_df.cu -- the Ewald matrix and its derivative (assemble_ewald,
// j.ASSEMBLERS/M_assemble_ewald_DOGS.f90:633-918; Dassemble_ewald,
// k.DASSEMBLERS/M_Dassemble_ewald_DOGS.f90:878-1000) in double-float on the
// FP32 pipe.  At SiC4096 the reference's box choice gives kappa = 0.05 / A,
// so the screened lattice sum reaches 5.5 / kappa = 108 A: about 124 of the
// 343 lattice vectors contribute an erfc term to each of the 8.4 M atom
// pairs, a billion erfc evaluations that take most of the FP64 kernel's
// time.  Here:
//   * erfc(x) and erfc(x) + 2 x exp(-x^2) / sqrt(pi) are piecewise degree-12
//     polynomials (fb_ewald_fit.h, interpolation error < 1e-18), evaluated
//     in double-float (the high-order terms, below 1e-7, in float);
//   * z, 1/z and the lattice vectors c = L + r_i - r_j are double-float; a
//     float pre-test of |c|^2 against the cutoff skips the rest, and each
//     lane walks its own accepted lattice vectors so the warp stays converged
//     on the expensive part;
//   * the reciprocal sum over the structure factors accumulates in
//     double-float (dacc) from hi/lo float copies of cos / sin(g . r_i).
// Every term keeps a relative error near 1e-14; the matrix and its
// derivative agree with the FP64 oracle to ~1e-13 (1/A, 1/A^2).
#include "fb_common_df.cuh"
#include "fb_ewald.h"
#include "fb_ewald_fit.h"

namespace fb {

namespace {

// per-atom cos(g . r_i), sin(g . r_i) as hi/lo floats in the structure-factor
// buffers, [i * ng + k]
__global__ void k_ewald_sf_df(EwaldArgs e) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)e.N * e.ng) return;
  int i = (int)(t / e.ng), k = (int)(t % e.ng);
  const double *g = e.gvec + 3 * k;
  double gr = g[0] * e.ratom[3 * i] + g[1] * e.ratom[3 * i + 1] + g[2] * e.ratom[3 * i + 2];
  double sn, cs;
  sincos(gr, &sn, &cs);
  df c = df_from(cs), s = df_from(sn);
  reinterpret_cast<float2 *>(e.sfc)[t] = make_float2(c.h, c.l);
  reinterpret_cast<float2 *>(e.sfs)[t] = make_float2(s.h, s.l);
}

__device__ __forceinline__ df ld(const float2 *p) {
  float2 v = *p;
  return df_make(v.x, v.y);
}

// fit f of fb_ewald_fit.h at x in [0, 5.5] (staged in shared memory):
// interval k = floor(4 x), local t = 8 (x - k/4) - 1 = 8 x - (2k + 1)
__device__ __forceinline__ df ew_fit(const float2 *fit, df x) {
  int k = (int)(x.h * 4.0f);
  k = k < 0 ? 0 : (k >= EW_FIT_NINT ? EW_FIT_NINT - 1 : k);
  df t = df_make(__fmul_rn(x.h, 8.0f), __fmul_rn(x.l, 8.0f)) + df_make(-(float)(2 * k + 1));
  const float2 *c = fit + k * EW_FIT_NC;
  float pt = c[EW_FIT_NC - 1].x;
#pragma unroll
  for (int j = EW_FIT_NC - 2; j >= 7; j--) pt = __fmaf_rn(pt, t.h, c[j].x);
  df p = df_make(pt);
#pragma unroll
  for (int j = 6; j >= 0; j--) p = p * t + ld(c + j);
  return p;
}

__device__ __forceinline__ void stage_fit(float2 *fit, int f) {
  for (int q = threadIdx.x; q < EW_FIT_NINT * EW_FIT_NC; q += blockDim.x)
    fit[q] = make_float2(EW_FIT[f][q / EW_FIT_NC][q % EW_FIT_NC][0], EW_FIT[f][q / EW_FIT_NC][q % EW_FIT_NC][1]);
}

// the next lattice vector at or after k whose float |L + d|^2 passes the
// cutoff pre-test (z > 1e-4 as the reference: only the zero vector of i == j
// fails it, every other z is at least 0.5 A), or nl
__device__ __forceinline__ int next_lattice(const EwaldArgs &e, int k, const float *d, float rcut2) {
  for (; k < e.nl; k++) {
    const float2 *L = e.lvec_df + 3 * k;
    float c0 = __fadd_rn(L[0].x, d[0]), c1 = __fadd_rn(L[1].x, d[1]), c2 = __fadd_rn(L[2].x, d[2]);
    float z2 = __fmaf_rn(c0, c0, __fmaf_rn(c1, c1, __fmul_rn(c2, c2)));
    if (z2 <= rcut2 && z2 > 1.0e-6f) return k;
  }
  return e.nl;
}

// c = L + r_i - r_j in df from the hi/lo copy of L (no FP64 operation: at
// FP64's rate the conversions alone would cost more than the df terms)
__device__ __forceinline__ void lattice_vec(const EwaldArgs &e, int k, const df *dd, df *c, df &z2) {
  const float2 *L = e.lvec_df + 3 * k;
#pragma unroll
  for (int a = 0; a < 3; a++) c[a] = ld(L + a) + dd[a];
  z2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
}

}  // namespace

// value: one 32 x 32 tile (bi <= bj) per block of 32 x 8 threads, 4 rows each
__global__ void __launch_bounds__(256) k_ewald_tiles_df(EwaldArgs e) {
  __shared__ float2 Ci[32][33], Si[32][33], Cj[32][33], Sj[32][33];
  __shared__ float2 fit[EW_FIT_NINT * EW_FIT_NC];
  stage_fit(fit, 0);
  int nb = (e.N + 31) / 32;
  int t = blockIdx.x, bi = 0;
  while (t >= nb - bi) {
    t -= nb - bi;
    bi++;
  }
  int bj = bi + t;
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int j = bj * 32 + tx;
  const float2 *sfc = reinterpret_cast<const float2 *>(e.sfc), *sfs = reinterpret_cast<const float2 *>(e.sfs);
  dacc acc[4];
#pragma unroll
  for (int q = 0; q < 4; q++) acc[q].s = acc[q].c = 0.0f;
  for (int k0 = 0; k0 < e.ng; k0 += 32) {
    __syncthreads();
    int k = k0 + tx;
    bool kv = k < e.ng;
    df st = kv ? df_from(e.stuff[k]) : df_zero();
    for (int r = ty; r < 32; r += 8) {
      int ii = bi * 32 + r, jj = bj * 32 + r;
      Ci[r][tx] = (kv && ii < e.N) ? sfc[(long long)ii * e.ng + k] : make_float2(0.0f, 0.0f);
      Si[r][tx] = (kv && ii < e.N) ? sfs[(long long)ii * e.ng + k] : make_float2(0.0f, 0.0f);
      df cj = (kv && jj < e.N) ? ld(sfc + (long long)jj * e.ng + k) : df_zero();
      df sj = (kv && jj < e.N) ? ld(sfs + (long long)jj * e.ng + k) : df_zero();
      cj = cj * st;
      sj = sj * st;
      Cj[r][tx] = make_float2(cj.h, cj.l);
      Sj[r][tx] = make_float2(sj.h, sj.l);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < 32; kk++) {
      df cj = ld(&Cj[tx][kk]), sj = ld(&Sj[tx][kk]);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        int r = ty + 8 * q;
        dacc_add(acc[q], ld(&Ci[r][kk]), cj);
        dacc_add(acc[q], ld(&Si[r][kk]), sj);
      }
    }
  }
  // screened lattice sum; lanes without an output (beyond N, lower
  // triangle of a diagonal tile) take no lattice vector but stay in the loop
  double rc = e.kappa > 0.0 ? 5.5 / e.kappa : 1.0e150;
  float rcut2 = (float)(rc * rc * (1.0 + 1.0e-5));
  df kap = df_from(e.kappa);
#pragma unroll 1
  for (int q = 0; q < 4; q++) {
    int i = bi * 32 + ty + 8 * q;
    bool act = j < e.N && i < e.N && !(bi == bj && j < i);
    double dd64[3] = {0.0, 0.0, 0.0};
    if (act)
      for (int a = 0; a < 3; a++) dd64[a] = e.ratom[3 * i + a] - e.ratom[3 * j + a];
    df dd[3] = {df_from(dd64[0]), df_from(dd64[1]), df_from(dd64[2])};
    float df3[3] = {dd[0].h, dd[1].h, dd[2].h};
    dacc lat;
    lat.s = lat.c = 0.0f;
    int k = act ? next_lattice(e, 0, df3, rcut2) : e.nl;
    while (__any_sync(0xffffffffu, k < e.nl)) {
      if (k < e.nl) {
        df c[3], z2;
        lattice_vec(e, k, dd, c, z2);
        df z = df_sqrt(z2);
        df x = kap * z;
        if (x.h < EW_FIT_XMAX) dacc_add(lat, ew_fit(fit, x), df_rcp(z));
        k = next_lattice(e, k + 1, df3, rcut2);
      }
    }
    if (!act) continue;
    df v = dacc_val(acc[q]) + dacc_val(lat);
    double vv = df_to(v);
    if (i == j) vv -= 2.0 * e.kappa / sqrt(3.141592653589793238462643);
    e.ewald[(long long)i * e.N + j] = vv;
    e.ewald[(long long)j * e.N + i] = vv;
  }
}

// derivative: dewald(:, i, j) = - sum_g stuff g sin(g . (r_i - r_j))
//   - sum_L c (2 exp(-x^2) x / sqrt(pi) + erfc(x)) / z^3, x = kappa z,
// c = L + r_i - r_j; dewald(:, j, i) = -dewald(:, i, j); zero for i == j
__global__ void __launch_bounds__(256) k_dewald_tiles_df(EwaldArgs e) {
  __shared__ float2 Ci[32][33], Si[32][33], Cj[32][33], Sj[32][33], W[3][32];
  __shared__ float2 fit[EW_FIT_NINT * EW_FIT_NC];
  stage_fit(fit, 1);
  int nb = (e.N + 31) / 32;
  int t = blockIdx.x, bi = 0;
  while (t >= nb - bi) {
    t -= nb - bi;
    bi++;
  }
  int bj = bi + t;
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int j = bj * 32 + tx;
  const float2 *sfc = reinterpret_cast<const float2 *>(e.sfc), *sfs = reinterpret_cast<const float2 *>(e.sfs);
  dacc acc[4][3];
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int c = 0; c < 3; c++) acc[q][c].s = acc[q][c].c = 0.0f;
  for (int k0 = 0; k0 < e.ng; k0 += 32) {
    __syncthreads();
    int k = k0 + tx;
    bool kv = k < e.ng;
    for (int r = ty; r < 32; r += 8) {
      int ii = bi * 32 + r, jj = bj * 32 + r;
      float2 z0 = make_float2(0.0f, 0.0f);
      Ci[r][tx] = (kv && ii < e.N) ? sfc[(long long)ii * e.ng + k] : z0;
      Si[r][tx] = (kv && ii < e.N) ? sfs[(long long)ii * e.ng + k] : z0;
      Cj[r][tx] = (kv && jj < e.N) ? sfc[(long long)jj * e.ng + k] : z0;
      Sj[r][tx] = (kv && jj < e.N) ? sfs[(long long)jj * e.ng + k] : z0;
    }
    if (ty < 3) {
      df w = kv ? df_from(e.stuff[k] * e.gvec[3 * k + ty]) : df_zero();
      W[ty][tx] = make_float2(w.h, w.l);
    }
    __syncthreads();
#pragma unroll 1
    for (int kk = 0; kk < 32; kk++) {
      df cj = ld(&Cj[tx][kk]), sj = ld(&Sj[tx][kk]);
      df w0 = ld(&W[0][kk]), w1 = ld(&W[1][kk]), w2 = ld(&W[2][kk]);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        int r = ty + 8 * q;
        // -sin(g . (r_i - r_j)) = ci sj - si cj
        df ms = ld(&Ci[r][kk]) * sj - ld(&Si[r][kk]) * cj;
        dacc_add(acc[q][0], w0, ms);
        dacc_add(acc[q][1], w1, ms);
        dacc_add(acc[q][2], w2, ms);
      }
    }
  }
  double rc = e.kappa > 0.0 ? 5.5 / e.kappa : 1.0e150;
  float rcut2 = (float)(rc * rc * (1.0 + 1.0e-5));
  df kap = df_from(e.kappa);
#pragma unroll 1
  for (int q = 0; q < 4; q++) {
    int i = bi * 32 + ty + 8 * q;
    bool act = j < e.N && i < e.N && !(bi == bj && j < i);
    bool diag = act && i == j;
    double dd64[3] = {0.0, 0.0, 0.0};
    if (act)
      for (int a = 0; a < 3; a++) dd64[a] = e.ratom[3 * i + a] - e.ratom[3 * j + a];
    df dd[3] = {df_from(dd64[0]), df_from(dd64[1]), df_from(dd64[2])};
    float df3[3] = {dd[0].h, dd[1].h, dd[2].h};
    dacc lat[3];
#pragma unroll
    for (int c = 0; c < 3; c++) lat[c].s = lat[c].c = 0.0f;
    int k = (act && !diag) ? next_lattice(e, 0, df3, rcut2) : e.nl;
    while (__any_sync(0xffffffffu, k < e.nl)) {
      if (k < e.nl) {
        df c[3], z2;
        lattice_vec(e, k, dd, c, z2);
        df z = df_sqrt(z2);
        df x = kap * z;
        if (x.h < EW_FIT_XMAX) {
          df rz = df_rcp(z);
          df F = ew_fit(fit, x) * (rz * rz * rz);
#pragma unroll
          for (int a = 0; a < 3; a++) dacc_add(lat[a], c[a], F);
        }
        k = next_lattice(e, k + 1, df3, rcut2);
      }
    }
    if (!act) continue;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      double v = diag ? 0.0 : df_to(dacc_val(acc[q][a]) - dacc_val(lat[a]));
      e.dewald[((long long)i * e.N + j) * 3 + a] = v;
      e.dewald[((long long)j * e.N + i) * 3 + a] = -v;
    }
  }
}

int launch_ewald_matrix_df(const EwaldArgs &e, cudaStream_t s) {
  if (e.ng > 0) {
    long long n = (long long)e.N * e.ng;
    k_ewald_sf_df<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(e);
    FB_LAUNCH_CHECK();
  }
  long long nb = (e.N + 31) / 32;
  k_ewald_tiles_df<<<(unsigned)(nb * (nb + 1) / 2), 256, 0, s>>>(e);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dewald_tiles_df(const EwaldArgs &e, cudaStream_t s) {
  if (e.ng > 0) {
    long long n = (long long)e.N * e.ng;
    k_ewald_sf_df<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(e);
    FB_LAUNCH_CHECK();
  }
  long long nb = (e.N + 31) / 32;
  k_dewald_tiles_df<<<(unsigned)(nb * (nb + 1) / 2), 256, 0, s>>>(e);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
