// fb_mlp.cu -- MLP-3c surrogate: training-data generator (the FP64 table
// interpolator), BF16 tensor-core GEMMs with fused epilogues for the forward
// and backward passes, Adam.  All on the GPU; the host only sequences.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "fb_common.cuh"
#include "fb_mlp.h"
#include "fb_mma.cuh"

namespace fb {

// ---------------------------------------------------------------------------
// counter-based random numbers (splitmix64 finalizer of seed + index)
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ double unit_rand(unsigned long long seed, unsigned long long k) {
  return (double)(mix64(seed ^ mix64(k)) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
}

// ---------------------------------------------------------------------------
// per-Legendre-term table interpolation, FP64, with the reference's stencil
// and branch rules (getMEs_Fdata_3c, e.FDATA/M_Fdata_3c.f90:367-482): I[th][e]
// is the value the reference multiplies by P_th(cos theta)
// ---------------------------------------------------------------------------
__device__ void interp3c_terms(const MlpTables &tb, const Cell3cDev &cell, double x, double y,
                               double I[NTHETA][MLP_ME]) {
  const int NE = cell.nME;
  int ix = (int)(x / cell.dx) + 1;
  int iy = (int)(y / cell.dy) + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > cell.nx - 2) ix = cell.nx - 2;
  if (iy > cell.ny - 2) iy = cell.ny - 2;
  double px = x / cell.dx - ix + 1.0;
  double py = y / cell.dy - iy + 1.0;
  int nx = cell.nx;
  long long node0 = (long long)(iy - 1) * nx + (ix - 1);
  const double *tab = tb.table3c + cell.off;
  for (int th = 0; th < NTHETA; th++)
    for (int e = 0; e < MLP_ME; e++) I[th][e] = 0.0;
  if (tb.lin[cell.node_off + node0]) {
    double w00 = 1.0 - px - py;
    const double *T00 = tab + node0 * NTHETA * NE;
    const double *T10 = tab + (node0 + 1) * NTHETA * NE;
    const double *T01 = tab + (node0 + nx) * NTHETA * NE;
    for (int th = 0; th < NTHETA; th++)
      for (int e = 0; e < NE; e++)
        I[th][e] = w00 * T00[th * NE + e] + px * T10[th * NE + e] + py * T01[th * NE + e];
    return;
  }
  double wx[4], wy[4];
  lagrange4(px, wx, nullptr);
  lagrange4(py, wy, nullptr);
  const double *Tb = tab + (node0 - nx - 1) * NTHETA * NE;
  for (int j = 0; j < 4; j++)
    for (int k = 0; k < 4; k++) {
      double w = wx[k] * wy[j];
      const double *Tn = Tb + ((long long)j * nx + k) * NTHETA * NE;
      for (int th = 0; th < NTHETA; th++)
        for (int e = 0; e < NE; e++) I[th][e] = fma(w, Tn[th * NE + e], I[th][e]);
    }
}

// one training sample per thread: a species triple with a table, uniform
// (x, y) over its grid domain, uniform cos(theta) in [-1, 1]
__global__ void k_mlp_gen(long long n, long long first, unsigned long long seed, MlpTables tb,
                          const int *__restrict__ valid, int nvalid, int nsp, const float *__restrict__ scale,
                          float *__restrict__ feat3, int *__restrict__ trip, float *__restrict__ Y) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  unsigned long long k = (unsigned long long)(first + s) * 4ull;
  int tr = valid[min((int)(unit_rand(seed, k) * nvalid), nvalid - 1)];
  double u = unit_rand(seed, k + 1), v = unit_rand(seed, k + 2), c = 2.0 * unit_rand(seed, k + 3) - 1.0;
  int a = tr / (nsp * nsp), b = (tr / nsp) % nsp, kk = tr % nsp;
  const Cell3cDev &cell = tb.fd->c3[a][b][kk];
  double I[NTHETA][MLP_ME];
  interp3c_terms(tb, cell, u * cell.xmax, v * cell.ymax, I);
  feat3[3 * s] = (float)(2.0 * u - 1.0);
  feat3[3 * s + 1] = (float)(2.0 * v - 1.0);
  feat3[3 * s + 2] = (float)c;
  trip[s] = tr;
  for (int th = 0; th < NTHETA; th++)
    for (int e = 0; e < MLP_ME; e++) {
      int o = th * MLP_ME + e;
      Y[s * MLP_OUT + o] = (float)(I[th][e] / (double)scale[tr * MLP_OUT + o]);
    }
  for (int o = NTHETA * MLP_ME; o < MLP_OUT; o++) Y[s * MLP_OUT + o] = 0.0f;
}

// Validation samples, stratified by interpolation bin: bin = (triple, node
// (ix, iy) of the 4 x 4 stencil); the bin's region is the set of (x, y) whose
// clamped stencil index is (ix, iy) (getMEs_Fdata_3c, :367-376).  Targets as
// in k_mlp_gen; samples of bins without a table are marked with trip = -1.
__global__ void k_mlp_gen_bins(long long n, long long first, int per_bin, int cells, unsigned long long seed,
                               MlpTables tb, int nsp, const float *__restrict__ scale, float *__restrict__ feat3,
                               int *__restrict__ trip, float *__restrict__ Y) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  long long gs = first + s;
  int bin = (int)(gs / per_bin);
  int tr = bin / cells, node = bin % cells;
  int a = tr / (nsp * nsp), b = (tr / nsp) % nsp, kk = tr % nsp;
  const Cell3cDev &cell = tb.fd->c3[a][b][kk];
  bool ok = cell.off >= 0 && node < cell.nx * cell.ny;
  int ix = ok ? node % cell.nx + 1 : 2, iy = ok ? node / cell.nx + 1 : 2;  // 1-based
  ok = ok && ix >= 2 && ix <= cell.nx - 2 && iy >= 2 && iy <= cell.ny - 2;
  if (!ok) {
    trip[s] = -1;
    feat3[3 * s] = feat3[3 * s + 1] = feat3[3 * s + 2] = 0.0f;
    for (int o = 0; o < MLP_OUT; o++) Y[s * MLP_OUT + o] = 0.0f;
    return;
  }
  unsigned long long k = (unsigned long long)gs * 4ull;
  double xl = ix == 2 ? 0.0 : (ix - 1) * cell.dx, xh = ix == cell.nx - 2 ? cell.xmax : ix * cell.dx;
  double yl = iy == 2 ? 0.0 : (iy - 1) * cell.dy, yh = iy == cell.ny - 2 ? cell.ymax : iy * cell.dy;
  double x = xl + (xh - xl) * unit_rand(seed, k), y = yl + (yh - yl) * unit_rand(seed, k + 1);
  double c = 2.0 * unit_rand(seed, k + 2) - 1.0;
  double I[NTHETA][MLP_ME];
  interp3c_terms(tb, cell, x, y, I);
  feat3[3 * s] = (float)(2.0 * x / cell.xmax - 1.0);
  feat3[3 * s + 1] = (float)(2.0 * y / cell.ymax - 1.0);
  feat3[3 * s + 2] = (float)c;
  trip[s] = tr;
  for (int th = 0; th < NTHETA; th++)
    for (int e = 0; e < MLP_ME; e++) {
      int o = th * MLP_ME + e;
      Y[s * MLP_OUT + o] = (float)(I[th][e] / (double)scale[tr * MLP_OUT + o]);
    }
  for (int o = NTHETA * MLP_ME; o < MLP_OUT; o++) Y[s * MLP_OUT + o] = 0.0f;
}

// per-bin maximum over samples of max_ime |sum_theta P_theta(cos) (out - target) * scale|
__global__ void k_mlp_bin_err(long long n, long long first, int per_bin, const float *__restrict__ feat3,
                              const int *__restrict__ trip, const float *__restrict__ O, const float *__restrict__ Y,
                              const float *__restrict__ scale, const int *__restrict__ tmeta,
                              unsigned *__restrict__ bin_err) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int tr = trip[s];
  if (tr < 0) return;
  float c = feat3[3 * s + 2], c2 = c * c;
  float pl[5] = {1.0f, c, 0.5f * (3.0f * c2 - 1.0f), 0.5f * c * (5.0f * c2 - 3.0f),
                 0.125f * (3.0f - c2 * (30.0f - 35.0f * c2))};
  float mx = 0.0f;
  for (int e = 0; e < tmeta[tr]; e++) {
    float d = 0.0f;
    for (int th = 0; th < NTHETA; th++) {
      int o = th * MLP_ME + e;
      d += pl[th] * (O[s * MLP_OUT + o] - Y[s * MLP_OUT + o]) * scale[tr * MLP_OUT + o];
    }
    mx = fmaxf(mx, fabsf(d));
  }
  atomicMax(bin_err + (first + s) / per_bin, __float_as_uint(mx));  // non-negative floats order as integers
}

// input rows: 3 coordinates, the triple's embedding, zeros; plain and transposed
__global__ void k_mlp_input(int B, const float *__restrict__ feat3, const int *__restrict__ trip,
                            const float *__restrict__ emb, __nv_bfloat16 *__restrict__ X,
                            __nv_bfloat16 *__restrict__ Xt) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * MLP_IN) return;
  int r = idx / MLP_IN, k = idx % MLP_IN;
  int tr = trip[r] < 0 ? 0 : trip[r];
  __nv_bfloat16 h = __float2bfloat16_rn(0.0f);
  if (k < 3) {
    h = __float2bfloat16_rn(feat3[3 * r + k]);
  } else if (k < 3 + MLP_EMB) {
    h = __float2bfloat16_rn(emb[tr * MLP_EMB + (k - 3)]);
  } else if (k < MLP_LO + 3) {
    float f = feat3[3 * r + (k - MLP_LO)];
    h = __float2bfloat16_rn(f - __bfloat162float(__float2bfloat16_rn(f)));
  }
  X[idx] = h;
  if (Xt) Xt[(long long)k * B + r] = h;
}

// ---------------------------------------------------------------------------
// C[M][N] = sum_k A[m][k] B[n][k] (both BF16, K contiguous), FP32 accumulate.
// CTA tile 64 x 32, 4 warps of 16 rows; K staged through shared memory in
// steps of 32.  M % 64 == 0, N % 32 == 0, K % 32 == 0, lda and ldb % 8 == 0.
// blockIdx.z splits K (partial products into out + z * M * N).
// ---------------------------------------------------------------------------
enum { EPI_HIDDEN = 0, EPI_OUT = 1, EPI_BACK = 2, EPI_STORE = 3 };

struct EpiArgs {
  const float *bias;      // EPI_HIDDEN, EPI_OUT
  float *Z;               // EPI_HIDDEN: pre-activation out; EPI_BACK: pre-activation in
  __nv_bfloat16 *H, *Ht;  // EPI_HIDDEN: silu(z); EPI_BACK: dz = acc * silu'(z)
  float *out;             // EPI_OUT, EPI_STORE
  int ldz;                // row stride of Z / H / out
  int ldt;                // row stride of the transposed output
};

template <int EPI>
__global__ void __launch_bounds__(128) k_gemm_nt(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, int lda,
                                                 const __nv_bfloat16 *__restrict__ Bm, int ldb, EpiArgs ep) {
  __shared__ __align__(16) __nv_bfloat16 sA[64][40];
  __shared__ __align__(16) __nv_bfloat16 sB[32][40];
  int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  int m0 = blockIdx.x * 64, n0 = blockIdx.y * 32;
  int kslice = K / gridDim.z, k0 = blockIdx.z * kslice, k1 = k0 + kslice;
  float acc[4][4];
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0.0f;
  for (int kb = k0; kb < k1; kb += 32) {
    // A tile 64 x 32 = 256 chunks of 8 BF16; B tile 32 x 32 = 128 chunks
#pragma unroll
    for (int c = tid; c < 256; c += 128) {
      int r = c >> 2, cc = (c & 3) * 8;
      *reinterpret_cast<uint4 *>(&sA[r][cc]) =
          *reinterpret_cast<const uint4 *>(A + (long long)(m0 + r) * lda + kb + cc);
    }
    {
      int r = tid >> 2, cc = (tid & 3) * 8;
      *reinterpret_cast<uint4 *>(&sB[r][cc]) =
          *reinterpret_cast<const uint4 *>(Bm + (long long)(n0 + r) * ldb + kb + cc);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < 32; ks += 16) {
      uint32_t a[4];
      int r = warp * 16 + g;
      a[0] = *reinterpret_cast<const uint32_t *>(&sA[r][ks + 2 * t]);
      a[1] = *reinterpret_cast<const uint32_t *>(&sA[r + 8][ks + 2 * t]);
      a[2] = *reinterpret_cast<const uint32_t *>(&sA[r][ks + 2 * t + 8]);
      a[3] = *reinterpret_cast<const uint32_t *>(&sA[r + 8][ks + 2 * t + 8]);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        uint32_t b[2];
        b[0] = *reinterpret_cast<const uint32_t *>(&sB[8 * j + g][ks + 2 * t]);
        b[1] = *reinterpret_cast<const uint32_t *>(&sB[8 * j + g][ks + 2 * t + 8]);
        mma_bf16(acc[j], a, b);
      }
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int m = m0 + warp * 16 + g + (q >= 2 ? 8 : 0);
      int n = n0 + 8 * j + 2 * t + (q & 1);
      float v = acc[j][q];
      long long o = (long long)m * ep.ldz + n;
      if (EPI == EPI_HIDDEN) {
        float z = v + ep.bias[n];
        ep.Z[o] = z;
        __nv_bfloat16 h = __float2bfloat16_rn(silu(z));
        ep.H[o] = h;
        if (ep.Ht) ep.Ht[(long long)n * ep.ldt + m] = h;
      } else if (EPI == EPI_OUT) {
        ep.out[o] = v + ep.bias[n];
      } else if (EPI == EPI_BACK) {
        __nv_bfloat16 h = __float2bfloat16_rn(v * dsilu(ep.Z[o]));
        ep.H[o] = h;
        ep.Ht[(long long)n * ep.ldt + m] = h;
      } else {
        ep.out[(long long)blockIdx.z * M * N + o] = v;
      }
    }
}

// loss = sum over rows and used outputs of (O - Y)^2 / (50 B); dO = its gradient
__global__ void k_mlp_loss(int B, const float *__restrict__ O, const float *__restrict__ Y,
                           const int *__restrict__ trip, const int *__restrict__ tmeta, __nv_bfloat16 *__restrict__ dO,
                           __nv_bfloat16 *__restrict__ dOt, double *__restrict__ loss) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (idx < B * MLP_OUT) {
    int r = idx / MLP_OUT, o = idx % MLP_OUT;
    int e = o % MLP_ME;
    bool used = o < NTHETA * MLP_ME && e < tmeta[trip[r]];
    float d = used ? O[idx] - Y[idx] : 0.0f;
    const float inv = 1.0f / (float)(NTHETA * MLP_ME);
    l = d * d * inv;
    __nv_bfloat16 gd = __float2bfloat16_rn(2.0f * d * inv / (float)B);
    dO[idx] = gd;
    dOt[(long long)o * B + r] = gd;
  }
  // warp sum, one atomic per warp
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, (double)l / (double)B);
}

// sum of split-K partials into the gradient; rows >= mrows_used and columns
// >= ncols_used stay zero (padding of W1 columns and W4 rows); tie > 0:
// columns tie .. tie+2 share the weights of columns 0..2, so their
// gradients are added there
__global__ void k_wgrad_reduce(int M, int N, int S, const float *__restrict__ part, float *__restrict__ g,
                               int mrows_used, int ncols_used, int tie) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * N) return;
  int m = idx / N, n = idx % N;
  float v = 0.0f;
  for (int s = 0; s < S; s++) v += part[(long long)s * M * N + idx];
  if (tie > 0 && n < 3)
    for (int s = 0; s < S; s++) v += part[(long long)s * M * N + m * N + tie + n];
  g[idx] = (m < mrows_used && n < ncols_used) ? v : 0.0f;
}

// bias gradient: row sums of the transposed output gradients (one warp per row)
__global__ void k_bias_grad(int N, int B, const __nv_bfloat16 *__restrict__ Gt, float *__restrict__ g, int nused) {
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= N) return;
  float v = 0.0f;
  for (int b = lane; b < B; b += 32) v += __bfloat162float(Gt[(long long)w * B + b]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) g[w] = w < nused ? v : 0.0f;
}

// embedding gradient: input-gradient columns 3..18 added into the triple's row
__global__ void k_emb_grad(int B, const float *__restrict__ dXg, const int *__restrict__ trip, float *__restrict__ gemb) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * MLP_EMB) return;
  int r = idx / MLP_EMB, k = idx % MLP_EMB;
  atomicAdd(gemb + trip[r] * MLP_EMB + k, dXg[(long long)r * MLP_IN + 3 + k]);
}

__global__ void k_adam(long long n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.0f - b1) * gi;
  float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// BF16 copies of a weight matrix W[N][K]: plain and transposed (Wt[K][N]);
// tie > 0: columns tie .. tie+2 repeat columns 0..2 (W1's low-part inputs)
__global__ void k_pack_w(int N, int K, const float *__restrict__ W, __nv_bfloat16 *__restrict__ Wb,
                         __nv_bfloat16 *__restrict__ Wt, int tie) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * K) return;
  int n = idx / K, k = idx % K;
  int ks = (tie > 0 && k >= tie && k < tie + 3) ? k - tie : k;
  __nv_bfloat16 h = __float2bfloat16_rn(W[n * K + ks]);
  Wb[idx] = h;
  Wt[(long long)k * N + n] = h;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

#define MCU(call)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                              \
      return FB_ERR_CUDA;                                                                    \
    }                                                                                        \
  } while (0)
#define MCHK(call)                                        \
  do {                                                    \
    if ((call)) {                                         \
      err = std::string("allocation failed: ") + #call;   \
      return FB_ERR_CUDA;                                 \
    }                                                     \
  } while (0)

// BF16 weight blocks inside m.wbf (element offsets)
struct WOff {
  long long w1, w2, w3, w4, w1t, w2t, w3t, w4t, total;
};
WOff woff() {
  WOff o;
  o.w1 = 0;
  o.w2 = o.w1 + MLP_H * MLP_IN;
  o.w3 = o.w2 + MLP_H * MLP_H;
  o.w4 = o.w3 + MLP_H * MLP_H;
  o.w1t = o.w4 + MLP_OUT * MLP_H;
  o.w2t = o.w1t + MLP_H * MLP_IN;
  o.w3t = o.w2t + MLP_H * MLP_H;
  o.w4t = o.w3t + MLP_H * MLP_H;
  o.total = o.w4t + MLP_OUT * MLP_H;
  return o;
}

int pack_weights(MlpState &m, cudaStream_t s, std::string &err) {
  WOff o = woff();
  float *P = m.params.as<float>();
  __nv_bfloat16 *W = m.wbf.as<__nv_bfloat16>();
  struct {
    long long src, b, t;
    int n, k;
  } L[4] = {{m.o_w1, o.w1, o.w1t, MLP_H, MLP_IN},
            {m.o_w2, o.w2, o.w2t, MLP_H, MLP_H},
            {m.o_w3, o.w3, o.w3t, MLP_H, MLP_H},
            {m.o_w4, o.w4, o.w4t, MLP_OUT, MLP_H}};
  for (auto &l : L) {
    int n = l.n * l.k;
    k_pack_w<<<(n + 255) / 256, 256, 0, s>>>(l.n, l.k, P + l.src, W + l.b, W + l.t, l.src == m.o_w1 ? MLP_LO : 0);
  }
  MCU(cudaGetLastError());
  return FB_OK;
}

template <int EPI>
int gemm(int M, int N, int K, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, const EpiArgs &ep,
         int splitk, cudaStream_t s) {
  dim3 grid(M / 64, N / 32, splitk);
  k_gemm_nt<EPI><<<grid, 128, 0, s>>>(M, N, K, A, lda, B, ldb, ep);
  return (int)cudaGetLastError();
}

int ensure_batch(MlpState &m, int B, std::string &err) {
  if (B <= m.batch_cap) return FB_OK;
  size_t b = (size_t)B;
  MCHK(m.Z.ensure(3 * b * MLP_H * sizeof(float)));
  MCHK(m.H.ensure((4 * b * MLP_H) * sizeof(__nv_bfloat16)));
  MCHK(m.Ht.ensure((4 * b * MLP_H) * sizeof(__nv_bfloat16)));
  MCHK(m.O.ensure(b * MLP_OUT * sizeof(float)));
  MCHK(m.dO.ensure(b * MLP_OUT * sizeof(__nv_bfloat16)));
  MCHK(m.dOt.ensure(b * MLP_OUT * sizeof(__nv_bfloat16)));
  MCHK(m.dZ.ensure(3 * b * MLP_H * sizeof(__nv_bfloat16)));
  MCHK(m.dZt.ensure(3 * b * MLP_H * sizeof(__nv_bfloat16)));
  MCHK(m.dXg.ensure(b * MLP_IN * sizeof(float)));
  MCHK(m.part.ensure((size_t)64 * MLP_H * MLP_H * sizeof(float)));
  m.batch_cap = B;
  return FB_OK;
}

// activations of one batch: H[0] = input (B x 32, stride 32), H[1..3] hidden
struct Acts {
  __nv_bfloat16 *X, *Xt, *H[3], *Ht[3], *dZ[3], *dZt[3];
  float *Z[3];
};
Acts acts(MlpState &m, int B) {
  Acts a;
  __nv_bfloat16 *H = m.H.as<__nv_bfloat16>(), *Ht = m.Ht.as<__nv_bfloat16>();
  a.X = H;  // B x MLP_IN at the start of H
  a.Xt = Ht;
  for (int l = 0; l < 3; l++) {
    a.H[l] = H + (size_t)B * MLP_IN + (size_t)l * B * MLP_H;
    a.Ht[l] = Ht + (size_t)B * MLP_IN + (size_t)l * B * MLP_H;
    a.dZ[l] = m.dZ.as<__nv_bfloat16>() + (size_t)l * B * MLP_H;
    a.dZt[l] = m.dZt.as<__nv_bfloat16>() + (size_t)l * B * MLP_H;
    a.Z[l] = m.Z.as<float>() + (size_t)l * B * MLP_H;
  }
  return a;
}

// forward of B rows whose features / triples are on the device; outputs in m.O
int forward(MlpState &m, int B, const float *feat3, const int *trip, bool keep_t, cudaStream_t s, std::string &err) {
  Acts a = acts(m, B);
  WOff o = woff();
  const float *P = m.params.as<float>();
  const __nv_bfloat16 *W = m.wbf.as<__nv_bfloat16>();
  k_mlp_input<<<(B * MLP_IN + 255) / 256, 256, 0, s>>>(B, feat3, trip, P + m.o_emb, a.X, keep_t ? a.Xt : nullptr);
  MCU(cudaGetLastError());
  EpiArgs ep{};
  const __nv_bfloat16 *in = a.X;
  int kin = MLP_IN;
  const long long wo[3] = {o.w1, o.w2, o.w3}, bo[3] = {m.o_b1, m.o_b2, m.o_b3};
  for (int l = 0; l < 3; l++) {
    ep = EpiArgs{};
    ep.bias = P + bo[l];
    ep.Z = a.Z[l];
    ep.H = a.H[l];
    ep.Ht = keep_t ? a.Ht[l] : nullptr;
    ep.ldz = MLP_H;
    ep.ldt = B;
    MCU((cudaError_t)gemm<EPI_HIDDEN>(B, MLP_H, kin, in, kin, W + wo[l], kin, ep, 1, s));
    in = a.H[l];
    kin = MLP_H;
  }
  ep = EpiArgs{};
  ep.bias = P + m.o_b4;
  ep.out = m.O.as<float>();
  ep.ldz = MLP_OUT;
  MCU((cudaError_t)gemm<EPI_OUT>(B, MLP_OUT, MLP_H, in, MLP_H, W + o.w4, MLP_H, ep, 1, s));
  return FB_OK;
}

// loss and gradient of the batch already forwarded (keep_t); into m.grad
int backward(MlpState &m, int B, const float *Y, const int *trip, double *d_loss, cudaStream_t s, std::string &err) {
  Acts a = acts(m, B);
  WOff o = woff();
  const __nv_bfloat16 *W = m.wbf.as<__nv_bfloat16>();
  float *G = m.grad.as<float>();
  MCU(cudaMemsetAsync(G, 0, m.nparams * sizeof(float), s));
  __nv_bfloat16 *dO = m.dO.as<__nv_bfloat16>(), *dOt = m.dOt.as<__nv_bfloat16>();
  k_mlp_loss<<<(B * MLP_OUT + 255) / 256, 256, 0, s>>>(B, m.O.as<float>(), Y, trip, m.tmeta.as<int>(), dO, dOt,
                                                        d_loss);
  MCU(cudaGetLastError());
  int S = B >= 2048 ? 32 : (B >= 512 ? 8 : 1);  // split-K slices of the weight gradients
  while (S > 1 && (B / S) % 32) S >>= 1;
  float *part = m.part.as<float>();
  EpiArgs ep{};
  // layer 4: dW4 = dO^T H3, db4, dZ3 = (dO W4) * silu'(Z3)
  ep.out = part;
  ep.ldz = MLP_H;
  MCU((cudaError_t)gemm<EPI_STORE>(MLP_OUT, MLP_H, B, dOt, B, a.Ht[2], B, ep, S, s));
  k_wgrad_reduce<<<(MLP_OUT * MLP_H + 255) / 256, 256, 0, s>>>(MLP_OUT, MLP_H, S, part, G + m.o_w4,
                                                                 NTHETA * MLP_ME, MLP_H, 0);
  k_bias_grad<<<(MLP_OUT * 32 + 255) / 256, 256, 0, s>>>(MLP_OUT, B, dOt, G + m.o_b4, NTHETA * MLP_ME);
  MCU(cudaGetLastError());
  const __nv_bfloat16 *gin = dO;
  int kg = MLP_OUT;
  const long long wt[3] = {o.w2t, o.w3t, o.w4t};  // transposed weights of layers 2, 3, 4
  const long long wg[3] = {m.o_w1, m.o_w2, m.o_w3}, bg[3] = {m.o_b1, m.o_b2, m.o_b3};
  for (int l = 2; l >= 0; l--) {
    // dZ_l = (gin W_{l+1}) * silu'(Z_l); gin has kg columns, W_{l+1}^T is [128][kg]
    ep = EpiArgs{};
    ep.Z = a.Z[l];
    ep.H = a.dZ[l];
    ep.Ht = a.dZt[l];
    ep.ldz = MLP_H;
    ep.ldt = B;
    MCU((cudaError_t)gemm<EPI_BACK>(B, MLP_H, kg, gin, kg, W + wt[l], kg, ep, 1, s));
    // dW_l = dZ_l^T H_{l-1}, db_l
    const __nv_bfloat16 *hin_t = l == 0 ? a.Xt : a.Ht[l - 1];
    int kin = l == 0 ? MLP_IN : MLP_H;
    ep = EpiArgs{};
    ep.out = part;
    ep.ldz = kin;
    MCU((cudaError_t)gemm<EPI_STORE>(MLP_H, kin, B, a.dZt[l], B, hin_t, B, ep, S, s));
    k_wgrad_reduce<<<(MLP_H * kin + 255) / 256, 256, 0, s>>>(MLP_H, kin, S, part, G + wg[l], MLP_H,
                                                              l == 0 ? 3 + MLP_EMB : kin, l == 0 ? MLP_LO : 0);
    k_bias_grad<<<(MLP_H * 32 + 255) / 256, 256, 0, s>>>(MLP_H, B, a.dZt[l], G + bg[l], MLP_H);
    MCU(cudaGetLastError());
    gin = a.dZ[l];
    kg = MLP_H;
  }
  // input gradient (embedding columns): dX = dZ_1 W1, W1^T is [32][128]
  ep = EpiArgs{};
  ep.out = m.dXg.as<float>();
  ep.ldz = MLP_IN;
  MCU((cudaError_t)gemm<EPI_STORE>(B, MLP_IN, MLP_H, a.dZ[0], MLP_H, W + o.w1t, MLP_H, ep, 1, s));
  k_emb_grad<<<(B * MLP_EMB + 255) / 256, 256, 0, s>>>(B, m.dXg.as<float>(), trip, G + m.o_emb);
  MCU(cudaGetLastError());
  return FB_OK;
}

int adam_step(MlpState &m, double lr, cudaStream_t s, std::string &err) {
  const double b1 = 0.9, b2 = 0.999;
  m.adam_t++;
  float c1 = (float)(1.0 / (1.0 - std::pow(b1, (double)m.adam_t)));
  float c2 = (float)(1.0 / (1.0 - std::pow(b2, (double)m.adam_t)));
  long long n = m.nparams;
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, m.params.as<float>(), m.grad.as<float>(),
                                                      m.adam_m.as<float>(), m.adam_v.as<float>(), (float)lr,
                                                      (float)b1, (float)b2, c1, c2, 1.0e-8f);
  MCU(cudaGetLastError());
  return pack_weights(m, s, err);
}

}  // namespace

int mlp_init(MlpState &m, const FdataHost &f, unsigned long long seed, cudaStream_t s, std::string &err) {
  m.nsp = f.nspecies;
  m.ntrip = f.nspecies * f.nspecies * f.nspecies;
  // parameter blocks
  long long o = 0;
  m.o_emb = o;
  o += (long long)m.ntrip * MLP_EMB;
  m.o_w1 = o;
  o += MLP_H * MLP_IN;
  m.o_b1 = o;
  o += MLP_H;
  m.o_w2 = o;
  o += MLP_H * MLP_H;
  m.o_b2 = o;
  o += MLP_H;
  m.o_w3 = o;
  o += MLP_H * MLP_H;
  m.o_b3 = o;
  o += MLP_H;
  m.o_w4 = o;
  o += MLP_OUT * MLP_H;
  m.o_b4 = o;
  o += MLP_OUT;
  m.nparams = o;
  // output scales and ME counts per triple, from the host copy of the tables
  m.h_scale.assign((size_t)m.ntrip * MLP_OUT, 1.0f);
  m.h_nme.assign(m.ntrip, 0);
  for (int a = 0; a < m.nsp; a++)
    for (int b = 0; b < m.nsp; b++)
      for (int k = 0; k < m.nsp; k++) {
        const Cell3cDev &c = f.dev.c3[a][b][k];
        int tr = (a * m.nsp + b) * m.nsp + k;
        if (c.off < 0) continue;
        if (c.nME > MLP_ME) {
          err = "MLP-3c covers s and sp bases (at most 10 bcna matrix elements)";
          return FB_ERR_UNSUPPORTED;
        }
        m.h_nme[tr] = c.nME;
        long long nodes = (long long)c.nx * c.ny;
        for (int th = 0; th < NTHETA; th++)
          for (int e = 0; e < c.nME; e++) {
            double mx = 0.0;
            for (long long nd = 0; nd < nodes; nd++)
              mx = std::max(mx, std::fabs(f.table3c[c.off + nd * NTHETA * c.nME + th * c.nME + e]));
            m.h_scale[(size_t)tr * MLP_OUT + th * MLP_ME + e] = mx > 0.0 ? (float)mx : 1.0f;
          }
      }
  // seeded initial parameters: Glorot-uniform weights over the used fan-in,
  // zero biases, N(0, 1)-like embeddings (sum of uniforms)
  std::vector<float> p(m.nparams, 0.0f);
  unsigned long long k = 0;
  auto U = [&]() { return (float)unit_rand(seed, k++); };
  for (long long i = 0; i < (long long)m.ntrip * MLP_EMB; i++) p[m.o_emb + i] = (U() + U() + U() - 1.5f) * 2.0f;
  auto glorot = [&](long long off, int n, int kk, int nused, int kused) {
    float a = std::sqrt(6.0f / (float)(kused + nused));
    for (int r = 0; r < n; r++)
      for (int c = 0; c < kk; c++) p[off + (long long)r * kk + c] = (r < nused && c < kused) ? a * (2.0f * U() - 1.0f) : 0.0f;
  };
  glorot(m.o_w1, MLP_H, MLP_IN, MLP_H, 3 + MLP_EMB);
  glorot(m.o_w2, MLP_H, MLP_H, MLP_H, MLP_H);
  glorot(m.o_w3, MLP_H, MLP_H, MLP_H, MLP_H);
  glorot(m.o_w4, MLP_OUT, MLP_H, NTHETA * MLP_ME, MLP_H);
  MCHK(m.params.ensure(m.nparams * sizeof(float)));
  MCHK(m.grad.ensure(m.nparams * sizeof(float)));
  MCHK(m.adam_m.ensure(m.nparams * sizeof(float)));
  MCHK(m.adam_v.ensure(m.nparams * sizeof(float)));
  MCHK(m.wbf.ensure(woff().total * sizeof(__nv_bfloat16)));
  MCHK(m.scale.ensure(m.h_scale.size() * sizeof(float)));
  MCHK(m.tmeta.ensure(m.ntrip * sizeof(int)));
  MCU(cudaMemcpyAsync(m.params.p, p.data(), m.nparams * sizeof(float), cudaMemcpyHostToDevice, s));
  MCU(cudaMemsetAsync(m.adam_m.p, 0, m.nparams * sizeof(float), s));
  MCU(cudaMemsetAsync(m.adam_v.p, 0, m.nparams * sizeof(float), s));
  MCU(cudaMemcpyAsync(m.scale.p, m.h_scale.data(), m.h_scale.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  MCU(cudaMemcpyAsync(m.tmeta.p, m.h_nme.data(), m.ntrip * sizeof(int), cudaMemcpyHostToDevice, s));
  m.adam_t = 0;
  int st = pack_weights(m, s, err);
  if (st) return st;
  MCU(cudaStreamSynchronize(s));
  m.ready = true;
  return FB_OK;
}

static int gen_samples(MlpState &m, const MlpTables &t, long long n, long long first, unsigned long long seed,
                       float *feat3, int *trip, float *Y, cudaStream_t s, std::string &err) {
  std::vector<int> valid;
  for (int tr = 0; tr < m.ntrip; tr++)
    if (m.h_nme[tr] > 0) valid.push_back(tr);
  if (valid.empty()) {
    err = "no three-center tables loaded";
    return FB_ERR_STATE;
  }
  DevBuf dv;
  MCHK(dv.ensure(valid.size() * sizeof(int)));
  MCU(cudaMemcpyAsync(dv.p, valid.data(), valid.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  k_mlp_gen<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, first, seed, t, dv.as<int>(), (int)valid.size(), m.nsp,
                                                        m.scale.as<float>(), feat3, trip, Y);
  MCU(cudaGetLastError());
  MCU(cudaStreamSynchronize(s));
  dv.release();
  return FB_OK;
}

int mlp_samples(MlpState &m, const MlpTables &t, int n, unsigned long long seed, float *feat3, int *trip,
                float *target, cudaStream_t s, std::string &err) {
  if (!m.ready) {
    err = "MLP not initialized";
    return FB_ERR_STATE;
  }
  DevBuf f, tr, y;
  MCHK(f.ensure((size_t)n * 3 * sizeof(float)));
  MCHK(tr.ensure((size_t)n * sizeof(int)));
  MCHK(y.ensure((size_t)n * MLP_OUT * sizeof(float)));
  int st = gen_samples(m, t, n, 0, seed, f.as<float>(), tr.as<int>(), y.as<float>(), s, err);
  if (st) return st;
  MCU(cudaMemcpy(feat3, f.p, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost));
  MCU(cudaMemcpy(trip, tr.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
  MCU(cudaMemcpy(target, y.p, (size_t)n * MLP_OUT * sizeof(float), cudaMemcpyDeviceToHost));
  f.release();
  tr.release();
  y.release();
  return FB_OK;
}

int mlp_train(MlpState &m, const MlpTables &t, long long nsamples, int epochs, int batch, double lr,
              unsigned long long seed, double *hist, cudaStream_t s, std::string &err) {
  if (!m.ready) {
    err = "MLP not initialized";
    return FB_ERR_STATE;
  }
  if (batch < 64 || batch % 64 || nsamples < batch || epochs < 1) {
    err = "batch must be a positive multiple of 64 and at most nsamples";
    return FB_ERR_ARG;
  }
  long long nb = nsamples / batch;
  long long n = nb * batch;
  if (n > m.data_cap) {
    MCHK(m.dX.ensure((size_t)n * 3 * sizeof(float)));
    MCHK(m.dTrip.ensure((size_t)n * sizeof(int)));
    MCHK(m.dY.ensure((size_t)n * MLP_OUT * sizeof(float)));
    m.data_cap = n;
  }
  int st = gen_samples(m, t, n, 0, seed, m.dX.as<float>(), m.dTrip.as<int>(), m.dY.as<float>(), s, err);
  if (st) return st;
  if ((st = ensure_batch(m, batch, err))) return st;
  DevBuf dl;
  MCHK(dl.ensure(sizeof(double)));
  long long total = nb * epochs, step = 0;
  for (int ep = 0; ep < epochs; ep++) {
    MCU(cudaMemsetAsync(dl.p, 0, sizeof(double), s));
    // batches in a seeded order per epoch
    std::vector<long long> order(nb);
    for (long long b = 0; b < nb; b++) order[b] = b;
    for (long long b = nb - 1; b > 0; b--) {
      long long r = (long long)(unit_rand(seed ^ 0x5EEDull, (unsigned long long)(ep * nb + b)) * (b + 1));
      std::swap(order[b], order[std::min(r, b)]);
    }
    for (long long bi = 0; bi < nb; bi++, step++) {
      long long b0 = order[bi] * batch;
      // cosine decay to 1 % of the initial rate
      double lr_t = lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(M_PI * (double)step / (double)total)));
      if ((st = forward(m, batch, m.dX.as<float>() + 3 * b0, m.dTrip.as<int>() + b0, true, s, err))) return st;
      if ((st = backward(m, batch, m.dY.as<float>() + b0 * MLP_OUT, m.dTrip.as<int>() + b0, dl.as<double>(), s, err)))
        return st;
      if ((st = adam_step(m, lr_t, s, err))) return st;
    }
    double l = 0.0;
    MCU(cudaMemcpyAsync(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    MCU(cudaStreamSynchronize(s));
    if (hist) hist[ep] = l / (double)nb;
  }
  dl.release();
  return FB_OK;
}

int mlp_grad(MlpState &m, int n, const float *feat3, const int *trip, const float *target, float *grad,
             double *loss, cudaStream_t s, std::string &err) {
  if (!m.ready) {
    err = "MLP not initialized";
    return FB_ERR_STATE;
  }
  if (n < 64 || n % 64) {
    err = "the batch must be a positive multiple of 64 rows";
    return FB_ERR_ARG;
  }
  int st;
  if ((st = ensure_batch(m, n, err))) return st;
  DevBuf f, tr, y, dl;
  MCHK(f.ensure((size_t)n * 3 * sizeof(float)));
  MCHK(tr.ensure((size_t)n * sizeof(int)));
  MCHK(y.ensure((size_t)n * MLP_OUT * sizeof(float)));
  MCHK(dl.ensure(sizeof(double)));
  for (int r = 0; r < n; r++)
    if (trip[r] < 0 || trip[r] >= m.ntrip) {
      err = "triple index out of range";
      return FB_ERR_ARG;
    }
  MCU(cudaMemcpyAsync(f.p, feat3, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s));
  MCU(cudaMemcpyAsync(tr.p, trip, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s));
  MCU(cudaMemcpyAsync(y.p, target, (size_t)n * MLP_OUT * sizeof(float), cudaMemcpyHostToDevice, s));
  MCU(cudaMemsetAsync(dl.p, 0, sizeof(double), s));
  if ((st = forward(m, n, f.as<float>(), tr.as<int>(), true, s, err))) return st;
  if ((st = backward(m, n, y.as<float>(), tr.as<int>(), dl.as<double>(), s, err))) return st;
  MCU(cudaMemcpyAsync(grad, m.grad.p, m.nparams * sizeof(float), cudaMemcpyDeviceToHost, s));
  MCU(cudaMemcpyAsync(loss, dl.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  MCU(cudaStreamSynchronize(s));
  f.release();
  tr.release();
  y.release();
  dl.release();
  return FB_OK;
}

int mlp_validate(MlpState &m, const MlpTables &t, int per_bin, int cells, unsigned long long seed,
                 std::vector<float> &bin_err, cudaStream_t s, std::string &err) {
  if (!m.ready) {
    err = "MLP not initialized";
    return FB_ERR_STATE;
  }
  if (per_bin < 1) {
    err = "per_bin must be positive";
    return FB_ERR_ARG;
  }
  long long nbins = (long long)m.ntrip * cells, total = nbins * per_bin;
  const int chunk = 1 << 16;
  int st;
  if ((st = ensure_batch(m, chunk, err))) return st;
  DevBuf f, tr, y, be;
  MCHK(f.ensure((size_t)chunk * 3 * sizeof(float)));
  MCHK(tr.ensure((size_t)chunk * sizeof(int)));
  MCHK(y.ensure((size_t)chunk * MLP_OUT * sizeof(float)));
  MCHK(be.ensure((size_t)nbins * sizeof(unsigned)));
  MCU(cudaMemsetAsync(be.p, 0, nbins * sizeof(unsigned), s));
  for (long long first = 0; first < total; first += chunk) {
    long long n = std::min<long long>(chunk, total - first);
    int rows = (int)((n + 63) / 64 * 64);
    if (rows > n) {
      // pad rows: a valid triple index with zero features; excluded from the error
      MCU(cudaMemsetAsync(f.p, 0, (size_t)rows * 3 * sizeof(float), s));
      MCU(cudaMemsetAsync(tr.p, 0xff, (size_t)rows * sizeof(int), s));
    }
    k_mlp_gen_bins<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, first, per_bin, cells, seed, t, m.nsp,
                                                               m.scale.as<float>(), f.as<float>(), tr.as<int>(),
                                                               y.as<float>());
    MCU(cudaGetLastError());
    if ((st = forward(m, rows, f.as<float>(), tr.as<int>(), false, s, err))) return st;
    k_mlp_bin_err<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, first, per_bin, f.as<float>(), tr.as<int>(),
                                                              m.O.as<float>(), y.as<float>(), m.scale.as<float>(),
                                                              m.tmeta.as<int>(), be.as<unsigned>());
    MCU(cudaGetLastError());
  }
  std::vector<unsigned> bits(nbins);
  MCU(cudaMemcpyAsync(bits.data(), be.p, nbins * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  MCU(cudaStreamSynchronize(s));
  bin_err.resize(nbins);
  for (long long b = 0; b < nbins; b++) std::memcpy(&bin_err[b], &bits[b], sizeof(float));
  f.release();
  tr.release();
  y.release();
  be.release();
  return FB_OK;
}

int mlp_forward(MlpState &m, int n, const float *feat3, const int *trip, float *out, cudaStream_t s,
                std::string &err) {
  if (!m.ready) {
    err = "MLP not initialized";
    return FB_ERR_STATE;
  }
  if (n < 64 || n % 64) {
    err = "the batch must be a positive multiple of 64 rows";
    return FB_ERR_ARG;
  }
  for (int r = 0; r < n; r++)
    if (trip[r] < 0 || trip[r] >= m.ntrip) {
      err = "triple index out of range";
      return FB_ERR_ARG;
    }
  int st;
  if ((st = ensure_batch(m, n, err))) return st;
  DevBuf f, tr;
  MCHK(f.ensure((size_t)n * 3 * sizeof(float)));
  MCHK(tr.ensure((size_t)n * sizeof(int)));
  MCU(cudaMemcpyAsync(f.p, feat3, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s));
  MCU(cudaMemcpyAsync(tr.p, trip, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s));
  if ((st = forward(m, n, f.as<float>(), tr.as<int>(), false, s, err))) return st;
  MCU(cudaMemcpyAsync(out, m.O.p, (size_t)n * MLP_OUT * sizeof(float), cudaMemcpyDeviceToHost, s));
  MCU(cudaStreamSynchronize(s));
  f.release();
  tr.release();
  return FB_OK;
}

}  // namespace fb
