// fb_mlp_eval.cu -- MLP-3c inference for the assembly: per triplet, the
// network's Legendre coefficients combined with P_l(cos theta) into the
// values the table walk of getMEs_Fdata_3c (e.FDATA/M_Fdata_3c.f90:293-517)
// produces, and, for the force pass, their derivatives with respect to the
// bond-charge distance, the neutral-atom distance and cos(theta)
// (getDMEs_Fdata_3c, :549-846) by forward-mode tangents through the network.
//
// BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation).  One warp takes
// 16 triplets at a time; the three tangents ride along as 48 extra rows of
// the same products (a tangent row's pre-activation needs no bias and its
// activation is silu'(z) times it, z being the primal row's pre-activation
// that the same thread holds).  The results go to a buffer that the
// double-float three-center kernels read in place of the table walk.
#include "fb_common_df.cuh"
#include "fb_mlp.h"
#include "fb_mma.cuh"

namespace fb {

namespace {

constexpr int WS1 = MLP_IN + 8;  // padded row strides (BF16 elements): conflict-free fragment loads
constexpr int WSH = MLP_H + 8;
constexpr int OUT_USED = NTHETA * MLP_ME;  // 50
constexpr int OST = 52;                    // row stride of the FP32 output staging

struct MlpSmemLayout {
  static constexpr int w1 = 0;
  static constexpr int w2 = w1 + MLP_H * WS1 * 2;
  static constexpr int w3 = w2 + MLP_H * WSH * 2;
  static constexpr int w4 = w3 + MLP_H * WSH * 2;
  static constexpr int bias = w4 + MLP_OUT * WSH * 2;           // b1, b2, b3 [128], b4 [64] (FP32)
  static constexpr int w1t = bias + (3 * MLP_H + MLP_OUT) * 4;  // W1 columns 0..2 as FP32 [3][128]
  static constexpr int warps = w1t + 3 * MLP_H * 4;             // per-warp areas start here
};

}  // namespace


template <int NTAN>
struct EvalShape {
  static constexpr int MT = 1 + NTAN;          // m-tiles per warp (primal + tangents)
  static constexpr int R = 16 * MT;            // rows per warp
  static constexpr int act_bytes = R * WSH * 2;
  static constexpr int warp_bytes = 2 * act_bytes + 16 * 16;  // two activation buffers + row info
  static constexpr int warps = NTAN ? 3 : 8;
  static constexpr int smem = MlpSmemLayout::warps + warps * warp_bytes;
};

// A fragment (rows r0 .. r0+15, k-step k0) from a BF16 row-major buffer
__device__ __forceinline__ void load_a(const __nv_bfloat16 *buf, int stride, int r0, int k0, int g, int t,
                                       uint32_t a[4]) {
  const __nv_bfloat16 *p = buf + (r0 + g) * stride + k0 + 2 * t;
  a[0] = *reinterpret_cast<const uint32_t *>(p);
  a[1] = *reinterpret_cast<const uint32_t *>(p + 8 * stride);
  a[2] = *reinterpret_cast<const uint32_t *>(p + 8);
  a[3] = *reinterpret_cast<const uint32_t *>(p + 8 * stride + 8);
}
// B fragment (n-tile n0, k-step k0) from a weight matrix W[n][k] in shared memory
__device__ __forceinline__ void load_b(const __nv_bfloat16 *W, int stride, int n0, int k0, int g, int t,
                                       uint32_t b[2]) {
  const __nv_bfloat16 *p = W + (n0 + g) * stride + k0 + 2 * t;
  b[0] = *reinterpret_cast<const uint32_t *>(p);
  b[1] = *reinterpret_cast<const uint32_t *>(p + 8);
}

// one hidden layer (K = 128, N = 128) for MT m-tiles: out = act(in W^T + b)
template <int MT>
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16 *in, __nv_bfloat16 *outb, const __nv_bfloat16 *W,
                                             const float *b, int g, int t) {
#pragma unroll 1
  for (int ng = 0; ng < MLP_H / 32; ng++) {
    float acc[MT][4][4];
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[m][j][q] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < MLP_H; k0 += 16) {
      uint32_t bf[4][2];
#pragma unroll
      for (int j = 0; j < 4; j++) load_b(W, WSH, ng * 32 + 8 * j, k0, g, t, bf[j]);
#pragma unroll
      for (int m = 0; m < MT; m++) {
        uint32_t a[4];
        load_a(in, WSH, 16 * m, k0, g, t, a);
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[m][j], a, bf[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        int r = g + (q >= 2 ? 8 : 0), n = ng * 32 + 8 * j + 2 * t + (q & 1);
        float z = acc[0][j][q] + b[n];
        float sg = sigmoid(z);
        outb[r * WSH + n] = __float2bfloat16_rn(z * sg);
        if (MT > 1) {
          float ds = sg * (1.0f + z * (1.0f - sg));
#pragma unroll
          for (int m = 1; m < MT; m++) outb[(16 * m + r) * WSH + n] = __float2bfloat16_rn(ds * acc[m][j][q]);
        }
      }
  }
}

template <int NTAN>
__global__ void __launch_bounds__(32 * EvalShape<NTAN>::warps) k_mlp_eval(MlpEvalArgs a, const FdataDev *__restrict__ fdp,
                                                                           const double *__restrict__ ratom,
                                                                           const int *__restrict__ isp,
                                                                           Ctx3c c) {
  using S = EvalShape<NTAN>;
  constexpr int MT = S::MT;
  extern __shared__ __align__(16) unsigned char smem[];
  using L = MlpSmemLayout;
  __nv_bfloat16 *W1 = reinterpret_cast<__nv_bfloat16 *>(smem + L::w1);
  __nv_bfloat16 *W2 = reinterpret_cast<__nv_bfloat16 *>(smem + L::w2);
  __nv_bfloat16 *W3 = reinterpret_cast<__nv_bfloat16 *>(smem + L::w3);
  __nv_bfloat16 *W4 = reinterpret_cast<__nv_bfloat16 *>(smem + L::w4);
  float *bias = reinterpret_cast<float *>(smem + L::bias);
  float *w1t = reinterpret_cast<float *>(smem + L::w1t);
  // stage the network (plain weights; padded rows)
  const __nv_bfloat16 *gw = a.wbf;
  for (int i = threadIdx.x; i < MLP_H * MLP_IN; i += blockDim.x) W1[(i / MLP_IN) * WS1 + i % MLP_IN] = gw[i];
  gw += MLP_H * MLP_IN;
  for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x) W2[(i / MLP_H) * WSH + i % MLP_H] = gw[i];
  gw += MLP_H * MLP_H;
  for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x) W3[(i / MLP_H) * WSH + i % MLP_H] = gw[i];
  gw += MLP_H * MLP_H;
  for (int i = threadIdx.x; i < MLP_OUT * MLP_H; i += blockDim.x) W4[(i / MLP_H) * WSH + i % MLP_H] = gw[i];
  for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
    bias[i] = a.params[a.o_b1 + i];
    bias[MLP_H + i] = a.params[a.o_b2 + i];
    bias[2 * MLP_H + i] = a.params[a.o_b3 + i];
#pragma unroll
    for (int q = 0; q < 3; q++) w1t[q * MLP_H + i] = __bfloat162float(a.wbf[i * MLP_IN + q]);
  }
  for (int i = threadIdx.x; i < MLP_OUT; i += blockDim.x) bias[3 * MLP_H + i] = a.params[a.o_b4 + i];
  __syncthreads();

  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  unsigned char *wbase = smem + L::warps + warp * S::warp_bytes;
  __nv_bfloat16 *act0 = reinterpret_cast<__nv_bfloat16 *>(wbase);
  __nv_bfloat16 *act1 = reinterpret_cast<__nv_bfloat16 *>(wbase + S::act_bytes);
  float *outs = reinterpret_cast<float *>(wbase);  // layer-4 output staging (aliases act0)
  float *rinfo = reinterpret_cast<float *>(wbase + 2 * S::act_bytes);  // [16][4]: triple, cos, 2/xmax, 2/ymax
  const FdataDev &fd = *fdp;
  int nchunks = (a.n + 15) / 16;
  int gw_id = blockIdx.x * S::warps + warp, nw = gridDim.x * S::warps;
  for (int ch = gw_id; ch < nchunks; ch += nw) {
    // ---- inputs: one lane per triplet ------------------------------------
    if (lane < 16) {
      int i = ch * 16 + lane;
      float f[3] = {0.0f, 0.0f, 0.0f}, sx = 0.0f, sy = 0.0f;
      int tr = 0;
      if (i < a.n && a.pts) {
        tr = a.ptrip[i];
        int ka = tr / (a.nsp * a.nsp), kb = (tr / a.nsp) % a.nsp, kc = tr % a.nsp;
        const Cell3cDev &cell = fd.c3[ka][kb][kc];
        sx = (float)(2.0 / cell.xmax);
        sy = (float)(2.0 / cell.ymax);
        f[0] = (float)(a.pts[3 * i] * (2.0 / cell.xmax) - 1.0);
        f[1] = (float)(a.pts[3 * i + 1] * (2.0 / cell.ymax) - 1.0);
        f[2] = a.pts[3 * i + 2];
      } else if (i < a.n) {
        GeomFP64 h;
        trip_geom_fp64(c, a.list[i], h);
        int ka = isp[h.iat], kb = isp[h.jat], kc = isp[h.ia];
        const Cell3cDev &cell = fd.c3[ka][kb][kc];
        tr = (ka * a.nsp + kb) * a.nsp + kc;
        sx = (float)(2.0 / cell.xmax);
        sy = (float)(2.0 / cell.ymax);
        f[0] = (float)(h.x * (2.0 / cell.xmax) - 1.0);
        f[1] = (float)(h.z * (2.0 / cell.ymax) - 1.0);
        f[2] = trip_cost_df(h).h;
      }
      __nv_bfloat16 *row = act0 + lane * WSH;
#pragma unroll
      for (int k = 0; k < 3; k++) row[k] = __float2bfloat16_rn(f[k]);
      const float *em = a.params + a.o_emb + tr * MLP_EMB;
#pragma unroll
      for (int k = 0; k < MLP_EMB; k++) row[3 + k] = __float2bfloat16_rn(em[k]);
#pragma unroll
      for (int k = 3 + MLP_EMB; k < MLP_IN; k++) row[k] = __float2bfloat16_rn(0.0f);
#pragma unroll
      for (int k = 0; k < 3; k++) row[MLP_LO + k] = __float2bfloat16_rn(f[k] - __bfloat162float(row[k]));
      rinfo[4 * lane] = __int_as_float(tr);
      rinfo[4 * lane + 1] = f[2];
      rinfo[4 * lane + 2] = sx;
      rinfo[4 * lane + 3] = sy;
    }
    __syncwarp();
    // ---- layer 1 (K = 32): primal by MMA, tangents from W1's columns ---------
    float sxg[2], syg[2];
#pragma unroll
    for (int h2 = 0; h2 < 2; h2++) {
      sxg[h2] = rinfo[4 * (g + 8 * h2) + 2];
      syg[h2] = rinfo[4 * (g + 8 * h2) + 3];
    }
#pragma unroll 1
    for (int ng = 0; ng < MLP_H / 32; ng++) {
      float acc[4][4];
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = 0.0f;
#pragma unroll
      for (int k0 = 0; k0 < MLP_IN; k0 += 16) {
        uint32_t ar[4];
        load_a(act0, WSH, 0, k0, g, t, ar);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          uint32_t bf[2];
          load_b(W1, WS1, ng * 32 + 8 * j, k0, g, t, bf);
          mma_bf16(acc[j], ar, bf);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          int h2 = q >= 2 ? 1 : 0, r = g + 8 * h2, n = ng * 32 + 8 * j + 2 * t + (q & 1);
          float z = acc[j][q] + bias[n];
          float sg = sigmoid(z);
          act1[r * WSH + n] = __float2bfloat16_rn(z * sg);
          if (NTAN) {
            float ds = sg * (1.0f + z * (1.0f - sg));
            act1[(16 + r) * WSH + n] = __float2bfloat16_rn(ds * w1t[n] * sxg[h2]);
            act1[(32 + r) * WSH + n] = __float2bfloat16_rn(ds * w1t[MLP_H + n] * syg[h2]);
            act1[(48 + r) * WSH + n] = __float2bfloat16_rn(ds * w1t[2 * MLP_H + n]);
          }
        }
    }
    __syncwarp();
    // ---- layers 2 and 3 ----------------------------------------------------
    hidden_layer<MT>(act1, act0, W2, bias + MLP_H, g, t);
    __syncwarp();
    hidden_layer<MT>(act0, act1, W3, bias + 2 * MLP_H, g, t);
    __syncwarp();
    // ---- layer 4 (N = 50 used: n-tiles 0..6) -> FP32 staging ------------------
#pragma unroll 1
    for (int ng = 0; ng < 2; ng++) {
      float acc[MT][4][4];
#pragma unroll
      for (int m = 0; m < MT; m++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc[m][j][q] = 0.0f;
      const int nt = ng == 0 ? 4 : 3;
#pragma unroll
      for (int k0 = 0; k0 < MLP_H; k0 += 16) {
        uint32_t bf[4][2];
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (j < nt) load_b(W4, WSH, ng * 32 + 8 * j, k0, g, t, bf[j]);
#pragma unroll
        for (int m = 0; m < MT; m++) {
          uint32_t ar[4];
          load_a(act1, WSH, 16 * m, k0, g, t, ar);
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (j < nt) mma_bf16(acc[m][j], ar, bf[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          int r = g + (q >= 2 ? 8 : 0), n = ng * 32 + 8 * j + 2 * t + (q & 1);
          if (j < nt && n < OUT_USED) {
            outs[r * OST + n] = acc[0][j][q] + bias[3 * MLP_H + n];
#pragma unroll
            for (int m = 1; m < MT; m++) outs[(16 * m + r) * OST + n] = acc[m][j][q];
          }
        }
    }
    __syncwarp();
    // ---- Legendre combination, 2 lanes per triplet (5 MEs each) ----------------
    {
      int r = lane >> 1, i = ch * 16 + r;
      if (i < a.n) {
        int tr = __float_as_int(rinfo[4 * r]);
        float cth = rinfo[4 * r + 1];
        float c2 = cth * cth;
        float pl[5] = {1.0f, cth, 0.5f * (3.0f * c2 - 1.0f), 0.5f * cth * (5.0f * c2 - 3.0f),
                       0.125f * (3.0f - c2 * (30.0f - 35.0f * c2))};
        float dpl[5] = {0.0f, 1.0f, 3.0f * cth, (15.0f * c2 - 3.0f) * 0.5f, 0.5f * cth * (35.0f * c2 - 15.0f)};
        const float *sc = a.scale + tr * MLP_OUT;
#pragma unroll
        for (int ee = 0; ee < 5; ee++) {
          int e = (lane & 1) * 5 + ee;
          float F = 0.0f, Dp = 0.0f, Dx = 0.0f, Dy = 0.0f;
#pragma unroll
          for (int th = 0; th < NTHETA; th++) {
            int o = th * MLP_ME + e;
            float v = outs[r * OST + o] * sc[o];
            F = fmaf(pl[th], v, F);
            if (NTAN) {
              Dp = fmaf(dpl[th], v, Dp);
              Dx = fmaf(pl[th], outs[(16 + r) * OST + o] * sc[o], Dx);
              Dy = fmaf(pl[th], outs[(32 + r) * OST + o] * sc[o], Dy);
              Dp = fmaf(pl[th], outs[(48 + r) * OST + o] * sc[o], Dp);
            }
          }
          if (NTAN) {
            float *o4 = a.out + (long long)i * 4 * MLP_ME;
            o4[e] = F;
            o4[MLP_ME + e] = Dp;
            o4[2 * MLP_ME + e] = Dx;
            o4[3 * MLP_ME + e] = Dy;
          } else {
            a.out[(long long)i * MLP_ME + e] = F;
          }
        }
      }
    }
    __syncwarp();
  }
}

int launch_mlp_eval(const MlpEvalArgs &m, const AsmArgs &a, bool tangents, int nsm, cudaStream_t s) {
  if (m.n == 0) return 0;
  Ctx3c c = make3c(a);
  if (tangents) {
    using S = EvalShape<3>;
    cudaError_t e = cudaFuncSetAttribute(k_mlp_eval<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem);
    if (e != cudaSuccess) return (int)e;
    int chunks = (m.n + 15) / 16, blocks = (chunks + S::warps - 1) / S::warps;
    if (blocks > nsm) blocks = nsm;
    k_mlp_eval<3><<<blocks, 32 * S::warps, S::smem, s>>>(m, a.fd, a.ratom, a.isp, c);
  } else {
    using S = EvalShape<0>;
    cudaError_t e = cudaFuncSetAttribute(k_mlp_eval<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem);
    if (e != cudaSuccess) return (int)e;
    int chunks = (m.n + 15) / 16, blocks = (chunks + S::warps - 1) / S::warps;
    if (blocks > nsm) blocks = nsm;
    k_mlp_eval<0><<<blocks, 32 * S::warps, S::smem, s>>>(m, a.fd, a.ratom, a.isp, c);
  }
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
