// fb_mlp_tc.cu -- MLP-3c evaluation on the Blackwell tensor cores
// (tcgen05.mma kind::f16, BF16 operands from shared memory, FP32
// accumulators in TMEM).  Same contract as k_mlp_eval (fb_mlp_eval.cu):
// per triplet of the list, the Legendre-combined values of getMEs_Fdata_3c
// (e.FDATA/M_Fdata_3c.f90:293-517) and, with tangents, their cos / x / y
// derivatives (getDMEs_Fdata_3c, :549-846).
//
// A CTA works on tiles of 128 triplets, two or four threads per triplet:
// they own row t of every operand and TMEM lane t of every accumulator and
// split the columns, so the epilogue of a layer (bias, SiLU, the tangents'
// silu'(z) factor, BF16 conversion into the next layer's operand) needs no
// data exchange; only the final Legendre sums are added across them.  The
// three tangents d/dx, d/dy, d/dcos are three more 128-row operands of the
// same products; their layer-1 pre-activations are columns of W1 times the
// input derivative and need no product.  One thread issues the MMAs of a
// layer and commits them to an mbarrier the CTA waits on (bounded).
#include "fb_common_df.cuh"
#include "fb_mlp.h"
#include "fb_mma.cuh"
#include "fb_tc.cuh"

namespace fb {

namespace {

// shared-memory plan (bytes): the network's weights, the input rows, the
// hidden operands, biases and W1's coordinate columns, per-row set-up, the
// mbarrier and the TMEM address slot.  With tangents the input tile shares
// the bytes of the last tangent operand (read by layer 1's product, then
// written by layer 1's epilogue).
template <int NTAN, int TILES, int SPLIT_ = 2>
struct TcShape {
  static constexpr int MT = 1 + NTAN;  // operands per tile: primal + tangents
  static constexpr int SPLIT = SPLIT_; // threads per triplet row (column parts)
  static constexpr int w1 = 0;
  static constexpr int w2 = w1 + MLP_H * MLP_IN * 2;
  static constexpr int w3 = w2 + MLP_H * MLP_H * 2;
  static constexpr int w4 = w3 + MLP_H * MLP_H * 2;
  static constexpr int h = w4 + MLP_OUT * MLP_H * 2;
  static constexpr int hsize = TILES * MT * 128 * MLP_H * 2;
  static constexpr int x = NTAN ? h + (MT - 1) * 128 * MLP_H * 2 : h + hsize;
  static constexpr int consts = NTAN ? h + hsize : x + TILES * 128 * MLP_IN * 2;
  static constexpr int nconst = 3 * MLP_H + MLP_OUT + 3 * MLP_H;  // b1 b2 b3 b4, W1 columns 0..2
  static constexpr int rinfo = consts + nconst * 4;
  static constexpr int bar = rinfo + TILES * 128 * 16;  // mbarrier, TMEM slot, tangents' mbarrier
  static constexpr int smem = bar + 24;
  static constexpr int threads = 128 * TILES * SPLIT;
  static constexpr int cols = TILES * MT * 128;  // TMEM columns (a power of 2)
};
constexpr int TAN_SPLIT = 4, VAL_SPLIT = 2;
static_assert(TcShape<3, 1, TAN_SPLIT>::smem <= 232448, "tangent plan exceeds 227 KB of shared memory");
static_assert(TcShape<0, 2, VAL_SPLIT>::smem <= 232448, "value plan exceeds 227 KB of shared memory");
static_assert(TcShape<3, 1, TAN_SPLIT>::cols == 512 && TcShape<0, 2, VAL_SPLIT>::cols == 256, "TMEM columns");
// the partial Legendre sums of parts 1.. go to the start of the hidden operands
static_assert((TAN_SPLIT - 1) * 128 * 4 * MLP_ME * 4 <= (TcShape<3, 1, TAN_SPLIT>::x - TcShape<3, 1, TAN_SPLIT>::h),
              "tangent exchange overlaps the input tile");
static_assert((VAL_SPLIT - 1) * 2 * 128 * 4 * MLP_ME * 4 <= TcShape<0, 2, VAL_SPLIT>::hsize, "value exchange");

constexpr long long TC_WAIT_LIMIT = 1LL << 22;  // mbarrier polls before the kernel gives up

// 8 consecutive K values of one row of a canonical operand: one 16-byte store
__device__ __forceinline__ void st_row8(__nv_bfloat16 *tile, int row, int k0, int K, const float v[8]) {
  uint4 u;
  u.x = pack_bf16(v[0], v[1]);
  u.y = pack_bf16(v[2], v[3]);
  u.z = pack_bf16(v[4], v[5]);
  u.w = pack_bf16(v[6], v[7]);
  *reinterpret_cast<uint4 *>(tile + canon_off(row, k0, K)) = u;
}

}  // namespace

template <int NTAN, int TILES, int SPLIT>
__global__ void __launch_bounds__(TcShape<NTAN, TILES, SPLIT>::threads, 1)
    k_mlp_tc(MlpEvalArgs a, Ctx3c c, unsigned *status) {
  using S = TcShape<NTAN, TILES, SPLIT>;
  constexpr int MT = S::MT, HALF = MLP_H / SPLIT, OPART = MLP_OUT / SPLIT;
  extern __shared__ __align__(1024) unsigned char smem[];
  __nv_bfloat16 *W1s = reinterpret_cast<__nv_bfloat16 *>(smem + S::w1);
  __nv_bfloat16 *W2s = reinterpret_cast<__nv_bfloat16 *>(smem + S::w2);
  __nv_bfloat16 *W3s = reinterpret_cast<__nv_bfloat16 *>(smem + S::w3);
  __nv_bfloat16 *W4s = reinterpret_cast<__nv_bfloat16 *>(smem + S::w4);
  __nv_bfloat16 *Xs = reinterpret_cast<__nv_bfloat16 *>(smem + S::x);
  __nv_bfloat16 *Hs = reinterpret_cast<__nv_bfloat16 *>(smem + S::h);
  float *cst = reinterpret_cast<float *>(smem + S::consts);
  float *rinfo = reinterpret_cast<float *>(smem + S::rinfo);  // [TILES * 128][4]: triple, cos, 2/xmax, 2/ymax
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + S::bar);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + S::bar + 8);
  // with tangents, the primal products commit to `bar` and the tangents'
  // to `bart`, so that each half's epilogue overlaps the other's products
  uint64_t *bart = reinterpret_cast<uint64_t *>(smem + S::bar + 16);
  const float *b1 = cst, *b2 = cst + MLP_H, *b3 = cst + 2 * MLP_H, *b4 = cst + 3 * MLP_H;
  const float *w1c = cst + 3 * MLP_H + MLP_OUT;  // [3][128]
  const int tid = threadIdx.x, warp = tid >> 5;
  // thread -> (tile, column part, row): warps w and w + 4 of a tile read the
  // same TMEM lane quarter (w % 4) and split the columns
  const int grp = tid >> 7, row = tid & 127;
  const int tt = grp / S::SPLIT, part = grp % S::SPLIT;

  const __nv_bfloat16 *gw = a.wbf;
  for (int i = tid; i < MLP_H * MLP_IN; i += S::threads) W1s[canon_off(i / MLP_IN, i % MLP_IN, MLP_IN)] = gw[i];
  gw += MLP_H * MLP_IN;
  for (int i = tid; i < MLP_H * MLP_H; i += S::threads) W2s[canon_off(i / MLP_H, i % MLP_H, MLP_H)] = gw[i];
  gw += MLP_H * MLP_H;
  for (int i = tid; i < MLP_H * MLP_H; i += S::threads) W3s[canon_off(i / MLP_H, i % MLP_H, MLP_H)] = gw[i];
  gw += MLP_H * MLP_H;
  for (int i = tid; i < MLP_OUT * MLP_H; i += S::threads) W4s[canon_off(i / MLP_H, i % MLP_H, MLP_H)] = gw[i];
  for (int i = tid; i < MLP_H; i += S::threads) {
    cst[i] = a.params[a.o_b1 + i];
    cst[MLP_H + i] = a.params[a.o_b2 + i];
    cst[2 * MLP_H + i] = a.params[a.o_b3 + i];
#pragma unroll
    for (int q = 0; q < 3; q++) cst[3 * MLP_H + MLP_OUT + q * MLP_H + i] = __bfloat162float(a.wbf[i * MLP_IN + q]);
  }
  for (int i = tid; i < MLP_OUT; i += S::threads) cst[3 * MLP_H + i] = a.params[a.o_b4 + i];
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bart, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tslot, S::cols);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = static_cast<uint32_t>((warp & 3) * 32) << 16;
  const FdataDev &fd = *c.fd;
  constexpr uint32_t ID128 = umma_idesc_bf16(128, MLP_H), ID64 = umma_idesc_bf16(128, MLP_OUT);
  uint32_t phase = 0, phaset = 0;
  bool ok = true, pend = false, pendt = false;  // commits not yet waited for
  const int ntiles = (a.n + 127) / 128;
  float *ri = rinfo + 4 * (tt * 128 + row);

  for (int t0 = blockIdx.x * TILES; t0 < ntiles; t0 += gridDim.x * TILES) {
    const int i = (t0 + tt) * 128 + row;
    const bool valid = i < a.n;
    // ---- inputs (part 0 of each row): coordinates as BF16 hi/lo pairs, embedding
    if (part == 0) {
      float f[3] = {0.0f, 0.0f, 0.0f}, sx = 0.0f, sy = 0.0f;
      int tr = 0;
      if (valid && a.pts) {
        tr = a.ptrip[i];
        const Cell3cDev &cell = fd.c3[tr / (a.nsp * a.nsp)][(tr / a.nsp) % a.nsp][tr % a.nsp];
        sx = (float)(2.0 / cell.xmax);
        sy = (float)(2.0 / cell.ymax);
        f[0] = (float)(a.pts[3 * i] * (2.0 / cell.xmax) - 1.0);
        f[1] = (float)(a.pts[3 * i + 1] * (2.0 / cell.ymax) - 1.0);
        f[2] = a.pts[3 * i + 2];
      } else if (valid) {
        GeomFP64 h;
        trip_geom_fp64(c, a.list[i], h);
        int ka = c.isp[h.iat], kb = c.isp[h.jat], kc = c.isp[h.ia];
        const Cell3cDev &cell = fd.c3[ka][kb][kc];
        tr = (ka * a.nsp + kb) * a.nsp + kc;
        sx = (float)(2.0 / cell.xmax);
        sy = (float)(2.0 / cell.ymax);
        f[0] = (float)(h.x * (2.0 / cell.xmax) - 1.0);
        f[1] = (float)(h.z * (2.0 / cell.ymax) - 1.0);
        f[2] = trip_cost_df(h).h;
      }
      __nv_bfloat16 *X = Xs + tt * 128 * MLP_IN;
      const float *em = a.params + a.o_emb + tr * MLP_EMB;
#pragma unroll
      for (int k0 = 0; k0 < MLP_IN; k0 += 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int k = k0 + j;
          float x = 0.0f;
          if (k < 3) x = f[k];
          else if (k < 3 + MLP_EMB) x = em[k - 3];
          else if (k < MLP_LO + 3) x = f[k - MLP_LO] - __bfloat162float(__float2bfloat16_rn(f[k - MLP_LO]));
          v[j] = x;
        }
        st_row8(X, row, k0, MLP_IN, v);
      }
      ri[0] = __int_as_float(tr);
      ri[1] = f[2];
      ri[2] = sx;
      ri[3] = sy;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- layer 1 (K = 32): primal only --------------------------------------
    if (tid == 0) {
      for (int q = 0; q < TILES; q++) {
        uint32_t xa = smem_u32(Xs + q * 128 * MLP_IN), wb = smem_u32(W1s);
        for (int ks = 0; ks < MLP_IN / 16; ks++)
          umma_bf16(tmem + q * MT * 128, umma_desc(xa + ks * 256, 128, (MLP_IN / 8) * 128),
                    umma_desc(wb + ks * 256, 128, (MLP_IN / 8) * 128), ID128, ks > 0);
      }
      umma_commit(bar);
    }
    pend = true;
    ok = __syncthreads_and(mbar_wait(bar, phase, TC_WAIT_LIMIT) ? 1 : 0) != 0;
    if (!ok) break;
    phase ^= 1;
    pend = false;
    tc_fence_after();
    const float sx = ri[2], sy = ri[3];
    __nv_bfloat16 *H = Hs + tt * MT * 128 * MLP_H;
    const uint32_t dbase = tmem + lane_base + tt * MT * 128;
#pragma unroll 1
    for (int c0 = part * HALF; c0 < (part + 1) * HALF; c0 += 16) {
      float z[16];
      tmem_ld16(dbase + c0, z);
#pragma unroll
      for (int hh = 0; hh < 2; hh++) {
        float hv[8], t1[8], t2[8], t3[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int n = c0 + 8 * hh + j;
          float zz = z[8 * hh + j] + b1[n];
          float sg = sigmoid_fast(zz);
          hv[j] = zz * sg;
          if (NTAN) {
            float ds = sg * (1.0f + zz * (1.0f - sg));
            t1[j] = ds * w1c[n] * sx;
            t2[j] = ds * w1c[MLP_H + n] * sy;
            t3[j] = ds * w1c[2 * MLP_H + n];
          }
        }
        st_row8(H, row, c0 + 8 * hh, MLP_H, hv);
        if (NTAN) {
          st_row8(H + 1 * 128 * MLP_H, row, c0 + 8 * hh, MLP_H, t1);
          st_row8(H + 2 * 128 * MLP_H, row, c0 + 8 * hh, MLP_H, t2);
          st_row8(H + 3 * 128 * MLP_H, row, c0 + 8 * hh, MLP_H, t3);
        }
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // MMAs of one layer for operands [op0, op1) of every tile into their
    // accumulators (the output layer: N = 64, accumulators 64 columns apart)
    auto issue = [&](const __nv_bfloat16 *W, int op0, int op1, bool out_layer) {
      uint32_t wb = smem_u32(W);
      for (int q = 0; q < TILES; q++)
        for (int op = op0; op < op1; op++) {
          uint32_t ha = smem_u32(Hs + (q * MT + op) * 128 * MLP_H);
          uint32_t d = tmem + (q * MT + op) * (out_layer ? MLP_OUT : 128);
          for (int ks = 0; ks < MLP_H / 16; ks++)
            umma_bf16(d, umma_desc(ha + ks * 256, 128, (MLP_H / 8) * 128),
                      umma_desc(wb + ks * 256, 128, (MLP_H / 8) * 128), out_layer ? ID64 : ID128, ks > 0);
        }
    };
    if constexpr (NTAN == 0) {
      // ---- layers 2 and 3 (K = N = 128) ----------------------------------------
#pragma unroll 1
      for (int l = 0; l < 2; l++) {
        const __nv_bfloat16 *W = l == 0 ? W2s : W3s;
        const float *bl = l == 0 ? b2 : b3;
        if (tid == 0) {
          uint32_t wb = smem_u32(W);
          for (int q = 0; q < TILES; q++)
            for (int op = 0; op < MT; op++) {
              uint32_t ha = smem_u32(Hs + (q * MT + op) * 128 * MLP_H);
              for (int ks = 0; ks < MLP_H / 16; ks++)
                umma_bf16(tmem + (q * MT + op) * 128, umma_desc(ha + ks * 256, 128, (MLP_H / 8) * 128),
                          umma_desc(wb + ks * 256, 128, (MLP_H / 8) * 128), ID128, ks > 0);
            }
          umma_commit(bar);
        }
        pend = true;
        ok = __syncthreads_and(mbar_wait(bar, phase, TC_WAIT_LIMIT) ? 1 : 0) != 0;
        if (!ok) break;
        phase ^= 1;
        pend = false;
        tc_fence_after();
#pragma unroll 1
        for (int c0 = part * HALF; c0 < (part + 1) * HALF; c0 += 16) {
          float z[16], ds[16];
          tmem_ld16(dbase + c0, z);
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            float hv[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
              float zz = z[8 * hh + j] + bl[c0 + 8 * hh + j];
              float sg = sigmoid_fast(zz);
              hv[j] = zz * sg;
              ds[8 * hh + j] = sg * (1.0f + zz * (1.0f - sg));
            }
            st_row8(H, row, c0 + 8 * hh, MLP_H, hv);
          }
#pragma unroll
          for (int op = 1; op < MT; op++) {
            float dz[16];
            tmem_ld16(dbase + op * 128 + c0, dz);
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
              float tv[8];
#pragma unroll
              for (int j = 0; j < 8; j++) tv[j] = ds[8 * hh + j] * dz[8 * hh + j];
              st_row8(H + op * 128 * MLP_H, row, c0 + 8 * hh, MLP_H, tv);
            }
          }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
      }
      if (!ok) break;
      // ---- layer 4 (N = 64, 50 used) --------------------------------------------
      if (tid == 0) {
        uint32_t wb = smem_u32(W4s);
        for (int q = 0; q < TILES; q++)
          for (int op = 0; op < MT; op++) {
            uint32_t ha = smem_u32(Hs + (q * MT + op) * 128 * MLP_H);
            for (int ks = 0; ks < MLP_H / 16; ks++)
              umma_bf16(tmem + (q * MT + op) * MLP_OUT, umma_desc(ha + ks * 256, 128, (MLP_H / 8) * 128),
                        umma_desc(wb + ks * 256, 128, (MLP_H / 8) * 128), ID64, ks > 0);
          }
        umma_commit(bar);
      }
      pend = true;
      ok = __syncthreads_and(mbar_wait(bar, phase, TC_WAIT_LIMIT) ? 1 : 0) != 0;
      if (!ok) break;
      phase ^= 1;
      pend = false;
    } else {
      // Layers 2 and 3 with tangents, pipelined: the primal products commit
      // to `bar`, the tangent products to `bart`.  The primal epilogue
      // (SiLU and silu') runs while the tangent products of its layer run;
      // the next layer's primal product (it reads only the primal operand
      // and writes only the primal accumulator) is issued as soon as the
      // primal operand is written, and runs while the tangent epilogue reads
      // the tangent accumulators.  TMEM: layer l's accumulators at columns
      // op * 128; the output layer's at op * 64, its primal (columns 0..63)
      // issued during layer 3's tangent epilogue (columns 128..511), its
      // tangents (64..255) only after it.
      if (tid == 0) {
        issue(W2s, 0, 1, false);
        umma_commit(bar);
        issue(W2s, 1, MT, false);
        umma_commit(bart);
      }
      pend = pendt = true;
#pragma unroll 1
      for (int l = 0; l < 2; l++) {
        const float *bl = l == 0 ? b2 : b3;
        ok = __syncthreads_and(mbar_wait(bar, phase, TC_WAIT_LIMIT) ? 1 : 0) != 0;
        if (!ok) break;
        phase ^= 1;
        pend = false;
        tc_fence_after();
        float ds[HALF];  // silu'(z) of this thread's columns
#pragma unroll
        for (int cc = 0; cc < HALF / 16; cc++) {
          const int c0 = part * HALF + 16 * cc;
          float z[16];
          tmem_ld16(dbase + c0, z);
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            float hv[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
              float zz = z[8 * hh + j] + bl[c0 + 8 * hh + j];
              float sg = sigmoid_fast(zz);
              hv[j] = zz * sg;
              ds[16 * cc + 8 * hh + j] = sg * (1.0f + zz * (1.0f - sg));
            }
            st_row8(H, row, c0 + 8 * hh, MLP_H, hv);
          }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
          issue(l == 0 ? W3s : W4s, 0, 1, l == 1);
          umma_commit(bar);
        }
        pend = true;
        ok = __syncthreads_and(mbar_wait(bart, phaset, TC_WAIT_LIMIT) ? 1 : 0) != 0;
        if (!ok) break;
        phaset ^= 1;
        pendt = false;
        tc_fence_after();
#pragma unroll
        for (int cc = 0; cc < HALF / 16; cc++) {
          const int c0 = part * HALF + 16 * cc;
#pragma unroll
          for (int op = 1; op < MT; op++) {
            float dz[16];
            tmem_ld16(dbase + op * 128 + c0, dz);
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
              float tv[8];
#pragma unroll
              for (int j = 0; j < 8; j++) tv[j] = ds[16 * cc + 8 * hh + j] * dz[8 * hh + j];
              st_row8(H + op * 128 * MLP_H, row, c0 + 8 * hh, MLP_H, tv);
            }
          }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
          issue(l == 0 ? W3s : W4s, 1, MT, l == 1);
          umma_commit(bart);
        }
        pendt = true;
      }
      if (!ok) break;
      // the output layer's products, both halves
      bool w = mbar_wait(bar, phase, TC_WAIT_LIMIT);
      if (w) {
        phase ^= 1;
        pend = false;
        w = mbar_wait(bart, phaset, TC_WAIT_LIMIT);
        if (w) {
          phaset ^= 1;
          pendt = false;
        }
      }
      ok = __syncthreads_and(w ? 1 : 0) != 0;
      if (!ok) break;
    }
    tc_fence_after();
    // ---- Legendre combination: each part sums its share of the output
    // columns, parts 1.. hand their partial sums to part 0 ------------------
    {
      const int tr = __float_as_int(ri[0]);
      const float cth = ri[1], c2 = cth * cth;
      float pl[5] = {1.0f, cth, 0.5f * (3.0f * c2 - 1.0f), 0.5f * cth * (5.0f * c2 - 3.0f),
                     0.125f * (3.0f - c2 * (30.0f - 35.0f * c2))};
      float dpl[5] = {0.0f, 1.0f, 3.0f * cth, (15.0f * c2 - 3.0f) * 0.5f, 0.5f * cth * (35.0f * c2 - 15.0f)};
      const float *sc = a.scale + tr * MLP_OUT;
      float acc[4][MLP_ME];
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int e = 0; e < MLP_ME; e++) acc[q][e] = 0.0f;
      const uint32_t obase = tmem + lane_base + tt * MT * MLP_OUT;
#pragma unroll
      for (int op = 0; op < MT; op++) {
#pragma unroll
        for (int cc = 0; cc < OPART / 16; cc++) {
          const int c0 = part * OPART + 16 * cc;
          float v[16];
          tmem_ld16(obase + op * MLP_OUT + c0, v);
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const int o = c0 + j;
            if (o < NTHETA * MLP_ME) {
              const int th = o / MLP_ME, e = o % MLP_ME;
              float val = (op == 0 ? v[j] + b4[o] : v[j]) * sc[o];
              if (op == 0) {
                acc[0][e] = fmaf(pl[th], val, acc[0][e]);
                acc[1][e] = fmaf(dpl[th], val, acc[1][e]);
              } else if (op == 1) {
                acc[2][e] = fmaf(pl[th], val, acc[2][e]);
              } else if (op == 2) {
                acc[3][e] = fmaf(pl[th], val, acc[3][e]);
              } else {
                acc[1][e] = fmaf(pl[th], val, acc[1][e]);
              }
            }
          }
        }
      }
      constexpr int NQ = NTAN ? 4 : 1;
      // the hidden operands are free now: they carry the partial sums
      float *xch = reinterpret_cast<float *>(Hs);
      auto slot = [&](int p) { return xch + (((p - 1) * TILES + tt) * 128 + row) * 4 * MLP_ME; };
      if (part > 0) {
        float *d = slot(part);
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
          for (int e = 0; e < MLP_ME; e++) d[q * MLP_ME + e] = acc[q][e];
      }
      __syncthreads();
      if (part == 0 && valid) {
        for (int p = 1; p < SPLIT; p++) {
          const float *d = slot(p);
#pragma unroll
          for (int q = 0; q < NQ; q++)
#pragma unroll
            for (int e = 0; e < MLP_ME; e++) acc[q][e] += d[q * MLP_ME + e];
        }
        float *dst = a.out + (long long)i * NQ * MLP_ME;
#pragma unroll
        for (int q = 0; q < NQ; q++)
#pragma unroll
          for (int e = 0; e < MLP_ME; e++) dst[q * MLP_ME + e] = acc[q][e];
      }
    }
    // the next tile's MMAs and inputs overwrite accumulators and operands: all reads done first
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  if (!ok) {
    // a product never completed: report it, give it one more bounded wait, release TMEM
    if (tid == 0) atomicOr(status, DEVERR_WATCHDOG);
    if (pend) mbar_wait(bar, phase, TC_WAIT_LIMIT);
    if (pendt) mbar_wait(bart, phaset, TC_WAIT_LIMIT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, S::cols);
}

// The network's inputs per list position, ahead of the tensor-core kernel:
// (x, y, cos theta) of the triplet in float and its species triple.  The
// inputs enter the network as BF16 hi/lo pairs (16 bits), so float geometry
// from the float copies of the positions is exact enough, and a thread per
// triplet at full occupancy takes the position gathers off the
// one-CTA-per-SM tensor-core kernel (where they were its leading stall).
// The tails recompute the geometry exactly (fb_dasm3c_df.cu, fb_asm3c_df.cu).
__global__ void k_mlp_points(int n, const int *__restrict__ list, const int *__restrict__ talpha,
                             const int *__restrict__ ci_j, const int *__restrict__ ci_b,
                             const int *__restrict__ cj_j, const int *__restrict__ cj_b, const int *__restrict__ sid,
                             const int *__restrict__ isp, int nsp, const float4 *__restrict__ pos4,
                             const float *__restrict__ xlf0, float *__restrict__ pts, int *__restrict__ ptrip) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int t = list[i];
  int ia = talpha[t], iat = ci_j[t], jat = cj_j[t], ib = ci_b[t], jb = cj_b[t];
  const float *xl = xlf0 + (long long)sid[ia] * XL_STRIDE;
  float4 p1 = pos4[iat], p2 = pos4[jat], pa = pos4[ia];
  float r1[3] = {p1.x + xl[3 * ib], p1.y + xl[3 * ib + 1], p1.z + xl[3 * ib + 2]};
  float r2[3] = {p2.x + xl[3 * jb], p2.y + xl[3 * jb + 1], p2.z + xl[3 * jb + 2]};
  float rn[3] = {pa.x, pa.y, pa.z};
  float r21[3], rc[3], z2 = 0.0f, x2 = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r21[k] = r2[k] - r1[k];
    rc[k] = rn[k] - (r1[k] + 0.5f * r21[k]);
    z2 += r21[k] * r21[k];
    x2 += rc[k] * rc[k];
  }
  float z = sqrtf(z2), x = sqrtf(x2);
  float cost = 0.0f;
  if (x > 1.0e-5f) {
    if (z < 1.0e-5f) cost = rc[2] / x;  // sighat = (0, 0, 1)
    else cost = (r21[0] * rc[0] + r21[1] * rc[1] + r21[2] * rc[2]) / (z * x);
  }
  pts[3 * i] = x;
  pts[3 * i + 1] = z;
  pts[3 * i + 2] = cost;
  ptrip[i] = (isp[iat] * nsp + isp[jat]) * nsp + isp[ia];
}

int launch_mlp_points(const MlpEvalArgs &m, const AsmArgs &a, const float4 *pos4, const float *xlf, float *pts,
                      int *ptrip, cudaStream_t s) {
  if (m.n == 0) return 0;
  int threads = 256;
  k_mlp_points<<<(m.n + threads - 1) / threads, threads, 0, s>>>(m.n, m.list, a.trip_alpha, a.ci_j, a.ci_b, a.cj_j,
                                                                  a.cj_b, a.sid, a.isp, m.nsp, pos4, xlf, pts,
                                                                  ptrip);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_mlp_tc(const MlpEvalArgs &m, const AsmArgs &a, bool tangents, int nsm, cudaStream_t s) {
  if (m.n == 0) return 0;
  Ctx3c c = make3c(a);
  int ntiles = (m.n + 127) / 128;
  if (tangents) {
    using S = TcShape<3, 1, TAN_SPLIT>;
    cudaError_t e =
        cudaFuncSetAttribute(k_mlp_tc<3, 1, TAN_SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem);
    if (e != cudaSuccess) return (int)e;
    int blocks = ntiles < nsm ? ntiles : nsm;
    k_mlp_tc<3, 1, TAN_SPLIT><<<blocks, S::threads, S::smem, s>>>(m, c, a.status);
  } else {
    using S = TcShape<0, 2, VAL_SPLIT>;
    cudaError_t e =
        cudaFuncSetAttribute(k_mlp_tc<0, 2, VAL_SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::smem);
    if (e != cudaSuccess) return (int)e;
    int blocks = (ntiles + 1) / 2 < nsm ? (ntiles + 1) / 2 : nsm;
    k_mlp_tc<0, 2, VAL_SPLIT><<<blocks, S::threads, S::smem, s>>>(m, c, a.status);
  }
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
