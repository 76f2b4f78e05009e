// fb_pp.cu -- sm_103a kernels of the non-local pseudopotential (vnl) path.
//
// Neighbor maps (c.SYSTEM/M_neighbors_PP.f90): PP pairs (basis of i within
// reach of the projectors of j: |r| < rcA_i + rc_PP_j - 0.01), PPx pairs
// (projectors of i, basis of j), PPp pairs (two basis atoms sharing a
// projector atom, first occurrences in the reference's loop order), the
// maps of PP and PPx pairs into PPp and the PPx points into PP(j), and the
// PP common-neighbor triplets (alpha, i, j) with their svnl indices.
//
// Blocks: svnl(i, j) = <basis i | projectors j>, norb_i x norb_PP_j per PP
// pair (rotate_PP frame); vnl(i, k) = sum over projector atoms m of
// svnl(i, m) cl_m svnl(k, m)^T, norb_i x norb_k per PPp pair, split as the
// reference splits it into atom, ontop-left, ontop-right (2c) and three-center
// terms.  All in FP64: the path is a few small contractions per pair and
// triplet and is bound by memory and atomics, not arithmetic.
#include "fb_common.cuh"
#include "fb_pp.h"

namespace fb {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// PP / PPx pairs (find_neighbors_PP :409-516, find_neighbors_PPx :672-778):
// one warp per atom, images in increasing mbeta, lanes over the atoms of the
// structure, so hits come out mbeta outer, jatom inner.  kind 0: PP (rcA_i +
// rc_PP_j), kind 1: PPx (rc_PP_i + rcA_j).
template <bool FILL>
__global__ void k_pp_pairs(PPArgs a, int kind) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp, s = a.sid[i];
  int a0 = a.satom_off[s], a1 = a.satom_off[s + 1];
  const double *X = a.xl + (long long)s * XL_STRIDE;
  const float *Xf = a.xlf + (long long)s * XL_STRIDE;
  float4 lo = a.sbbox[2 * s], hi = a.sbbox[2 * s + 1];
  double ri[3] = {a.ratom[3 * i], a.ratom[3 * i + 1], a.ratom[3 * i + 2]};
  float4 pi = a.pos4[i];
  const SpeciesDev &si = a.fd->sp[a.isp[i]];
  double rci = kind == 0 ? si.rcA : si.rc_pp;
  float reach = a.reach + 1.0e-2f;
  int *J = kind == 0 ? a.pp_j : a.ppx_j;
  int *B = kind == 0 ? a.pp_b : a.ppx_b;
  int *self = kind == 0 ? a.pp_self : a.ppx_self;
  int base = FILL ? (kind == 0 ? a.pp_off[i] : a.ppx_off[i]) : 0;
  long long bbase = (FILL && kind == 0) ? a.svnl_base[i] : 0;
  int ni = si.norb, num = 0;
  long long nsum = 0;
  for (int ii = a.simg_off[s]; ii < a.simg_off[s + 1]; ii++) {
    int mb = a.imgs[ii];
    float L0 = Xf[3 * mb], L1 = Xf[3 * mb + 1], L2 = Xf[3 * mb + 2];
    float ox = fmaxf(fmaxf(lo.x + L0 - pi.x, pi.x - (hi.x + L0)), 0.0f);
    float oy = fmaxf(fmaxf(lo.y + L1 - pi.y, pi.y - (hi.y + L1)), 0.0f);
    float oz = fmaxf(fmaxf(lo.z + L2 - pi.z, pi.z - (hi.z + L2)), 0.0f);
    if (ox * ox + oy * oy + oz * oz > reach * reach) continue;
    double X0 = X[3 * mb], X1 = X[3 * mb + 1], X2 = X[3 * mb + 2];
    for (int j0 = a0; j0 < a1; j0 += 32) {
      int j = j0 + lane;
      bool hit = false;
      if (j < a1) {
        const SpeciesDev &sj = a.fd->sp[a.isp[j]];
        double rcj = kind == 0 ? sj.rc_pp : sj.rcA;
        float4 pj = a.pos4[j];
        float d0 = (pj.x + L0) - pi.x, d1 = (pj.y + L1) - pi.y, d2 = (pj.z + L2) - pi.z;
        float lim = (float)(rci + rcj) + 1.0e-2f;
        if (d0 * d0 + d1 * d1 + d2 * d2 < lim * lim) {
          double range = __dsub_rn(__dadd_rn(rci, rcj), 0.01);
          double r2[3] = {__dadd_rn(a.ratom[3 * j], X0), __dadd_rn(a.ratom[3 * j + 1], X1),
                          __dadd_rn(a.ratom[3 * j + 2], X2)};
          hit = dist_rn(ri, r2) < range;
        }
      }
      unsigned m = __ballot_sync(FULL, hit);
      if (m == 0u) continue;
      int nj = (hit && kind == 0) ? a.fd->sp[a.isp[j]].norb_pp : 0;
      int incl = nj;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        int u = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += u;
      }
      if (FILL && hit) {
        int idx = num + __popc(m & lanemask_lt(lane));
        J[base + idx] = j;
        B[base + idx] = mb;
        if (kind == 0) a.svnl_off[base + idx] = bbase + (long long)ni * (nsum + incl - nj);
        if (j == i && mb == 0) self[i] = idx;
      }
      num += __popc(m);
      nsum += __shfl_sync(FULL, incl, 31);
    }
  }
  if (!FILL && lane == 0) {
    if (kind == 0) {
      a.pp_cnt[i] = num;
      a.svnl_sum[i] = (long long)ni * nsum;
    } else {
      a.ppx_cnt[i] = num;
    }
  }
  if (FILL) {
    __syncwarp();
    if (lane == 0 && self[i] < 0) atomicOr(a.status, DEVERR_SELF);
  }
}

// upper bound of the PPp candidates of atom i: sum over its PP neighbors
// alpha of |PPx(alpha)|
__global__ void k_ppp_bounds(PPArgs a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.N) return;
  int u = 0;
  for (int p = a.pp_off[i]; p < a.pp_off[i + 1]; p++) {
    int al = a.pp_j[p];
    u += a.ppx_off[al + 1] - a.ppx_off[al];
  }
  a.ub[i] = u;
}

// find_neighbors_PPp (:922-980): for each PP neighbor (alpha, ibeta) of i,
// each PPx neighbor (j, jbeta) of alpha, the image of xl(jbeta) + xl(ibeta);
// (j, mbeta) is appended unless already listed.  One warp per atom; the
// candidates of a chunk are tested against the list so far and against the
// earlier lanes of the chunk, so the list holds first occurrences in the
// reference's order.  The image of the sum is the sum of the integer cell
// shifts (an image outside the 9 x 9 x 9 box is an error, as it has no xl).
__global__ void k_ppp(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  long long sb = a.slot_off[i];
  int n = 0;
  long long nsum = 0;
  for (int p = a.pp_off[i]; p < a.pp_off[i + 1]; p++) {
    int al = a.pp_j[p], ib = a.pp_b[p];
    int ibx, iby, ibz;
    mbeta_shift(ib, ibx, iby, ibz);
    for (int q0 = a.ppx_off[al]; q0 < a.ppx_off[al + 1]; q0 += 32) {
      int q = q0 + lane;
      bool valid = q < a.ppx_off[al + 1];
      int j = -1, mb = -1;
      if (valid) {
        j = a.ppx_j[q];
        int jbx, jby, jbz;
        mbeta_shift(a.ppx_b[q], jbx, jby, jbz);
        int sx = ibx + jbx, sy = iby + jby, sz = ibz + jbz;
        if (sx < -4 || sx > 4 || sy < -4 || sy > 4 || sz < -4 || sz > 4) {
          atomicOr(a.status, DEVERR_CAP);
          a.errinfo[0] = i;
          a.errinfo[1] = j;
          valid = false;
        } else {
          mb = shift_mbeta(sx, sy, sz);
        }
      }
      bool dup = false;
      if (valid)
        for (int k = 0; k < n; k++)
          if (a.slot_j[sb + k] == j && a.slot_b[sb + k] == mb) {
            dup = true;
            break;
          }
      unsigned long long key = valid ? (unsigned long long)j * NIMG + (unsigned long long)mb : ~0ull;
      unsigned same = __match_any_sync(FULL, key);
      bool add = valid && !dup && (__ffs(same) - 1) == lane;
      unsigned m = __ballot_sync(FULL, add);
      if (add) {
        int idx = n + __popc(m & lanemask_lt(lane));
        a.slot_j[sb + idx] = j;
        a.slot_b[sb + idx] = mb;
      }
      int nj = add ? a.fd->sp[a.isp[j]].norb : 0;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) nj += __shfl_xor_sync(FULL, nj, d);
      nsum += nj;
      n += __popc(m);
      __syncwarp();
    }
  }
  if (lane == 0) {
    a.ppp_cnt[i] = n;
    a.vnl_sum[i] = (long long)a.fd->sp[a.isp[i]].norb * nsum;
  }
}

// the PPp slots into CSR with the vnl block offsets and the self index
__global__ void k_ppp_compact(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  long long sb = a.slot_off[i], vb = a.vnl_base[i];
  int base = a.ppp_off[i], n = a.ppp_off[i + 1] - base;
  int ni = a.fd->sp[a.isp[i]].norb;
  long long nsum = 0;
  for (int k0 = 0; k0 < n; k0 += 32) {
    int k = k0 + lane;
    bool valid = k < n;
    int j = valid ? a.slot_j[sb + k] : 0, mb = valid ? a.slot_b[sb + k] : 0;
    int nj = valid ? a.fd->sp[a.isp[j]].norb : 0;
    int incl = nj;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int u = __shfl_up_sync(FULL, incl, d);
      if (lane >= d) incl += u;
    }
    if (valid) {
      a.ppp_j[base + k] = j;
      a.ppp_b[base + k] = mb;
      a.vnl_off[base + k] = vb + (long long)ni * (nsum + incl - nj);
      if (j == i && mb == 0) a.ppp_self[i] = k;
    }
    nsum += __shfl_sync(FULL, incl, 31);
  }
  __syncwarp();
  if (lane == 0 && a.ppp_self[i] < 0) atomicOr(a.status, DEVERR_SELF);
}

// maps of the PP and PPx pairs into PPp (:1030-1057) and the PPx points
// into PP(j) (:1060-1080): first (katom, kbeta) of i's PPp list equal to the
// pair; the point is the first PP neighbor k of j with
// |ratom(katom) + xl(kbeta) + xl(jbeta) - ratom(i)| < 1e-4.  Warp per atom.
__global__ void k_pp_maps(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  const double *X = a.xl + (long long)a.sid[i] * XL_STRIDE;
  int k0 = a.ppp_off[i], k1 = a.ppp_off[i + 1];
  for (int w = 0; w < 2; w++) {
    const int *off = w ? a.ppx_off : a.pp_off;
    const int *J = w ? a.ppx_j : a.pp_j;
    const int *B = w ? a.ppx_b : a.pp_b;
    int *map = w ? a.ppx_map : a.pp_map;
    for (int p = off[i] + lane; p < off[i + 1]; p += 32) {
      int j = J[p], jb = B[p], m = -1;
      for (int k = k0; k < k1; k++)
        if (a.ppp_j[k] == j && a.ppp_b[k] == jb) {
          m = k - k0;
          break;
        }
      map[p] = m;
      if (m < 0) atomicOr(a.status, DEVERR_BACK);
      if (w == 1) {
        int pt = -1;
        double r1[3] = {a.ratom[3 * i], a.ratom[3 * i + 1], a.ratom[3 * i + 2]};
        for (int k = a.pp_off[j]; k < a.pp_off[j + 1]; k++) {
          int ka = a.pp_j[k], kb = a.pp_b[k];
          double r2[3];
#pragma unroll
          for (int c = 0; c < 3; c++) r2[c] = __dadd_rn(__dadd_rn(a.ratom[3 * ka + c], X[3 * kb + c]), X[3 * jb + c]);
          if (dist_rn(r1, r2) < 1.0e-04) {
            pt = k - a.pp_off[j];
            break;
          }
        }
        a.ppx_point[p] = pt;
        if (pt < 0) atomicOr(a.status, DEVERR_BACK);
      }
    }
  }
}

// the image of the cell shift (sx, sy, sz), or -1 outside the 9 x 9 x 9 box
__device__ __forceinline__ int image_of_shift(int sx, int sy, int sz) {
  if (sx < -4 || sx > 4 || sy < -4 || sy > 4 || sz < -4 || sz > 4) return -1;
  return shift_mbeta(sx, sy, sz);
}

// mpairnay (M_assemble_PP_3c.f90:266-365): the PP neighbor of atom `at` that
// is atom al at the vector r12 = r_al - r_at(image); exactly one must match.
// The entry that can match is (al, mb_hint), mb_hint the image of the
// negated shift of at's image: it is found by an integer search and then
// tested exactly; only when that fails does the reference's full count run.
__device__ __forceinline__ int mpairnay(const PPArgs &a, const double *X, int at, int al, const double *r12,
                                        int mb_hint, int &imatch) {
  if (mb_hint >= 0) {
    for (int k = a.pp_off[at]; k < a.pp_off[at + 1]; k++) {
      if (a.pp_j[k] != al || a.pp_b[k] != mb_hint) continue;
      double r21[3];
#pragma unroll
      for (int c = 0; c < 3; c++)
        r21[c] = __dsub_rn(__dadd_rn(a.ratom[3 * al + c], X[3 * mb_hint + c]), a.ratom[3 * at + c]);
      if (dist_rn(r12, r21) < 0.0001) {
        imatch = 1;
        return k - a.pp_off[at];
      }
      break;
    }
  }
  int m = -1;
  imatch = 0;
  for (int k = a.pp_off[at]; k < a.pp_off[at + 1]; k++) {
    if (a.pp_j[k] != al) continue;
    int mb = a.pp_b[k];
    double r21[3];
#pragma unroll
    for (int c = 0; c < 3; c++) r21[c] = __dsub_rn(__dadd_rn(a.ratom[3 * al + c], X[3 * mb + c]), a.ratom[3 * at + c]);
    if (dist_rn(r12, r21) < 0.0001) {
      imatch++;
      m = k - a.pp_off[at];
    }
  }
  return m;
}

// find_common_neighbors_PP (:1301-1420): for each alpha the ordered pairs
// (i, j) of its PPx neighbors, neither alpha itself, i != j as list entries;
// neigh_common = the first k of i's PPp list with |(r_j - r_i) - (xl(kbeta)
// + r_katom - r_iatom)| < 1e-4 (the pair is dropped when there is none); m31
// and m32 from mpairnay.  One warp per alpha, lanes over j.
template <bool FILL>
__global__ void k_ppc(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int al = warp;
  const double *X = a.xl + (long long)a.sid[al] * XL_STRIDE;
  int q0 = a.ppx_off[al], q1 = a.ppx_off[al + 1];
  int cnt = 0, base = FILL ? a.ppc_off[al] : 0;
  double rna[3] = {a.ratom[3 * al], a.ratom[3 * al + 1], a.ratom[3 * al + 2]};
  for (int qa = q0; qa < q1; qa++) {
    int i = a.ppx_j[qa], ib = a.ppx_b[qa];
    if (i == al && ib == 0) continue;
    double r1[3], r31[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      r1[c] = __dadd_rn(a.ratom[3 * i + c], X[3 * ib + c]);
      r31[c] = __dsub_rn(rna[c], r1[c]);
    }
    int ibx, iby, ibz;
    mbeta_shift(ib, ibx, iby, ibz);
    int im31 = 0, m31 = FILL ? mpairnay(a, X, i, al, r31, image_of_shift(-ibx, -iby, -ibz), im31) : 0;
    for (int qb0 = q0; qb0 < q1; qb0 += 32) {
      int qb = qb0 + lane;
      bool keep = false;
      int j = -1, jb = 0, m = -1, m32 = -1;
      if (qb < q1 && qb != qa) {
        j = a.ppx_j[qb];
        jb = a.ppx_b[qb];
        if (!(j == al && jb == 0)) {
          double r2[3], r[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            r2[c] = __dadd_rn(a.ratom[3 * j + c], X[3 * jb + c]);
            r[c] = __dsub_rn(r2[c], r1[c]);
          }
          // the entry that can match: (j, image of shift(jb) - shift(ib)),
          // found by an integer search and tested exactly; otherwise the
          // reference's scan (first k within 1e-4) decides
          int jbx, jby, jbz;
          mbeta_shift(jb, jbx, jby, jbz);
          int kb0 = image_of_shift(jbx - ibx, jby - iby, jbz - ibz);
          if (kb0 >= 0)
            for (int k = a.ppp_off[i]; k < a.ppp_off[i + 1]; k++) {
              if (a.ppp_j[k] != j || a.ppp_b[k] != kb0) continue;
              double r3[3];
#pragma unroll
              for (int c = 0; c < 3; c++)
                r3[c] = __dsub_rn(__dadd_rn(X[3 * kb0 + c], a.ratom[3 * j + c]), a.ratom[3 * i + c]);
              if (dist_rn(r, r3) < 1.0e-4) m = k - a.ppp_off[i];
              break;
            }
          if (m < 0)
            for (int k = a.ppp_off[i]; k < a.ppp_off[i + 1]; k++) {
              int ka = a.ppp_j[k], kb = a.ppp_b[k];
              double r3[3];
#pragma unroll
              for (int c = 0; c < 3; c++)
                r3[c] = __dsub_rn(__dadd_rn(X[3 * kb + c], a.ratom[3 * ka + c]), a.ratom[3 * i + c]);
              if (dist_rn(r, r3) < 1.0e-4) {
                m = k - a.ppp_off[i];
                break;
              }
            }
          keep = m >= 0;
          if (FILL && keep) {
            double r32[3];
#pragma unroll
            for (int c = 0; c < 3; c++) r32[c] = __dsub_rn(rna[c], r2[c]);
            int im32 = 0;
            m32 = mpairnay(a, X, j, al, r32, image_of_shift(-jbx, -jby, -jbz), im32);
            if (im32 != 1 || im31 != 1) {
              atomicOr(a.status, DEVERR_BACK);
              a.errinfo[0] = al;
              a.errinfo[1] = im31 != 1 ? i : j;
              keep = false;
            }
          }
        }
      }
      unsigned bm = __ballot_sync(FULL, keep);
      if (FILL && keep) {
        int t = base + cnt + __popc(bm & lanemask_lt(lane));
        a.t_alpha[t] = al;
        a.t_i[t] = i;
        a.t_ib[t] = ib;
        a.t_j[t] = j;
        a.t_jb[t] = jb;
        a.t_m[t] = m;
        a.t_m31[t] = m31;
        a.t_m32[t] = m32;
      }
      cnt += __popc(bm);
    }
  }
  if (!FILL && lane == 0) a.ppc_cnt[al] = cnt;
}

// ---------------------------------------------------------------------------
// svnl and its derivative (assemble_svnl, M_assemble_PP_2c.f90:86-206;
// Dassemble_svnl, M_Dassemble_PP_2c.f90:296-380)
// ---------------------------------------------------------------------------
template <int PA, int PB, bool HASD, bool DERIV>
__device__ __forceinline__ void pair_svnl(const Ctx2c &c, const PPArgs &a, int i, int p) {
  using PL = Plan<PA, PB, K2C>;
  constexpr int NA = PL::NA, NB = PL::NB, NE = PL::m.n;
  double r1[3], r2[3], z, e[3][3];
  pair_geom(c, i, p, r1, r2, z, e);
  const Cell2cDev &cell = c.fd->c2vnl[c.isp[i]][c.isp[c.neigh_j[p]]];
  long long o = a.svnl_off[p];
  RotM R;
  twister<HASD>(e, R);
  if constexpr (!DERIV) {
    if (z > cell.xmax * (1.0 + 1.0e-5)) atomicOr(c.status, DEVERR_XLARGE);
    double w[7], v[NE], X[NA * NB];
    int i0 = 0;
    lagrange7(z, cell, i0, w, nullptr);
    interp2c<NE>(c.table2c, cell, i0, w, v);
    rotate_plan<PA, PB, K2C>(R, v, X);
#pragma unroll
    for (int q = 0; q < NA * NB; q++) a.svnl[o + q] = X[q];
  } else {
    double dd[3][3][3];
    depsilon_2c(r1, r2, z, e, dd);
    DRotM D;
    dtwister<HASD>(e, dd, D);
    double eta[3] = {e[0][2], e[1][2], e[2][2]};
    double v[NE], dv[NE], vd[3 * NE], Xd[3 * NA * NB];
    interp2c_d<NE>(c.table2c, cell, z, z < 1.0e-5, v, dv, c.status);
    vec2c<NE>(z, eta, dv, vd);
    drotate_plan<PA, PB, K2C>(R, D, v, vd, Xd);
#pragma unroll
    for (int q = 0; q < 3 * NA * NB; q++) a.dsvnl[3 * o + q] = Xd[q];
  }
}

template <int PA, bool HASD, bool DERIV>
__device__ __forceinline__ void pair_svnl_dispatch(const Ctx2c &c, const PPArgs &a, int i, int p) {
  int pb = c.fd->sp[c.isp[c.neigh_j[p]]].pp_pattern;
  if (pb == PAT_SP) pair_svnl<PA, PAT_SP, HASD, DERIV>(c, a, i, p);
  else if (pb == PAT_S) pair_svnl<PA, PAT_S, HASD, DERIV>(c, a, i, p);
  else if constexpr (HASD) pair_svnl<PA, PAT_SPD, HASD, DERIV>(c, a, i, p);
}

template <bool HASD, bool DERIV>
__global__ void __launch_bounds__(256) k_svnl(Ctx2c c, PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  int pa = c.fd->sp[c.isp[i]].pattern;
  for (int p = a.pp_off[i] + lane; p < a.pp_off[i + 1]; p += 32) {
    if (pa == PAT_SP) pair_svnl_dispatch<PAT_SP, HASD, DERIV>(c, a, i, p);
    else if (pa == PAT_S) pair_svnl_dispatch<PAT_S, HASD, DERIV>(c, a, i, p);
    else if constexpr (HASD) pair_svnl_dispatch<PAT_SPD, HASD, DERIV>(c, a, i, p);
  }
}

// sum_ncc cl(ncc) A(imu, ncc) B(inu, ncc), A and B column-major with leading
// dimensions na, nb
__device__ __forceinline__ double cl_dot(const double *cl, int ncl, const double *A, int na, int imu, const double *B,
                                         int nb, int inu) {
  double s = 0.0;
  for (int k = 0; k < ncl; k++) s = fma(cl[k] * A[imu + na * k], B[inu + nb * k], s);
  return s;
}

// assemble_vnl_2c (M_assemble_PP_2c.f90:232-511).  One warp per atom i; its
// vnl blocks are cleared, then the ontop-left terms (projectors of i, PPx
// pairs), the ontop-right terms (projectors of j, PP pairs) and the atom term
// (both orbitals on i, projectors of each PP neighbor, a warp reduction into
// the self block).  Within each phase the lanes write distinct blocks.
template <int PA>
__device__ void atom_vnl_2c(const PPArgs &a, int i, int lane) {
  constexpr int NA = pat_norb(PA);
  const FdataDev &fd = *a.fd;
  int in1 = a.isp[i];
  for (long long q = a.vnl_base[i] + lane; q < a.vnl_base[i + 1]; q += 32) a.vnl[q] = 0.0;
  __syncwarp();
  const double *bself = a.svnl + a.svnl_off[a.pp_off[i] + a.pp_self[i]];
  for (int p = a.ppx_off[i] + lane; p < a.ppx_off[i + 1]; p += 32) {
    int j = a.ppx_j[p];
    if (j == i && a.ppx_b[p] == 0) continue;
    int nj = fd.sp[a.isp[j]].norb;
    const double *b2 = a.svnl + a.svnl_off[a.pp_off[j] + a.ppx_point[p]];
    double *dst = a.vnl + a.vnl_off[a.ppp_off[i] + a.ppx_map[p]];
    for (int inu = 0; inu < nj; inu++)
#pragma unroll
      for (int imu = 0; imu < NA; imu++)
        dst[imu + NA * inu] += cl_dot(fd.sp[in1].cl, fd.sp[in1].norb_pp, bself, NA, imu, b2, nj, inu);
  }
  __syncwarp();
  for (int p = a.pp_off[i] + lane; p < a.pp_off[i + 1]; p += 32) {
    int j = a.pp_j[p];
    if (j == i && a.pp_b[p] == 0) continue;
    const SpeciesDev &sj = fd.sp[a.isp[j]];
    int nj = sj.norb;
    const double *b1 = a.svnl + a.svnl_off[p];
    const double *b2 = a.svnl + a.svnl_off[a.pp_off[j] + a.pp_self[j]];
    double *dst = a.vnl + a.vnl_off[a.ppp_off[i] + a.pp_map[p]];
    for (int inu = 0; inu < nj; inu++)
#pragma unroll
      for (int imu = 0; imu < NA; imu++) dst[imu + NA * inu] += cl_dot(sj.cl, sj.norb_pp, b1, NA, imu, b2, nj, inu);
  }
  __syncwarp();
  double acc[NA * NA];
#pragma unroll
  for (int q = 0; q < NA * NA; q++) acc[q] = 0.0;
  for (int p = a.pp_off[i] + lane; p < a.pp_off[i + 1]; p += 32) {
    const SpeciesDev &sj = fd.sp[a.isp[a.pp_j[p]]];
    const double *b = a.svnl + a.svnl_off[p];
#pragma unroll
    for (int inu = 0; inu < NA; inu++)
#pragma unroll
      for (int imu = 0; imu < NA; imu++) acc[imu + NA * inu] += cl_dot(sj.cl, sj.norb_pp, b, NA, imu, b, NA, inu);
  }
#pragma unroll
  for (int q = 0; q < NA * NA; q++) {
    double v = acc[q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    acc[q] = v;
  }
  if (lane == 0) {
    double *dst = a.vnl + a.vnl_off[a.ppp_off[i] + a.ppp_self[i]];
#pragma unroll
    for (int q = 0; q < NA * NA; q++) dst[q] += acc[q];
  }
}

template <bool HASD>
__global__ void __launch_bounds__(256) k_vnl_2c(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int pa = a.fd->sp[a.isp[warp]].pattern;
  if (pa == PAT_SP) atom_vnl_2c<PAT_SP>(a, warp, lane);
  else if (pa == PAT_S) atom_vnl_2c<PAT_S>(a, warp, lane);
  else if constexpr (HASD) atom_vnl_2c<PAT_SPD>(a, warp, lane);
}

// assemble_vnl_3c (M_assemble_PP_3c.f90:94-229): one thread per triplet,
// FP64 atomics into block (i, neigh_common)
__global__ void __launch_bounds__(256) k_vnl_3c(PPArgs a, int T) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const FdataDev &fd = *a.fd;
  int al = a.t_alpha[t], i = a.t_i[t], j = a.t_j[t];
  const SpeciesDev &sa = fd.sp[a.isp[al]];
  int ni = fd.sp[a.isp[i]].norb, nj = fd.sp[a.isp[j]].norb;
  const double *b1 = a.svnl + a.svnl_off[a.pp_off[i] + a.t_m31[t]];
  const double *b2 = a.svnl + a.svnl_off[a.pp_off[j] + a.t_m32[t]];
  double *dst = a.vnl + a.vnl_off[a.ppp_off[i] + a.t_m[t]];
  for (int inu = 0; inu < nj; inu++)
    for (int imu = 0; imu < ni; imu++) atomicAdd(dst + imu + ni * inu, cl_dot(sa.cl, sa.norb_pp, b1, ni, imu, b2, nj, inu));
}

// ---------------------------------------------------------------------------
// force pass (Dassemble_vnl_2c, M_Dassemble_PP_2c.f90:420-745;
// Dassemble_vnl_3c, M_Dassemble_PP_3c.f90:127-265)
// ---------------------------------------------------------------------------
// sum_ncc cl(ncc) D(c, imu, ncc) B(inu, ncc) for the three c; D is the
// Dblock (3, na, ncl)
__device__ __forceinline__ void cl_dot_d(const double *cl, int ncl, const double *D, int na, int imu, const double *B,
                                         int nb, int inu, double out[3]) {
  out[0] = out[1] = out[2] = 0.0;
  for (int k = 0; k < ncl; k++) {
    double w = cl[k] * B[inu + nb * k];
#pragma unroll
    for (int c = 0; c < 3; c++) out[c] = fma(D[c + 3 * (imu + na * k)], w, out[c]);
  }
}

// vnl_atom per PP pair (the self pair stays zero) and vnl_ontop per PPx pair
// (ontop left; the reference leaves the ontop-right force out, :737-738, and
// build_forces doubles the left one).  One warp per atom, lanes over pairs.
__global__ void __launch_bounds__(256) k_dvnl_2c(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  const FdataDev &fd = *a.fd;
  const SpeciesDev &si = fd.sp[a.isp[i]];
  int ni = si.norb;
  const double *rs = a.rho_pp + a.vnl_off[a.ppp_off[i] + a.ppp_self[i]];
  for (int p = a.pp_off[i] + lane; p < a.pp_off[i + 1]; p += 32) {
    double f[3] = {0.0, 0.0, 0.0};
    if (p - a.pp_off[i] != a.pp_self[i]) {
      const SpeciesDev &sj = fd.sp[a.isp[a.pp_j[p]]];
      const double *b = a.svnl + a.svnl_off[p], *D = a.dsvnl + 3 * a.svnl_off[p];
      for (int inu = 0; inu < ni; inu++)
        for (int imu = 0; imu < ni; imu++) {
          double x1[3], x2[3];
          cl_dot_d(sj.cl, sj.norb_pp, D, ni, imu, b, ni, inu, x1);
          cl_dot_d(sj.cl, sj.norb_pp, D, ni, inu, b, ni, imu, x2);
          double r = rs[imu + ni * inu];
#pragma unroll
          for (int c = 0; c < 3; c++) f[c] -= r * (x1[c] + x2[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) a.vnl_atom[3 * (long long)p + c] = f[c];
  }
  const double *bself = a.svnl + a.svnl_off[a.pp_off[i] + a.pp_self[i]];
  for (int p = a.ppx_off[i] + lane; p < a.ppx_off[i + 1]; p += 32) {
    double f[3] = {0.0, 0.0, 0.0};
    int j = a.ppx_j[p];
    if (!(j == i && a.ppx_b[p] == 0)) {
      int nj = fd.sp[a.isp[j]].norb;
      const double *D2 = a.dsvnl + 3 * a.svnl_off[a.pp_off[j] + a.ppx_point[p]];
      const double *r = a.rho_pp + a.vnl_off[a.ppp_off[i] + a.ppx_map[p]];
      for (int inu = 0; inu < nj; inu++)
        for (int imu = 0; imu < ni; imu++) {
          // PPx = - sum cl svnl1(imu, ncc) Dsvnl2(:, inu, ncc); f -= rho PPx
          double x[3];
          cl_dot_d(si.cl, si.norb_pp, D2, nj, inu, bself, ni, imu, x);
          double rr = r[imu + ni * inu];
#pragma unroll
          for (int c = 0; c < 3; c++) f[c] += rr * x[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) a.vnl_ontop[3 * (long long)p + c] = f[c];
  }
}

// f3nl: xb = sum rho cl Dsvnl1 svnl2, xc = sum rho cl svnl1 Dsvnl2,
// f3nlb(i) -= xb, f3nlc(j) -= xc, f3nla(alpha) += xb + xc
__global__ void __launch_bounds__(256) k_dvnl_3c(PPArgs a, int T) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const FdataDev &fd = *a.fd;
  int al = a.t_alpha[t], i = a.t_i[t], j = a.t_j[t];
  const SpeciesDev &sa = fd.sp[a.isp[al]];
  int ni = fd.sp[a.isp[i]].norb, nj = fd.sp[a.isp[j]].norb;
  long long o1 = a.svnl_off[a.pp_off[i] + a.t_m31[t]], o2 = a.svnl_off[a.pp_off[j] + a.t_m32[t]];
  const double *b1 = a.svnl + o1, *b2 = a.svnl + o2, *D1 = a.dsvnl + 3 * o1, *D2 = a.dsvnl + 3 * o2;
  const double *r = a.rho_pp + a.vnl_off[a.ppp_off[i] + a.t_m[t]];
  double xb[3] = {0.0, 0.0, 0.0}, xc[3] = {0.0, 0.0, 0.0};
  for (int inu = 0; inu < nj; inu++)
    for (int imu = 0; imu < ni; imu++) {
      double rr = r[imu + ni * inu], u[3], v[3];
      cl_dot_d(sa.cl, sa.norb_pp, D1, ni, imu, b2, nj, inu, u);
      cl_dot_d(sa.cl, sa.norb_pp, D2, nj, inu, b1, ni, imu, v);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        xb[c] = fma(rr, u[c], xb[c]);
        xc[c] = fma(rr, v[c], xc[c]);
      }
    }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    atomicAdd(a.f3nla + 3 * al + c, xb[c] + xc[c]);
    atomicAdd(a.f3nlb + 3 * i + c, -xb[c]);
    atomicAdd(a.f3nlc + 3 * j + c, -xc[c]);
  }
}

// build_forces vnl terms (M_build_forces.f90:395-461): fvnl(i) += vnl_atom,
// fvnl(j) -= vnl_atom over PP pairs; += / -= 2 vnl_ontop over PPx pairs
__global__ void k_pp_force_sums(PPArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.N) return;
  int i = warp;
  double fi[3] = {0.0, 0.0, 0.0};
  for (int p = a.pp_off[i] + lane; p < a.pp_off[i + 1]; p += 32) {
    int j = a.pp_j[p];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double v = a.vnl_atom[3 * (long long)p + c];
      fi[c] += v;
      atomicAdd(a.fvnl + 3 * j + c, -v);
    }
  }
  for (int p = a.ppx_off[i] + lane; p < a.ppx_off[i + 1]; p += 32) {
    int j = a.ppx_j[p];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double v = 2.0 * a.vnl_ontop[3 * (long long)p + c];
      fi[c] += v;
      atomicAdd(a.fvnl + 3 * j + c, -v);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double v = fi[c];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    if (lane == 0) atomicAdd(a.fvnl + 3 * i + c, v);
  }
}

// ftot += fvnl + f3nla + f3nlb + f3nlc
__global__ void k_pp_ftot(PPArgs a) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 3 * a.N) return;
  a.ftot[k] += a.fvnl[k] + a.f3nla[k] + a.f3nlb[k] + a.f3nlc[k];
}

Ctx2c pp_ctx2c(const PPArgs &a) {
  Ctx2c c{};
  c.N = a.N;
  c.ratom = a.ratom;
  c.sid = a.sid;
  c.isp = a.isp;
  c.fd = a.fd;
  c.table2c = a.table2c;
  c.xl = a.xl;
  c.neigh_j = a.pp_j;
  c.neigh_b = a.pp_b;
  c.status = a.status;
  return c;
}

inline dim3 warp_grid(int n) { return dim3((unsigned)(((long long)n * 32 + 255) / 256)); }
inline dim3 thread_grid(long long n) { return dim3((unsigned)((n + 255) / 256)); }

}  // namespace

int launch_pp_pairs(const PPArgs &a, int kind, bool fill, cudaStream_t s) {
  if (fill) k_pp_pairs<true><<<warp_grid(a.N), 256, 0, s>>>(a, kind);
  else k_pp_pairs<false><<<warp_grid(a.N), 256, 0, s>>>(a, kind);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_ppp_bounds(const PPArgs &a, cudaStream_t s) {
  k_ppp_bounds<<<thread_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_ppp(const PPArgs &a, cudaStream_t s) {
  k_ppp<<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_ppp_compact(const PPArgs &a, int npp, int nppx, cudaStream_t s) {
  (void)npp;
  (void)nppx;
  k_ppp_compact<<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  k_pp_maps<<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_ppc(const PPArgs &a, bool fill, cudaStream_t s) {
  if (fill) k_ppc<true><<<warp_grid(a.N), 256, 0, s>>>(a);
  else k_ppc<false><<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_svnl(const PPArgs &a, int npp, bool deriv, cudaStream_t s) {
  if (npp == 0) return 0;
  Ctx2c c = pp_ctx2c(a);
  if (a.have_d) {
    if (deriv) k_svnl<true, true><<<warp_grid(a.N), 256, 0, s>>>(c, a);
    else k_svnl<true, false><<<warp_grid(a.N), 256, 0, s>>>(c, a);
  } else {
    if (deriv) k_svnl<false, true><<<warp_grid(a.N), 256, 0, s>>>(c, a);
    else k_svnl<false, false><<<warp_grid(a.N), 256, 0, s>>>(c, a);
  }
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_vnl_2c(const PPArgs &a, cudaStream_t s) {
  if (a.have_d) k_vnl_2c<true><<<warp_grid(a.N), 256, 0, s>>>(a);
  else k_vnl_2c<false><<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_vnl_3c(const PPArgs &a, int ntrip, cudaStream_t s) {
  if (ntrip == 0) return 0;
  k_vnl_3c<<<thread_grid(ntrip), 256, 0, s>>>(a, ntrip);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dvnl_2c(const PPArgs &a, int npp, int nppx, cudaStream_t s) {
  (void)npp;
  (void)nppx;
  k_dvnl_2c<<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_dvnl_3c(const PPArgs &a, int ntrip, cudaStream_t s) {
  if (ntrip == 0) return 0;
  k_dvnl_3c<<<thread_grid(ntrip), 256, 0, s>>>(a, ntrip);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_pp_forces(const PPArgs &a, int npp, int nppx, cudaStream_t s) {
  (void)npp;
  (void)nppx;
  k_pp_force_sums<<<warp_grid(a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  k_pp_ftot<<<thread_grid(3LL * a.N), 256, 0, s>>>(a);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
