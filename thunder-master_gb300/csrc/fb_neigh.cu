// fb_neigh.cu -- sm_103a kernels building the neighbor and common-neighbor maps.
#include "fb_common.cuh"

namespace fb {

// ===========================================================================
// neighbor maps (c.SYSTEM/M_neighbors.f90:356-519, :681-812)
// ===========================================================================
// One CTA per atom i.  Its warps take the periodic images in turn; in an
// image, lanes sweep jatom.  The count pass counts each image's hits (and
// their norb sum) into shared memory, warp 0 scans the counts in increasing
// mbeta and stores each image's first slot and norb start; the fill pass
// sweeps again, writing each image's hits from those starts: the list comes
// out in the reference order (mbeta outer, jatom inner).  In a batch, j runs over the atoms of i's own structure and
// the images are that structure's.  A float prefilter with a 1e-2 A margin
// discards far pairs; every candidate is decided by the uncontracted FP64
// test of the reference: z = distance(r1, r2) < rc_i + rc_j - 0.01.
constexpr int NEIGH_THREADS = 256;
// per-image counts and norb sums of one atom live in static shared memory
static_assert(NIMG * (sizeof(int) + sizeof(long long)) <= 48 * 1024, "image box too large for k_neigh");

struct NeighAtom {
  int i, a0, a1, ni;
  double ri[3], rci;
  float4 pi;    // (x, y, z, float cutoff of species)
  float reach;  // float reach of atom i: its cutoff + the largest cutoff + margin
  float4 lo, hi;
  const float4 *cb;  // chunk boxes of the structure
  const double *X;
  const float *Xf;
};

// one image mb swept by one warp: returns the hit count (warp-uniform) and
// adds their norb sum to orb.  CHECK flags atoms closer than 0.5 A; WRITE
// stores the hits from slot off of i's list, block offsets from orb.
template <bool CHECK, bool WRITE>
__device__ __forceinline__ int neigh_sweep(const NeighAtom &A, int mb, int lane, int off, long long &orb,
                                           const double *__restrict__ ratom, const float4 *__restrict__ pos4,
                                           const int *__restrict__ isp, const FdataDev *__restrict__ fd, int base,
                                           long long bbase, int *__restrict__ neigh_j, int *__restrict__ neigh_b,
                                           int *__restrict__ neigh_self, int *__restrict__ pair_owner,
                                           long long *__restrict__ blk_off, unsigned *__restrict__ status,
                                           int *__restrict__ errinfo) {
  float L0 = A.Xf[3 * mb], L1 = A.Xf[3 * mb + 1], L2 = A.Xf[3 * mb + 2];
  // skip an image whose shifted bounding box lies beyond reach (warp-uniform)
  float ox = fmaxf(fmaxf(A.lo.x + L0 - A.pi.x, A.pi.x - (A.hi.x + L0)), 0.0f);
  float oy = fmaxf(fmaxf(A.lo.y + L1 - A.pi.y, A.pi.y - (A.hi.y + L1)), 0.0f);
  float oz = fmaxf(fmaxf(A.lo.z + L2 - A.pi.z, A.pi.z - (A.hi.z + L2)), 0.0f);
  if (ox * ox + oy * oy + oz * oz > A.reach * A.reach) return 0;
  double X0 = A.X[3 * mb], X1 = A.X[3 * mb + 1], X2 = A.X[3 * mb + 2];
  int num = 0;
  for (int j0 = A.a0; j0 < A.a1; j0 += 32) {
    // skip the chunk of 32 atoms whose shifted box lies beyond reach (warp-uniform)
    {
      const float4 clo = A.cb[2 * ((j0 - A.a0) >> 5)], chi = A.cb[2 * ((j0 - A.a0) >> 5) + 1];
      float cx = fmaxf(fmaxf(clo.x + L0 - A.pi.x, A.pi.x - (chi.x + L0)), 0.0f);
      float cy = fmaxf(fmaxf(clo.y + L1 - A.pi.y, A.pi.y - (chi.y + L1)), 0.0f);
      float cz = fmaxf(fmaxf(clo.z + L2 - A.pi.z, A.pi.z - (chi.z + L2)), 0.0f);
      if (cx * cx + cy * cy + cz * cz > A.reach * A.reach) continue;
    }
    int j = j0 + lane;
    bool hit = false;
    if (j < A.a1) {
      float4 pj = pos4[j];
      float d0 = (pj.x + L0) - A.pi.x, d1 = (pj.y + L1) - A.pi.y, d2 = (pj.z + L2) - A.pi.z;
      float lim = A.pi.w + pj.w + 1.0e-2f;
      if (d0 * d0 + d1 * d1 + d2 * d2 < lim * lim) {
        // the reference's test, uncontracted FP64
        double range = __dsub_rn(__dadd_rn(A.rci, fd->sp[isp[j]].rcA), 0.01);
        double r2[3] = {__dadd_rn(ratom[3 * j], X0), __dadd_rn(ratom[3 * j + 1], X1),
                        __dadd_rn(ratom[3 * j + 2], X2)};
        double z = dist_rn(A.ri, r2);
        if (CHECK && A.i != j && z < 0.5) {
          atomicOr(status, DEVERR_CLOSE);
          errinfo[0] = A.i;
          errinfo[1] = j;
          errinfo[2] = mb;
        }
        hit = z < range;
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m == 0u) continue;
    // inclusive warp scan of norb_j over the hit lanes -> block offsets
    int nj = hit ? fd->sp[isp[j]].norb : 0;
    int incl = nj;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += u;
    }
    if (WRITE && hit) {
      int idx = off + num + __popc(m & ((1u << lane) - 1u));
      neigh_j[base + idx] = j;
      neigh_b[base + idx] = mb;
      pair_owner[base + idx] = A.i;
      blk_off[base + idx] = bbase + (long long)A.ni * (orb + incl - nj);
      if (j == A.i && mb == 0) neigh_self[A.i] = idx;
    }
    num += __popc(m);
    orb += __shfl_sync(0xffffffffu, incl, 31);
  }
  return num;
}

template <bool FILL>
__global__ void __launch_bounds__(NEIGH_THREADS)
    k_neigh(int N, const double *__restrict__ ratom, const float4 *__restrict__ pos4, const int *__restrict__ isp,
            const FdataDev *__restrict__ fd, const int *__restrict__ sid, const int *__restrict__ satom_off,
            const int *__restrict__ simg_off, const float4 *__restrict__ sbbox, const float4 *__restrict__ cbox,
            const int *__restrict__ cb_off, float rcmax,
            const double *__restrict__ xl, const float *__restrict__ xlf, const int *__restrict__ imgs,
            int *__restrict__ cnt, long long *__restrict__ bsum, const int *__restrict__ pair_off,
            const long long *__restrict__ blk_base, int *__restrict__ neigh_j, int *__restrict__ neigh_b,
            int *__restrict__ neigh_self, int *__restrict__ pair_owner, long long *__restrict__ blk_off,
            const long long *__restrict__ img_off, int *__restrict__ img_start, long long *__restrict__ img_orb,
            unsigned *__restrict__ status, int *__restrict__ errinfo) {
  __shared__ int s_cnt[NIMG];         // hits of each image, then their first slot
  __shared__ long long s_orb[NIMG];   // norb sum of each image's hits, then its running start
  int i = blockIdx.x;
  if (i >= N) return;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  NeighAtom A;
  A.i = i;
  int s = sid[i];
  A.a0 = satom_off[s];
  A.a1 = satom_off[s + 1];
  A.X = xl + (long long)s * XL_STRIDE;
  A.Xf = xlf + (long long)s * XL_STRIDE;
  A.lo = sbbox[2 * s];
  A.hi = sbbox[2 * s + 1];
  A.cb = cbox + 2 * (long long)cb_off[s];
#pragma unroll
  for (int k = 0; k < 3; k++) A.ri[k] = ratom[3 * i + k];
  A.pi = pos4[i];
  A.rci = fd->sp[isp[i]].rcA;
  A.reach = A.pi.w + rcmax + 1.0e-2f;
  A.ni = fd->sp[isp[i]].norb;
  int g0 = simg_off[s], nimg = simg_off[s + 1] - g0;
  if (nimg > NIMG) {  // the image list holds each mbeta at most once
    if (threadIdx.x == 0) atomicOr(status, DEVERR_CAP);
    return;
  }
  int base = FILL ? pair_off[i] : 0;
  long long bbase = FILL ? blk_base[i] : 0;
  // this atom's per-image first slots and norb starts (count pass -> fill pass)
  long long ibase = img_off[s] + (long long)(i - A.a0) * nimg;
  if constexpr (FILL) {
    for (int k = warp; k < nimg; k += nw) {
      long long orb = img_orb[ibase + k];
      neigh_sweep<false, true>(A, imgs[g0 + k], lane, img_start[ibase + k], orb, ratom, pos4, isp, fd, base, bbase,
                               neigh_j, neigh_b, neigh_self, pair_owner, blk_off, status, errinfo);
    }
    __syncthreads();
    if (threadIdx.x == 0 && neigh_self[i] < 0) atomicOr(status, DEVERR_SELF);
    return;
  }
  for (int k = warp; k < nimg; k += nw) {
    long long orb = 0;
    int c = neigh_sweep<!FILL, false>(A, imgs[g0 + k], lane, 0, orb, ratom, pos4, isp, fd, base, bbase, neigh_j,
                                      neigh_b, neigh_self, pair_owner, blk_off, status, errinfo);
    if (lane == 0) {
      s_cnt[k] = c;
      s_orb[k] = orb;
    }
  }
  __syncthreads();
  if (warp == 0) {  // exclusive scan over the images, in list order
    int carry = 0;
    long long corb = 0;
    for (int k0 = 0; k0 < nimg; k0 += 32) {
      int k = k0 + lane;
      int c = k < nimg ? s_cnt[k] : 0;
      long long o = k < nimg ? s_orb[k] : 0;
      int x = c;
      long long y = o;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, x, d);
        long long v = __shfl_up_sync(0xffffffffu, y, d);
        if (lane >= d) {
          x += u;
          y += v;
        }
      }
      if (k < nimg) {
        img_start[ibase + k] = carry + x - c;
        img_orb[ibase + k] = corb + y - o;
      }
      carry += __shfl_sync(0xffffffffu, x, 31);
      corb += __shfl_sync(0xffffffffu, y, 31);
    }
    if (lane == 0) {
      cnt[i] = carry;
      bsum[i] = (long long)A.ni * corb;
    }
  }
}

// neigh_back (M_neighbors.f90:469-486) and the per-pair vectors
// r3 = xl(mbeta) + ratom(j) - ratom(i) used by find_common_neighbors
// (:776-779), and its float copy; one thread per pair.
__global__ void k_neigh_back(int N, int P, const int *__restrict__ pair_owner, const int *__restrict__ pair_off,
                             const int *__restrict__ neigh_j, const int *__restrict__ neigh_b,
                             const int *__restrict__ sid, const double *__restrict__ xl0,
                             const double *__restrict__ ratom, const float4 *__restrict__ pos4,
                             int *__restrict__ neigh_back, double *__restrict__ r3v, float4 *__restrict__ r3f,
                             unsigned *__restrict__ status) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int i = pair_owner[p], j = neigh_j[p], mb = neigh_b[p];
  const double *xl = xl0 + (long long)sid[i] * XL_STRIDE;
  int found = -999, nfound = 0;
  for (int q = pair_off[j]; q < pair_off[j + 1]; q++) {
    int k = neigh_j[q], jb = neigh_b[q];
    if (i != k || fabs(__dadd_rn(xl[3 * mb], xl[3 * jb])) > 1.0e-3 ||
        fabs(__dadd_rn(xl[3 * mb + 1], xl[3 * jb + 1])) > 1.0e-3 ||
        fabs(__dadd_rn(xl[3 * mb + 2], xl[3 * jb + 2])) > 1.0e-3) {
    } else {
      nfound++;
      found = q - pair_off[j];
    }
  }
  if (nfound != 1) atomicOr(status, DEVERR_BACK);
  neigh_back[p] = found;
  float f[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double v = __dsub_rn(__dadd_rn(xl[3 * mb + k], ratom[3 * j + k]), ratom[3 * i + k]);
    r3v[3 * p + k] = v;
    f[k] = __double2float_rn(v);
  }
  // float copy for the pre-tests of the common-neighbor search, with the
  // neighbor's species cutoff (rcA) in .w
  r3f[p] = make_float4(f[0], f[1], f[2], pos4[j].w);
}


// the reference's vector match of find_common_neighbors (:776-779),
// uncontracted FP64
__device__ __forceinline__ bool common_match(const double *r3, const double *r1, const double *r2) {
  return fabs(__dadd_rn(__dsub_rn(r3[0], r2[0]), r1[0])) < 1.0e-4 &&
         fabs(__dadd_rn(__dsub_rn(r3[1], r2[1]), r1[1])) < 1.0e-4 &&
         fabs(__dadd_rn(__dsub_rn(r3[2], r2[2]), r1[2])) < 1.0e-4;
}

// The same match decided in float where it is certain: r2 - r1 is the
// difference b - a of two relative vectors of ialpha's list and r3 = c is a
// relative vector of iat's list, all a few bohr long, so the float value of
// r3 - (r2 - r1) is within 2 u (|a| + |b| + |c|) of the exact one (u = 2^-24;
// the FP64 values differ from the exact ones by ~1e-15).  Returns 1 when every
// component is certainly below 1e-4, -1 when one is certainly not, and 0 in
// the band between (8 u (|a| + |b| + |c| + 1) wide each side), where the FP64
// test decides.
__device__ __forceinline__ int common_match_f(float4 c, float4 a, float d0, float d1, float d2, float4 b) {
  const float u8 = 4.76837158e-7f;  // 8 * 2^-24
  float e[3] = {c.x - d0, c.y - d1, c.z - d2};
  float t[3] = {u8 * (fabsf(a.x) + fabsf(b.x) + fabsf(c.x) + 1.0f), u8 * (fabsf(a.y) + fabsf(b.y) + fabsf(c.y) + 1.0f),
                u8 * (fabsf(a.z) + fabsf(b.z) + fabsf(c.z) + 1.0f)};
  bool sure = true;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float m = fabsf(e[k]);
    if (m >= 1.0e-4f + t[k]) return -1;
    sure = sure && m < 1.0e-4f - t[k];
  }
  return sure ? 1 : 0;
}

// find_common_max / find_common_neighbors: one warp per pair row
// (ialpha, ineigh), ineigh non-self; lanes sweep jneigh; a candidate (i, j)
// with |r1 - r2| < rc_i + rc_j - 0.01 is kept only if j is found in i's
// list by the reference's vector match (first kneigh with
// |r3 - r2 + r1| < 1e-4 per component).  The entry that can match is
// (jatom, shift(jbeta) - shift(ibeta)); i's list is sorted by (mbeta, jatom),
// so it is found by binary search and then tested exactly.  When that entry
// is absent or fails the test, the full scan of the reference decides.
// Each row writes its kept pairs (ineigh, jneigh) and matches, in jneigh
// order, to its own run of slots: ialpha's slots start at slot_off[ialpha]
// and hold n_ns rows of n_ns - 1 (n_ns non-self neighbors), row k for the
// k-th non-self ineigh.  rcnt gets the row's count and tcnt[ialpha] (zeroed
// by the caller) the sum over the rows; k_common_compact packs the rows in
// ineigh order, so the triplets come out in the reference's loop order.
constexpr int COMMON_THREADS = 256;  // k_common's block: 8 pair rows
constexpr int COMMON_KEYS = 128;     // longest neighbor list staged in shared memory

__global__ void k_common(int P, int N, const int *__restrict__ speriodic, const double *__restrict__ ratom,
                         const int *__restrict__ isp, const FdataDev *__restrict__ fd, const int *__restrict__ sid,
                         const double *__restrict__ xl0, const int *__restrict__ pair_owner,
                         const int *__restrict__ pair_off, const int *__restrict__ neigh_j,
                         const int *__restrict__ neigh_b, const int *__restrict__ neigh_self,
                         const double *__restrict__ r3v, const float4 *__restrict__ r3f, int *__restrict__ tcnt,
                         int *__restrict__ rcnt,
                         const long long *__restrict__ slot_off, unsigned *__restrict__ slot_nn,
                         int *__restrict__ slot_found) {
  int pi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (pi >= P) return;
  int ia = pair_owner[pi];
  int p0 = pair_off[ia], n = pair_off[ia + 1] - p0, self = neigh_self[ia];
  int in = pi - p0;
  if (self < 0 || in == self) {
    if (lane == 0) rcnt[pi] = 0;
    return;
  }
  const double *xl = xl0 + (long long)sid[ia] * XL_STRIDE;
  int periodic = speriodic[sid[ia]];
  int kidx = in - (in > self ? 1 : 0);
  long long base = slot_off[ia] + (long long)kidx * (n - 2);
  int num = 0;
  int iat = neigh_j[pi], ib = neigh_b[pi];
  // ialpha -> (iat, ib) as a float relative vector, iat's cutoff in .w; the
  // FP64 positions r1 (iat shifted by ib) and r2 (jat shifted by jb) are
  // formed only in the bands where the FP64 tests decide
  const float4 a4 = r3f[pi];
  int q0 = pair_off[iat], qn = pair_off[iat + 1];
  // iat's list keys (mbeta * N + jatom), which the binary searches below
  // probe, staged once per row in shared memory (lists up to COMMON_KEYS)
  __shared__ long long s_key[COMMON_THREADS / 32][COMMON_KEYS];
  long long *key_s = s_key[threadIdx.x >> 5];
  const bool kshared = qn - q0 <= COMMON_KEYS;
  if (kshared)
    for (int k = lane; k < qn - q0; k += 32) key_s[k] = (long long)neigh_b[q0 + k] * N + neigh_j[q0 + k];
  __syncwarp();
  int ibx, iby, ibz;
  mbeta_shift(ib, ibx, iby, ibz);
  for (int j0 = 0; j0 < n; j0 += 32) {
    int jn = j0 + lane;
    bool keep = false;
    int found = -1;
    int jat = 0, jb = 0;
    if (jn < n && jn != self && jn != in) {
      int pj = p0 + jn;
      jat = neigh_j[pj];
      jb = neigh_b[pj];
      // float pre-test on the relative vectors r2 - r1 = b - a (error
      // ~1e-6 bohr; the species cutoffs in .w): clearly beyond the range ->
      // rejected, clearly inside (0.01 of margin) -> kept without the FP64
      // distance; only the band between takes the reference's uncontracted
      // FP64 test
      const float4 b4 = r3f[pj];
      float d0 = b4.x - a4.x, d1 = b4.y - a4.y, d2 = b4.z - a4.z;
      float dd = d0 * d0 + d1 * d1 + d2 * d2;
      float lim = a4.w + b4.w + 1.0e-2f, sure = a4.w + b4.w - 2.0e-2f;
      bool inside = false;
      if (dd < lim * lim) {
        if (dd < sure * sure) {
          inside = true;
        } else {
          double r1[3], r2[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            r1[k] = __dadd_rn(ratom[3 * iat + k], xl[3 * ib + k]);
            r2[k] = __dadd_rn(ratom[3 * jat + k], xl[3 * jb + k]);
          }
          double z = dist_rn(r1, r2);
          double range = __dsub_rn(__dadd_rn(fd->sp[isp[iat]].rcA, fd->sp[isp[jat]].rcA), 0.01);
          inside = z < range;
        }
      }
      if (inside) {
        // the vector match, in float where certain (common_match_f) and in
        // FP64 in its band
        auto match = [&](int q) {
          int m = common_match_f(r3f[q], a4, d0, d1, d2, b4);
          if (m != 0) return m > 0;
          double r1[3], r2[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            r1[k] = __dadd_rn(ratom[3 * iat + k], xl[3 * ib + k]);
            r2[k] = __dadd_rn(ratom[3 * jat + k], xl[3 * jb + k]);
          }
          return common_match(r3v + 3 * q, r1, r2);
        };
        int tmb = 0;
        bool inbox = true;
        if (periodic) {
          int jbx, jby, jbz;
          mbeta_shift(jb, jbx, jby, jbz);
          int tx = jbx - ibx, ty = jby - iby, tz = jbz - ibz;
          inbox = tx >= -4 && tx <= 4 && ty >= -4 && ty <= 4 && tz >= -4 && tz <= 4;
          if (inbox) tmb = shift_mbeta(tx, ty, tz);
        }
        if (inbox) {
          long long key = (long long)tmb * N + jat;
          int lo = q0, hi = qn - 1;
          while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            long long km = kshared ? key_s[mid - q0] : (long long)neigh_b[mid] * N + neigh_j[mid];
            if (km < key) lo = mid + 1;
            else if (km > key) hi = mid - 1;
            else {
              if (match(mid)) found = mid - q0;
              break;
            }
          }
        }
        if (found < 0) {
          // rare: candidate at the cutoff edge; decide by the reference scan
          for (int q = q0; q < qn; q++)
            if (match(q)) {
              found = q - q0;
              break;
            }
        }
        keep = found >= 0;
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      long long t = base + num + __popc(m & ((1u << lane) - 1u));
      slot_nn[t] = (unsigned)in | ((unsigned)jn << 16);
      slot_found[t] = found;
    }
    num += __popc(m);
  }
  if (lane == 0) {
    rcnt[pi] = num;
    if (num) atomicAdd(tcnt + ia, num);
  }
}

// slots -> CSR triplet lists in the reference's field layout (one warp per
// ialpha): 32 rows at a time, an inclusive scan of their counts places each
// row's run; each lane finds the row of its output entry by binary search
// over the scan.
__global__ void k_common_compact(int N, const int *__restrict__ pair_off, const int *__restrict__ neigh_j,
                                 const int *__restrict__ neigh_b, const int *__restrict__ neigh_self,
                                 const int *__restrict__ rcnt, const long long *__restrict__ slot_off,
                                 const unsigned *__restrict__ slot_nn, const int *__restrict__ slot_found,
                                 const int *__restrict__ trip_off, int *__restrict__ ci_j, int *__restrict__ ci_b,
                                 int *__restrict__ cj_j, int *__restrict__ cj_b, int *__restrict__ cneigh,
                                 int *__restrict__ tdst, int *__restrict__ talpha) {
  int ia = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (ia >= N) return;
  int p0 = pair_off[ia], n = pair_off[ia + 1] - p0, self = neigh_self[ia];
  if (self < 0) return;
  int t = trip_off[ia];
  long long s0 = slot_off[ia];
  for (int r0 = 0; r0 < n; r0 += 32) {
    int c = r0 + lane < n ? rcnt[p0 + r0 + lane] : 0;
    int x = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    int ex = x - c;
    int total = __shfl_sync(0xffffffffu, x, 31);
    for (int e0 = 0; e0 < total; e0 += 32) {
      int e = e0 + lane;
      int k = 0;  // first row of the chunk whose inclusive count exceeds e
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1) {
        int v = __shfl_sync(0xffffffffu, x, k + step - 1);
        if (v <= e) k += step;
      }
      int rex = __shfl_sync(0xffffffffu, ex, k);
      if (e < total) {
        int in = r0 + k;
        long long s = s0 + (long long)(in - (in > self ? 1 : 0)) * (n - 2) + (e - rex);
        unsigned nn = slot_nn[s];
        int found = slot_found[s];
        int pi = p0 + (int)(nn & 0xffffu), pj = p0 + (int)(nn >> 16);
        int iat = neigh_j[pi];
        int o = t + e;
        ci_j[o] = iat;
        ci_b[o] = neigh_b[pi];
        cj_j[o] = neigh_j[pj];
        cj_b[o] = neigh_b[pj];
        cneigh[o] = found;
        tdst[o] = pair_off[iat] + found;
        talpha[o] = ia;
      }
    }
    t += total;
  }
}

// ---------------------------------------------------------------------------
// Triplet binning: a counting sort of the triplets by (species triple, 3c
// grid cell of the interpolation stencil), bins approved for the MLP-3c
// surrogate first.  The three-center kernels walk
// the triplets in this order, so neighboring lanes read the same table
// stencil (broadcast loads) and take the same interpolation branch.  The
// cell is computed with the set-up of assemble_vna_3c
// (M_assemble_3c_Harris.f90:160-186) and the index rule of getMEs_Fdata_3c
// (M_Fdata_3c.f90:367-376); it only orders the work.
// ---------------------------------------------------------------------------
// The bin is a sort key for table locality (and, with an MLP gate, the
// routing unit): without a gate the float positions decide it (a triplet
// within ~1e-5 A of a grid line may land in the neighboring bin, which only
// changes its place in the order); with a gate the key is computed in FP64.
template <bool EXACT>
__global__ void k_trip_key(int T, int nsp, int cells, const double *__restrict__ ratom,
                           const float4 *__restrict__ pos4, const float *__restrict__ xlf0,
                           const int *__restrict__ isp,
                           const FdataDev *__restrict__ fd, const int *__restrict__ sid,
                           const double *__restrict__ xl0,
                           const int *__restrict__ talpha, const int *__restrict__ ci_j, const int *__restrict__ ci_b,
                           const int *__restrict__ cj_j, const int *__restrict__ cj_b,
                           const unsigned char *__restrict__ binok, int *__restrict__ key, int *__restrict__ rank,
                           int *__restrict__ hist) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int ia = talpha[t], i = ci_j[t], j = cj_j[t], ib = ci_b[t], jb = cj_b[t];
  int a = isp[i], b = isp[j], c = isp[ia];
  const Cell3cDev &cell = fd->c3[a][b][c];
  int ix, iy;
  if constexpr (EXACT) {
    const double *xl = xl0 + (long long)sid[ia] * XL_STRIDE;
    double r1[3], r2[3], rn[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      r1[k] = ratom[3 * i + k] + xl[3 * ib + k];
      r2[k] = ratom[3 * j + k] + xl[3 * jb + k];
      rn[k] = ratom[3 * ia + k] - 0.5 * (r1[k] + r2[k]);
    }
    double z = sqrt((r2[0] - r1[0]) * (r2[0] - r1[0]) + (r2[1] - r1[1]) * (r2[1] - r1[1]) +
                    (r2[2] - r1[2]) * (r2[2] - r1[2]));
    double x = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
    ix = (int)(x / cell.dx) + 1;
    iy = (int)(z / cell.dy) + 1;
  } else {
    const float *xl = xlf0 + (long long)sid[ia] * XL_STRIDE;
    float4 pi = pos4[i], pj = pos4[j], pa = pos4[ia];
    float r1[3] = {pi.x + xl[3 * ib], pi.y + xl[3 * ib + 1], pi.z + xl[3 * ib + 2]};
    float r2[3] = {pj.x + xl[3 * jb], pj.y + xl[3 * jb + 1], pj.z + xl[3 * jb + 2]};
    float pn[3] = {pa.x, pa.y, pa.z};
    float zz = 0.0f, xx = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float d = r2[k] - r1[k], n = pn[k] - 0.5f * (r1[k] + r2[k]);
      zz += d * d;
      xx += n * n;
    }
    ix = (int)(sqrtf(xx) * cell.idx_h) + 1;
    iy = (int)(sqrtf(zz) * cell.idy_h) + 1;
  }
  ix = min(max(ix, 2), cell.nx - 2);
  iy = min(max(iy, 2), cell.ny - 2);
  int node = (iy - 1) * cell.nx + (ix - 1);
  int k = ((a * nsp + b) * nsp + c) * cells + min(node, cells - 1);
  // bins approved for the MLP-3c surrogate come first
  if (!(binok && binok[k])) k += nsp * nsp * nsp * cells;
  key[t] = k;
  // neighboring triplets share bins: one atomic per bin and warp, the lanes
  // of a bin ranked in lane order after the slots it reserves
  unsigned act = __activemask();
  unsigned peers = __match_any_sync(act, k);
  int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  int r0 = 0;
  if (lane == leader) r0 = atomicAdd(hist + k, __popc(peers));
  r0 = __shfl_sync(peers, r0, leader);
  rank[t] = r0 + __popc(peers & ((1u << lane) - 1u));
}

// exclusive scan of the bin counts, one block
__global__ void k_scan_bins(int nbins, int *__restrict__ hist) {
  __shared__ int part[1024];
  int tid = threadIdx.x;
  int per = (nbins + 1023) / 1024;
  int lo = tid * per, hi = min(lo + per, nbins);
  int sum = 0;
  for (int b = lo; b < hi; b++) sum += hist[b];
  part[tid] = sum;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    int v = tid >= d ? part[tid - d] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int run = part[tid] - sum;
  for (int b = lo; b < hi; b++) {
    int c = hist[b];
    hist[b] = run;
    run += c;
  }
}

__global__ void k_trip_scatter(int T, const int *__restrict__ key, const int *__restrict__ rank,
                               const int *__restrict__ start, int *__restrict__ perm) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  perm[start[key[t]] + rank[t]] = t;
}

// the triplet lists in the binned order, list position i holding triplet
// perm[i] (six arrays of T: talpha, ci_j, ci_b, cj_j, cj_b, tdst): the
// three-center kernels read these in order instead of gathering through
// perm, which cost one 32-byte sector per array and triplet
__global__ void k_trip_gather(int T, const int *__restrict__ perm, const int *__restrict__ talpha,
                              const int *__restrict__ ci_j, const int *__restrict__ ci_b, const int *__restrict__ cj_j,
                              const int *__restrict__ cj_b, const int *__restrict__ tdst, int *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T) return;
  int t = perm[i];
  long long n = T;
  out[i] = talpha[t];
  out[n + i] = ci_j[t];
  out[2 * n + i] = ci_b[t];
  out[3 * n + i] = cj_j[t];
  out[4 * n + i] = cj_b[t];
  out[5 * n + i] = tdst[t];
}

int launch_trip_bins(const NeighArgs &a, int T, int nsp, int cells, const unsigned char *binok, int *key, int *rank,
                     int *hist, int *perm, int *binned, cudaStream_t s) {
  if (T == 0) return 0;
  int nbins = 2 * nsp * nsp * nsp * cells;
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)nbins * sizeof(int), s);
  if (e != cudaSuccess) return (int)e;
  int threads = 256, blocks = (T + threads - 1) / threads;
  if (binok)
    k_trip_key<true><<<blocks, threads, 0, s>>>(T, nsp, cells, a.ratom, a.pos4, a.xlf, a.isp, a.fd, a.sid, a.xl,
                                                a.talpha, a.ci_j, a.ci_b, a.cj_j, a.cj_b, binok, key, rank, hist);
  else
    k_trip_key<false><<<blocks, threads, 0, s>>>(T, nsp, cells, a.ratom, a.pos4, a.xlf, a.isp, a.fd, a.sid, a.xl,
                                                 a.talpha, a.ci_j, a.ci_b, a.cj_j, a.cj_b, binok, key, rank, hist);
  FB_LAUNCH_CHECK();
  k_scan_bins<<<1, 1024, 0, s>>>(nbins, hist);
  FB_LAUNCH_CHECK();
  k_trip_scatter<<<blocks, threads, 0, s>>>(T, key, rank, hist, perm);
  FB_LAUNCH_CHECK();
  if (binned) {
    k_trip_gather<<<blocks, threads, 0, s>>>(T, perm, a.talpha, a.ci_j, a.ci_b, a.cj_j, a.cj_b, a.tdst, binned);
    FB_LAUNCH_CHECK();
  }
  return 0;
}

int launch_neigh(const NeighArgs &a, bool fill, cudaStream_t s) {
  if (a.N == 0) return 0;
  int threads = NEIGH_THREADS, blocks = a.N;
  if (fill)
    k_neigh<true><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.pos4, a.isp, a.fd, a.sid, a.satom_off, a.simg_off,
                                             a.sbbox, a.cbox, a.cb_off, a.rcmax, a.xl, a.xlf, a.imgs, nullptr, nullptr,
                                             a.pair_off,
                                             a.blk_base,
                                             a.neigh_j, a.neigh_b, a.neigh_self, a.pair_owner_w, a.blk_off_w,
                                             a.img_off, a.img_start, a.img_orb, a.status, a.errinfo);
  else
    k_neigh<false><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.pos4, a.isp, a.fd, a.sid, a.satom_off, a.simg_off,
                                              a.sbbox, a.cbox, a.cb_off, a.rcmax, a.xl, a.xlf, a.imgs, a.cnt, a.bsum,
                                              nullptr, nullptr,
                                              nullptr,
                                              nullptr, nullptr, nullptr, nullptr, a.img_off, a.img_start, a.img_orb,
                                              a.status, a.errinfo);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_neigh_back(const NeighArgs &a, cudaStream_t s) {
  if (a.P == 0) return 0;
  int threads = 256, blocks = (a.P + threads - 1) / threads;
  k_neigh_back<<<blocks, threads, 0, s>>>(a.N, a.P, a.pair_owner, a.pair_off, a.neigh_j, a.neigh_b, a.sid, a.xl,
                                          a.ratom, a.pos4, a.neigh_back, a.r3v, a.r3f, a.status);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_common(const NeighArgs &a, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.tcnt, 0, (size_t)a.N * sizeof(int), s);
  if (e != cudaSuccess) return (int)e;
  if (a.P == 0) return 0;
  int threads = COMMON_THREADS;
  long long blocks = ((long long)a.P * 32 + threads - 1) / threads;
  k_common<<<(unsigned)blocks, threads, 0, s>>>(a.P, a.N, a.speriodic, a.ratom, a.isp, a.fd, a.sid, a.xl,
                                                a.pair_owner, a.pair_off, a.neigh_j, a.neigh_b, a.neigh_self, a.r3v,
                                                a.r3f, a.tcnt, a.rcnt, a.slot_off, a.slot_nn, a.slot_found);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_common_compact(const NeighArgs &a, cudaStream_t s) {
  int threads = 128, blocks = (a.N * 32 + threads - 1) / threads;
  k_common_compact<<<blocks, threads, 0, s>>>(a.N, a.pair_off, a.neigh_j, a.neigh_b, a.neigh_self, a.rcnt,
                                              a.slot_off, a.slot_nn, a.slot_found, a.trip_off, a.ci_j, a.ci_b,
                                              a.cj_j, a.cj_b, a.cneigh, a.tdst, a.talpha);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
