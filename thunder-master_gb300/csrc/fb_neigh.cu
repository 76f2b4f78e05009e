// fb_neigh.cu -- sm_103a kernels building the neighbor and common-neighbor maps.
#include "fb_common.cuh"

namespace fb {

// ===========================================================================
// neighbor maps (c.SYSTEM/M_neighbors.f90:356-519, :681-812)
// ===========================================================================
// One warp per atom i; lanes sweep jatom inside each periodic image, images
// in increasing mbeta, so hits come out in the reference order (mbeta
// outer, jatom inner).  A float prefilter with a 1e-2 A margin discards far
// pairs; every candidate is decided by the uncontracted FP64 test of the
// reference: z = distance(r1, r2) < rc_i + rc_j - 0.01.
template <bool FILL>
__global__ void k_neigh(int N, const double *__restrict__ ratom, const float *__restrict__ ratomf,
                        const int *__restrict__ isp, const FdataDev *__restrict__ fd, const double *__restrict__ xl,
                        const float *__restrict__ xlf, const int *__restrict__ imgs, int nimg, int *__restrict__ cnt,
                        long long *__restrict__ bsum, const int *__restrict__ pair_off,
                        const long long *__restrict__ blk_base, int *__restrict__ neigh_j, int *__restrict__ neigh_b,
                        int *__restrict__ neigh_self, int *__restrict__ pair_owner, long long *__restrict__ blk_off,
                        unsigned *__restrict__ status, int *__restrict__ errinfo) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= N) return;
  int i = warp;
  double ri[3] = {ratom[3 * i], ratom[3 * i + 1], ratom[3 * i + 2]};
  float rfi0 = ratomf[3 * i], rfi1 = ratomf[3 * i + 1], rfi2 = ratomf[3 * i + 2];
  double rci = fd->sp[isp[i]].rcA;
  int num = 0, base = FILL ? pair_off[i] : 0;
  long long norbsum = 0;  // sum of norb_j over the hits so far
  long long bbase = FILL ? blk_base[i] : 0;
  int ni = fd->sp[isp[i]].norb;
  for (int ii = 0; ii < nimg; ii++) {
    int mb = imgs[ii];
    float L0 = xlf[3 * mb], L1 = xlf[3 * mb + 1], L2 = xlf[3 * mb + 2];
    double X0 = xl[3 * mb], X1 = xl[3 * mb + 1], X2 = xl[3 * mb + 2];
    for (int j0 = 0; j0 < N; j0 += 32) {
      int j = j0 + lane;
      bool hit = false;
      if (j < N) {
        double rcj = fd->sp[isp[j]].rcA;
        double range = __dsub_rn(__dadd_rn(rci, rcj), 0.01);
        float d0 = (ratomf[3 * j] + L0) - rfi0, d1 = (ratomf[3 * j + 1] + L1) - rfi1,
              d2 = (ratomf[3 * j + 2] + L2) - rfi2;
        float lim = (float)range + 1.0e-2f;
        if (d0 * d0 + d1 * d1 + d2 * d2 < lim * lim) {
          double r2[3] = {__dadd_rn(ratom[3 * j], X0), __dadd_rn(ratom[3 * j + 1], X1),
                          __dadd_rn(ratom[3 * j + 2], X2)};
          double z = dist_rn(ri, r2);
          if (!FILL && i != j && z < 0.5) {
            atomicOr(status, DEVERR_CLOSE);
            errinfo[0] = i;
            errinfo[1] = j;
            errinfo[2] = mb;
          }
          hit = z < range;
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, hit);
      // inclusive warp scan of norb_j over the hit lanes -> block offsets
      int nj = hit ? fd->sp[isp[j]].norb : 0;
      int incl = nj;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += u;
      }
      if (FILL && hit) {
        int idx = num + __popc(m & ((1u << lane) - 1u));
        neigh_j[base + idx] = j;
        neigh_b[base + idx] = mb;
        pair_owner[base + idx] = i;
        blk_off[base + idx] = bbase + (long long)ni * (norbsum + incl - nj);
        if (j == i && mb == 0) neigh_self[i] = idx;
      }
      num += __popc(m);
      norbsum += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  if (!FILL && lane == 0) {
    cnt[i] = num;
    bsum[i] = (long long)ni * norbsum;
  }
  if (FILL) {
    __syncwarp();
    if (lane == 0 && neigh_self[i] < 0) atomicOr(status, DEVERR_SELF);
  }
}

// neigh_back (M_neighbors.f90:469-486) and the per-pair vectors
// r3 = xl(mbeta) + ratom(j) - ratom(i) used by find_common_neighbors
// (:776-779); one thread per pair.
__global__ void k_neigh_back(int N, int P, const int *__restrict__ pair_owner, const int *__restrict__ pair_off,
                             const int *__restrict__ neigh_j, const int *__restrict__ neigh_b,
                             const double *__restrict__ xl, const double *__restrict__ ratom,
                             int *__restrict__ neigh_back, double *__restrict__ r3v, float *__restrict__ r3f,
                             unsigned *__restrict__ status) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int i = pair_owner[p], j = neigh_j[p], mb = neigh_b[p];
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
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double v = __dsub_rn(__dadd_rn(xl[3 * mb + k], ratom[3 * j + k]), ratom[3 * i + k]);
    r3v[3 * p + k] = v;
    r3f[3 * p + k] = (float)v;
  }
}

// find_common_max / find_common_neighbors: one warp per ialpha; for each
// non-self ineigh (warp-uniform), lanes sweep jneigh; a candidate (i, j)
// with |r1 - r2| < rc_i + rc_j - 0.01 is kept only if j is found in i's
// list by vector match (first kneigh with |r3 - r2 + r1| < 1e-4 per
// component).  Output order matches the reference loops.
template <bool FILL>
__global__ void k_common(int N, const double *__restrict__ ratom, const int *__restrict__ isp,
                         const FdataDev *__restrict__ fd, const double *__restrict__ xl,
                         const int *__restrict__ pair_off, const int *__restrict__ neigh_j,
                         const int *__restrict__ neigh_b, const int *__restrict__ neigh_self,
                         const double *__restrict__ r3v, const float *__restrict__ r3f, int *__restrict__ tcnt,
                         const int *__restrict__ trip_off, int *__restrict__ ci_j, int *__restrict__ ci_b,
                         int *__restrict__ cj_j, int *__restrict__ cj_b, int *__restrict__ cneigh,
                         int *__restrict__ tdst, int *__restrict__ talpha) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= N) return;
  int ia = warp;
  int p0 = pair_off[ia], n = pair_off[ia + 1] - p0, self = neigh_self[ia];
  int num = 0, base = FILL ? trip_off[ia] : 0;
  for (int in = 0; in < n; in++) {
    if (in == self) continue;
    int pi = p0 + in, iat = neigh_j[pi], ib = neigh_b[pi];
    double r1[3];
#pragma unroll
    for (int k = 0; k < 3; k++) r1[k] = __dadd_rn(ratom[3 * iat + k], xl[3 * ib + k]);
    float r1f[3] = {(float)r1[0], (float)r1[1], (float)r1[2]};
    double rci = fd->sp[isp[iat]].rcA;
    int q0 = pair_off[iat], qn = pair_off[iat + 1];
    for (int j0 = 0; j0 < n; j0 += 32) {
      int jn = j0 + lane;
      bool keep = false;
      int found = -1;
      int jat = 0, jb = 0;
      if (jn < n && jn != self && jn != in) {
        int pj = p0 + jn;
        jat = neigh_j[pj];
        jb = neigh_b[pj];
        double r2[3];
#pragma unroll
        for (int k = 0; k < 3; k++) r2[k] = __dadd_rn(ratom[3 * jat + k], xl[3 * jb + k]);
        double z = dist_rn(r1, r2);
        double range = __dsub_rn(__dadd_rn(rci, fd->sp[isp[jat]].rcA), 0.01);
        if (z < range) {
          float r2f[3] = {(float)r2[0], (float)r2[1], (float)r2[2]};
          for (int q = q0; q < qn; q++) {
            // float prefilter of the 1e-4 vector match, then the exact test
            float e0 = fabsf(r3f[3 * q] - r2f[0] + r1f[0]);
            float e1 = fabsf(r3f[3 * q + 1] - r2f[1] + r1f[1]);
            float e2 = fabsf(r3f[3 * q + 2] - r2f[2] + r1f[2]);
            if (e0 < 1.0e-2f && e1 < 1.0e-2f && e2 < 1.0e-2f) {
              if (fabs(__dadd_rn(__dsub_rn(r3v[3 * q], r2[0]), r1[0])) < 1.0e-4 &&
                  fabs(__dadd_rn(__dsub_rn(r3v[3 * q + 1], r2[1]), r1[1])) < 1.0e-4 &&
                  fabs(__dadd_rn(__dsub_rn(r3v[3 * q + 2], r2[2]), r1[2])) < 1.0e-4) {
                found = q - q0;
                break;
              }
            }
          }
          keep = found >= 0;
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, keep);
      if (FILL && keep) {
        int t = base + num + __popc(m & ((1u << lane) - 1u));
        ci_j[t] = iat;
        ci_b[t] = ib;
        cj_j[t] = jat;
        cj_b[t] = jb;
        cneigh[t] = found;
        tdst[t] = q0 + found;
        talpha[t] = ia;
      }
      num += __popc(m);
    }
  }
  if (!FILL && lane == 0) tcnt[ia] = num;
}

int launch_neigh(const NeighArgs &a, bool fill, cudaStream_t s) {
  int threads = 128, blocks = (a.N * 32 + threads - 1) / threads;
  if (fill)
    k_neigh<true><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.ratomf, a.isp, a.fd, a.xl, a.xlf, a.imgs, a.nimg,
                                             nullptr, nullptr, a.pair_off, a.blk_base, a.neigh_j, a.neigh_b,
                                             a.neigh_self, a.pair_owner_w, a.blk_off_w, a.status, a.errinfo);
  else
    k_neigh<false><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.ratomf, a.isp, a.fd, a.xl, a.xlf, a.imgs, a.nimg,
                                              a.cnt, a.bsum, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                              nullptr, a.status, a.errinfo);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_neigh_back(const NeighArgs &a, cudaStream_t s) {
  if (a.P == 0) return 0;
  int threads = 256, blocks = (a.P + threads - 1) / threads;
  k_neigh_back<<<blocks, threads, 0, s>>>(a.N, a.P, a.pair_owner, a.pair_off, a.neigh_j, a.neigh_b, a.xl, a.ratom,
                                          a.neigh_back, a.r3v, a.r3f, a.status);
  FB_LAUNCH_CHECK();
  return 0;
}

int launch_common(const NeighArgs &a, bool fill, cudaStream_t s) {
  int threads = 128, blocks = (a.N * 32 + threads - 1) / threads;
  if (fill)
    k_common<true><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.isp, a.fd, a.xl, a.pair_off, a.neigh_j, a.neigh_b,
                                              a.neigh_self, a.r3v, a.r3f, nullptr, a.trip_off, a.ci_j, a.ci_b,
                                              a.cj_j, a.cj_b, a.cneigh, a.tdst, a.talpha);
  else
    k_common<false><<<blocks, threads, 0, s>>>(a.N, a.ratom, a.isp, a.fd, a.xl, a.pair_off, a.neigh_j, a.neigh_b,
                                               a.neigh_self, a.r3v, a.r3f, a.tcnt, nullptr, nullptr, nullptr,
                                               nullptr, nullptr, nullptr, nullptr, nullptr);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
