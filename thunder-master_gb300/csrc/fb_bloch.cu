// fb_bloch.cu -- Bloch sums of the neighbor blocks into dense complex
// H(k) and S(k), the step after the assembly (h.SOLVESH/M_kspace_Lowdin.f90:
// 680-708 for S, :796-853 for H): for every pair (iatom, ineigh)
//   M(jmu, jnu) += phase(k . (xl(mbeta) + r_j - r_i)) * block(imu, inu),
// jmu = imu + iblock_slot(iatom), jnu = inu + iblock_slot(jatom), with
// phase(dot) = cmplx(cos(dot), sin(dot))
// (h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:413-442).
#include "fb_common.cuh"

namespace fb {

// One thread per pair; pairs of the same (iatom, jatom) in different images
// add into the same entries, so the sums use FP64 atomics.  The output is
// column-major n x n complex (interleaved re, im), nk matrices one after
// another; the sum of up to three block sets (e.g. T + vna + vnao) is taken.
__global__ void k_bloch(int P, int nk, const double *__restrict__ kpts, const int *__restrict__ pair_owner,
                        const int *__restrict__ neigh_j, const double *__restrict__ r3v,
                        const long long *__restrict__ blk_off, const int *__restrict__ isp,
                        const FdataDev *__restrict__ fd, const int *__restrict__ slot, long long n,
                        const double *__restrict__ A, const double *__restrict__ B, const double *__restrict__ C,
                        double *__restrict__ out) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  int kk = blockIdx.y;
  if (p >= P || kk >= nk) return;
  int i = pair_owner[p], j = neigh_j[p];
  int ni = fd->sp[isp[i]].norb, nj = fd->sp[isp[j]].norb;
  const double *k = kpts + 3 * kk;
  double dot = k[0] * r3v[3 * p] + k[1] * r3v[3 * p + 1] + k[2] * r3v[3 * p + 2];
  double sn, cs;
  sincos(dot, &sn, &cs);
  long long o = blk_off[p];
  double *M = out + (long long)kk * 2 * n * n;
  long long r0 = slot[i], c0 = slot[j];
  for (int nu = 0; nu < nj; nu++)
    for (int mu = 0; mu < ni; mu++) {
      long long q = o + mu + (long long)ni * nu;
      double v = A[q];
      if (B) v += B[q];
      if (C) v += C[q];
      long long e = (r0 + mu) + n * (c0 + nu);
      atomicAdd(M + 2 * e, cs * v);
      atomicAdd(M + 2 * e + 1, sn * v);
    }
}

int launch_bloch(const AsmArgs &a, int P, int nk, const double *kpts, const int *pair_owner, const double *r3v,
                 const int *slot, long long n, const double *A, const double *B, const double *C, double *out,
                 cudaStream_t s) {
  if (P == 0 || nk == 0) return 0;
  dim3 block(128), grid((P + 127) / 128, nk);
  k_bloch<<<grid, block, 0, s>>>(P, nk, kpts, pair_owner, a.neigh_j, r3v, a.blk_off, a.isp, a.fd, slot, n, A, B, C,
                                  out);
  FB_LAUNCH_CHECK();
  return 0;
}

}  // namespace fb
