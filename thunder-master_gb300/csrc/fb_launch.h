// fb_launch.h -- kernel launchers of libfbgpu (host side of fb_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include "fb_internal.h"

namespace fb {

struct NeighArgs {
  int N, P, nimg;
  const double *ratom;
  const float4 *pos4;  // x, y, z, float cutoff of the atom's species
  float4 bbox_lo, bbox_hi;  // bounding box of the positions; bbox_lo.w = largest cutoff
  int periodic;
  const int *isp;
  const FdataDev *fd;
  const double *xl;
  const float *xlf;
  const int *imgs;
  int *cnt;
  long long *bsum;
  const long long *blk_base;
  int *pair_owner_w;
  long long *blk_off_w;
  int *talpha;
  const int *pair_off;
  int *neigh_j, *neigh_b, *neigh_self, *neigh_back;
  const int *pair_owner;
  double *r3v;
  int *tcnt;
  const int *trip_off;
  int *ci_j, *ci_b, *cj_j, *cj_b, *cneigh, *tdst;
  unsigned *status;
  int *errinfo;
};

struct AsmArgs {
  int N, ntrip, have_d;
  const double *ratom;
  const int *isp;
  const FdataDev *fd;
  const double *table2c, *table3c, *gxy;
  const unsigned char *lin;
  const double *xl;
  const int *pair_off, *neigh_j, *neigh_b, *neigh_self, *neigh_back;
  const long long *blk_off;
  const int *trip_alpha, *ci_j, *ci_b, *cj_j, *cj_b, *tdst;
  const int *tperm;  // triplet processing order (binned), or null
  double *S, *T, *vb, *vbo;
  const double *rho, *cape;
  double *dS, *dT;
  bool keep_dblocks;
  double *sumT, *sumS, *ontop, *atomf;
  double *f3naa, *f3nab, *f3nac;
  double *kin, *vna, *pul, *ftot;
  unsigned *status;
  const float2 *table3c_df;  // hi, lo float pairs of table3c
  float2 *rho_df;            // hi, lo float pairs of rho
};

int launch_neigh(const NeighArgs &a, bool fill, cudaStream_t s);
int launch_neigh_back(const NeighArgs &a, cudaStream_t s);
int launch_common(const NeighArgs &a, bool fill, cudaStream_t s);
// counting sort of the triplets by (species triple, 3c grid cell) -> perm
int launch_trip_bins(const NeighArgs &a, int T, int nsp, int cells, int *key, int *rank, int *hist, int *perm,
                     cudaStream_t s);
int launch_assemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s);
int launch_assemble_3c(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s);
int launch_dassemble_3c(const AsmArgs &a, cudaStream_t s);
int launch_build_forces(const AsmArgs &a, unsigned what, cudaStream_t s);
// double-float three-center kernels (s and sp bases) and the rho split
int launch_assemble_3c_df(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_3c_df(const AsmArgs &a, cudaStream_t s);
int launch_split_rho(const AsmArgs &a, long long nblock, cudaStream_t s);
// DFMA throughput probe: one warm-up and one timed launch
int probe_dfma(cudaStream_t s, double *ms, double *flops);
int probe_ffma(cudaStream_t s, double *ms, double *flops);

}  // namespace fb
