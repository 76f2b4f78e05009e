// fb_ewald.h -- device arguments and launchers of the DOGS Ewald terms
// (j.ASSEMBLERS/M_assemble_ewald_DOGS.f90).
#pragma once
#include <cuda_runtime.h>

#include "fb_internal.h"

namespace fb {

struct EwaldArgs {
  int N, T;
  const double *ratom;
  const int *sid, *isp;
  const FdataDev *fd;
  const double *xl;
  // the reciprocal vectors g != 0 with stuff(g), the lattice vectors L, kappa
  int ng, nl;
  const double *gvec, *stuff, *lvec;
  double kappa;
  // neighbor and common-neighbor maps, block offsets
  const int *pair_off, *neigh_j, *neigh_b, *neigh_self;
  const long long *blk_off;
  const int *trip_alpha, *ci_j, *ci_b, *cj_j, *cj_b, *tdst;
  // charges: shell charges dq[atom][MAXSUB] -> atom totals dqa
  const double *dq;
  double *dqa;
  // per-atom structure factors cos / sin(g . r_i), [i * ng + k]
  double *sfc, *sfs;
  // outputs and inputs
  double *ewald, *sum_ewald;
  const double *S, *dip;
  double *sr, *lr;
  // force pass: per pair rho sums (S, dip, dS, ddip; 8 per pair), Q0 per
  // atom, dewald [(i * N + j) * 3 + c], per-atom weights and sums, forces
  const double *dogs_ps;
  double *q0a, *dewald, *w, *sum_dewald, *cw, *fewald, *fsr, *flr;
  double *f3naa, *f3nab, *f3nac, *ftot;
  const int *pair_owner;
  int P;
  // the lattice and reciprocal sums of the matrix and its derivative in
  // double-float (fb_ewald_df.cu) instead of FP64, with the lattice
  // vectors as hi/lo float pairs [3 * nl]
  int df;
  const float2 *lvec_df;
};

int launch_ewald_matrix(const EwaldArgs &e, cudaStream_t s);
int launch_ewald_blocks(const EwaldArgs &e, int have_d, cudaStream_t s);
// force pass: dewald and the Ewald energy force; the ewaldsr three-center
// terms into f3na (before build_forces); the ewaldsr / ewaldlr forces added
// into ftot (after build_forces)
int launch_dewald(const EwaldArgs &e, cudaStream_t s);
int launch_ewald_f3c(const EwaldArgs &e, cudaStream_t s);
// the double-float matrix and derivative sums (structure factors + tiles)
int launch_ewald_matrix_df(const EwaldArgs &e, cudaStream_t s);
int launch_dewald_tiles_df(const EwaldArgs &e, cudaStream_t s);
int launch_ewald_forces(const EwaldArgs &e, cudaStream_t s);

}  // namespace fb
