// fb_pp.h -- device arguments and launchers of the non-local pseudopotential
// (vnl) path: the PP, PPx and PPp neighbor maps and the PP common triplets
// (c.SYSTEM/M_neighbors_PP.f90), svnl and vnl assembly
// (j.ASSEMBLERS/M_assemble_PP_{2c,3c}.f90), their derivatives
// (k.DASSEMBLERS/M_Dassemble_PP_{2c,3c}.f90) and the vnl force sums of
// build_forces (c.SYSTEM/M_build_forces.f90:395-461).
#pragma once
#include <cuda_runtime.h>

#include "fb_internal.h"

namespace fb {

struct PPArgs {
  int N;
  const double *ratom;
  const float4 *pos4;
  const int *sid, *isp;
  const FdataDev *fd;
  const double *table2c;
  const double *xl;
  const float *xlf;
  const int *satom_off, *simg_off, *imgs;
  const float4 *sbbox;
  float reach;  // the largest pair cutoff of either kind, Angstrom
  int have_d;   // d shells among the basis or projector shells
  // PP (basis i, projector j): counts, CSR, self, svnl block offsets
  int *pp_cnt;
  long long *svnl_sum;
  const int *pp_off;
  const long long *svnl_base;
  int *pp_j, *pp_b, *pp_self, *pp_map;
  long long *svnl_off;
  // PPx (projector i, basis j)
  int *ppx_cnt;
  const int *ppx_off;
  int *ppx_j, *ppx_b, *ppx_self, *ppx_map, *ppx_point;
  // PPp (pairs sharing a projector): candidate slots, counts, CSR, vnl offsets
  int *ub;
  const long long *slot_off;
  int *slot_j, *slot_b;
  int *ppp_cnt;
  long long *vnl_sum;
  const int *ppp_off;
  const long long *vnl_base;
  int *ppp_j, *ppp_b, *ppp_self;
  long long *vnl_off;
  // PP common triplets of each alpha
  int *ppc_cnt;
  const int *ppc_off;
  int *t_alpha, *t_i, *t_ib, *t_j, *t_jb, *t_m, *t_m31, *t_m32;
  // blocks and forces
  double *svnl, *dsvnl, *vnl;
  const double *rho_pp;
  double *vnl_atom, *vnl_ontop, *f3nla, *f3nlb, *f3nlc, *fvnl, *ftot;
  unsigned *status;
  int *errinfo;
};

// maps: PP / PPx pairs (count, then fill at pp_off / ppx_off)
int launch_pp_pairs(const PPArgs &a, int kind, bool fill, cudaStream_t s);
// PPp: candidate upper bounds per atom, then the first-occurrence search
// into the slots, then the compaction (with the PP / PPx maps and points)
int launch_ppp_bounds(const PPArgs &a, cudaStream_t s);
int launch_ppp(const PPArgs &a, cudaStream_t s);
int launch_ppp_compact(const PPArgs &a, int npp, int nppx, cudaStream_t s);
// PP common triplets (count, then fill at ppc_off)
int launch_ppc(const PPArgs &a, bool fill, cudaStream_t s);
// value pass: svnl (PP pairs), vnl 2c (atoms), vnl 3c (triplets, accumulates)
int launch_svnl(const PPArgs &a, int npp, bool deriv, cudaStream_t s);
int launch_vnl_2c(const PPArgs &a, cudaStream_t s);
int launch_vnl_3c(const PPArgs &a, int ntrip, cudaStream_t s);
// force pass: vnl_atom / vnl_ontop, f3nl (accumulates), the vnl force sums
int launch_dvnl_2c(const PPArgs &a, int npp, int nppx, cudaStream_t s);
int launch_dvnl_3c(const PPArgs &a, int ntrip, cudaStream_t s);
int launch_pp_forces(const PPArgs &a, int npp, int nppx, cudaStream_t s);

}  // namespace fb
