// fb_vxc.h -- device arguments and launchers of the McWEDA
// exchange-correlation assembly, Harris (j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90,
// M_assemble_rho_McWEDA_Harris.f90).
#pragma once
#include <cuda_runtime.h>

#include "fb_launch.h"

namespace fb {

// Orbital blocks (rho_in, rho_bond, vxc) use the pair block layout
// (blk_off); the shell-level weighted densities hold VXC_WSH doubles per
// pair, element (issh, jssh) at [VXC_WSH p + issh + nssh_i jssh].
constexpr int VXC_WSH = MAXSUB * MAXSUB;

struct VxcArgs {
  AsmArgs a;               // geometry, maps, tables; a.S is the overlap
  double *rho_in, *rho_bond;
  double *wrho_in, *wrho_bond;
  double *vxc;
  // force pass: the density matrix is a.rho; vxc_off_site / vxc_on_site
  // (3 per pair); the three-center weights of each pair, rho dmuxc (pair
  // block layout) and the shell sums of rho d2muxc (rho_in - W S)
  // (VXC_WSH per pair); f3xc a/b/c and the vxc pair-sum force (3 N); a.ftot
  double *off, *on;
  double *wd, *gd;
  double *f3a, *f3b, *f3c, *fvxc;
  // every species triple has Qneutral-summed three-center cells (one kernel
  // launch; otherwise a second one takes the triples that lack them)
  int qsum_all;
};

// assemble_rho_2c + assemble_rho_weighted_2c: writes all four density sets
int launch_rho_2c(const VxcArgs &v, cudaStream_t s);
// assemble_rho_3c + assemble_rho_weighted_3c: accumulates onto rho_in, wrho_in
int launch_rho_3c(const VxcArgs &v, cudaStream_t s);
// the same in double-float on the FP32 pipe (s and sp bases)
int launch_rho_3c_df(const VxcArgs &v, cudaStream_t s);
// assemble_vxc_SN + assemble_vxc_bond + their sum: writes vxc
int launch_vxc(const VxcArgs &v, cudaStream_t s);
// Dassemble_vxc_SN + Dassemble_vxc_bond (with the rho 2c derivatives): the
// pair forces and the three-center weights
int launch_dvxc_2c(const VxcArgs &v, cudaStream_t s);
// Dassemble_vxc_3c: accumulates onto f3a/b/c (cleared by the caller)
int launch_dvxc_3c(const VxcArgs &v, cudaStream_t s);
// the same in double-float on the FP32 pipe (s and sp bases)
int launch_dvxc_3c_df(const VxcArgs &v, cudaStream_t s);
// build_forces vxc terms: fvxc and ftot += fvxc + f3xca + f3xcb + f3xcc
int launch_vxc_forces(const VxcArgs &v, cudaStream_t s);

}  // namespace fb
