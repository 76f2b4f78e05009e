// fb_launch.h -- kernel launchers of libfbgpu and their argument blocks.
#pragma once
#include <cuda_runtime.h>
#include "fb_internal.h"

// A source whose template instantiations take long to compile is built in
// parts: the build compiles it once per part with -DFB_PART=k, and part k
// holds only the launchers marked FB_IN_PART(k), so the parts compile in
// parallel.  Compiled without FB_PART, a source holds every part.
#ifdef FB_PART
#define FB_IN_PART(k) (FB_PART == (k))
#else
#define FB_IN_PART(k) 1
#endif

namespace fb {

// Launch shape of one kernel: threads per CTA; ctas_per_sm > 0 selects the
// persistent form (nsm * ctas_per_sm CTAs whose warps take `chunk` task
// groups per grab from a device counter), 0 a grid that covers the work.
struct KCfg {
  int threads, ctas_per_sm, chunk, nsm;
};
// device side of a launch: the work counter (null: grid covers the work)
struct Sched {
  int *ctr;
  int chunk;
};

// A batch of structures is one concatenated system: atoms of structure s
// are satom_off[s] .. satom_off[s+1]-1, sid[atom] = s, and structure s owns
// XL_STRIDE doubles of image vectors at xl + s * XL_STRIDE.
struct NeighArgs {
  int N, P;
  const double *ratom;
  const float4 *pos4;     // x, y, z, float cutoff of the atom's species
  const int *sid;         // structure of each atom
  const int *satom_off;   // first atom of each structure (+ end)
  const int *simg_off;    // images of structure s: imgs[simg_off[s] .. simg_off[s+1]-1]
  const float4 *sbbox;    // bounding box (lo, hi) of each structure's positions
  const float4 *cbox;     // bounding box (lo, hi) of each chunk of 32 consecutive atoms
  const int *cb_off;      // first chunk of each structure
  const int *speriodic;   // 1 for a periodic structure, 0 for a cluster
  float rcmax;            // largest species cutoff
  const int *isp;
  const FdataDev *fd;
  const double *xl;
  const float *xlf;
  const int *imgs;
  // per atom and image (from img_off[s] + (i - first atom of s) * images of
  // s): the image's first slot in i's list and its norb start, written by the
  // count pass for the fill pass
  const long long *img_off;
  int *img_start;
  long long *img_orb;
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
  float4 *r3f;  // float r3v with the neighbor's species cutoff in .w
  int *tcnt;
  int *rcnt;  // kept (ineigh, jneigh) pairs of each pair row (ialpha, ineigh)
  const int *trip_off;
  int *ci_j, *ci_b, *cj_j, *cj_b, *cneigh, *tdst;
  // common-neighbor slots: ialpha's kept (ineigh, jneigh) pairs and matches
  const long long *slot_off;
  unsigned *slot_nn;
  int *slot_found;
  unsigned *status;
  int *errinfo;
};

struct AsmArgs {
  int N, ntrip, have_d;
  int P;                   // pairs (neighbor blocks)
  const int *pair_owner;   // atom of each pair
  const double *ratom;
  const int *sid;  // structure of each atom (image vectors at xl + sid * XL_STRIDE)
  const int *isp;
  const FdataDev *fd;
  const double *table2c, *table3c, *gxy;
  const unsigned char *lin;
  const double *xl;
  const int *pair_off, *neigh_j, *neigh_b, *neigh_self, *neigh_back;
  const long long *blk_off;
  const int *trip_alpha, *ci_j, *ci_b, *cj_j, *cj_b, *tdst;
  const int *tperm;  // triplet processing order (binned), or null
  // force pass: the three-center kernel also adds the value-pass vna terms
  // of its triplets (a step that computes both interpolates each once)
  int fuse_value;
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
  // MLP-3c: per list position, the network's values (and derivatives)
  const float *mlpF;
  // DOGS (charge-weighted neutral atom): shell charges [atom][MAXSUB], z-dipole blocks
  int dogs;
  const double *dq;
  double *dip;
  // DOGS force pass: per pair sum(rho S), sum(rho dip), sum(rho dS)[3],
  // sum(rho ddip)[3] (8 doubles), written by the 2c and read by the 3c kernel
  double *dogs_ps;
  // launch shapes (autotuned) and the work counters of persistent launches
  KCfg cfg_a2c, cfg_a3c, cfg_d2c, cfg_d3c;
  int *queue;  // 4 counters: assemble_2c, assemble_3c, dassemble_2c, dassemble_3c
};

int launch_neigh(const NeighArgs &a, bool fill, cudaStream_t s);
int launch_neigh_back(const NeighArgs &a, cudaStream_t s);
// common neighbors: the search into per-ialpha slots (+ counts), then the
// compaction into the CSR triplet lists at trip_off
int launch_common(const NeighArgs &a, cudaStream_t s);
int launch_common_compact(const NeighArgs &a, cudaStream_t s);
// counting sort of the triplets by (species triple, 3c grid cell) -> perm;
// bins with binok[bin] set (may be null) come first; hist has 2 x nbins
// entries and holds the exclusive bin starts afterwards; binned (may be
// null): 6 x T ints, the triplet lists copied into the binned order
int launch_trip_bins(const NeighArgs &a, int T, int nsp, int cells, const unsigned char *binok, int *key, int *rank,
                     int *hist, int *perm, int *binned, cudaStream_t s);
int launch_assemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s);
int launch_assemble_3c(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_2c(const AsmArgs &a, unsigned what, cudaStream_t s);
int launch_dassemble_3c(const AsmArgs &a, cudaStream_t s);
int launch_build_forces(const AsmArgs &a, unsigned what, cudaStream_t s);
// double-float three-center kernels (s and sp bases) and the rho split
int launch_assemble_3c_df(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_3c_df(const AsmArgs &a, cudaStream_t s);
// DOGS three-center value and force kernels in double-float (s and sp bases)
int launch_assemble_3c_dogs_df(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_3c_dogs_df(const AsmArgs &a, cudaStream_t s);
int launch_split_rho(const AsmArgs &a, long long nblock, cudaStream_t s);
// three-center kernels fed by MLP-3c results (a.mlpF) instead of the tables:
// list positions 0 .. a.ntrip-1 of a.tperm
int launch_assemble_3c_mlp(const AsmArgs &a, cudaStream_t s);
int launch_dassemble_3c_mlp(const AsmArgs &a, cudaStream_t s);
struct MlpEvalArgs;
int launch_mlp_eval(const MlpEvalArgs &m, const AsmArgs &a, bool tangents, int nsm, cudaStream_t s);
// the same on the tcgen05 tensor cores (TMEM accumulators)
int launch_mlp_tc(const MlpEvalArgs &m, const AsmArgs &a, bool tangents, int nsm, cudaStream_t s);
// the network's inputs (x, y, cos; species triple) per list position in float
int launch_mlp_points(const MlpEvalArgs &m, const AsmArgs &a, const float4 *pos4, const float *xlf, float *pts,
                      int *ptrip, cudaStream_t s);
// Bloch sums of up to three block sets (B, C may be null) into nk dense
// complex n x n matrices at out (column-major, re/im interleaved)
int launch_bloch(const AsmArgs &a, int P, int nk, const double *kpts, const int *pair_owner, const double *r3v,
                 const int *slot, long long n, const double *A, const double *B, const double *C, double *out,
                 cudaStream_t s);
// DFMA throughput probe: one warm-up and one timed launch
int probe_dfma(cudaStream_t s, double *ms, double *flops);
int probe_ffma(cudaStream_t s, double *ms, double *flops);

}  // namespace fb
