/*
 * fbgpu.h -- C ABI of the GB300 (sm_103a) FIREBALL Harris matrix-element
 * assembly library, libfbgpu.so.
 *
 * The library replaces, as a drop-in, the table-driven assembly path of the
 * reference (thunder-dft/thunder-master, Fortran):
 *
 *   module M_Fdata_2c / M_Fdata_3c   read_Fdata_2c / read_Fdata_3c
 *   module M_species                 read_info
 *   subroutine make_cells
 *   module M_neighbors               driver_neighbors (find_neighbors,
 *                                    find_common_neighbors)
 *   module M_assemble_2c             assemble_S, assemble_T, assemble_vna_2c
 *   module M_assemble_3c             assemble_vna_3c
 *   module M_Dassemble_2c            Dassemble_S, Dassemble_T, Dassemble_vna_2c
 *   module M_Dassemble_3c            Dassemble_vna_3c
 *   module M_build_forces            build_forces (the kinetic, vna, f3na and
 *                                    Pulay terms)
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (FB_OK = 0) and never aborts the process; fb_last_error() gives the text.
 * Where the reference would `stop`, the library returns the matching status.
 *
 * Data layout (identical to the Fortran per-neighbor block types):
 *   positions   ratom[3*i + k], Angstrom, i = 0..natoms-1
 *   species     imass[i], 1-based species number (order of nZ in
 *               fb_load_fdata, as in Fdata.inp)
 *   lattice     lattice[3*a + k] = component k of lattice vector a+1
 *   pairs       pair p = pair_off[i] + (ineigh-1), atoms in order, each
 *               atom's neighbors in the reference order (mbeta outer, jatom
 *               inner, c.SYSTEM/M_neighbors.f90:409-437)
 *   blocks      block of pair p at blk_off[p], column-major norb_i x norb_j:
 *               s%overlap(i)%neighbors(ineigh)%block(mu,nu) is
 *               S[blk_off[p] + (mu-1) + norb_i*(nu-1)]
 *   Dblocks     Dblock(ix,mu,nu) at 3*blk_off[p] + (ix-1) + 3*((mu-1) +
 *               norb_i*(nu-1))
 *   per-pair 3-vectors   vna_ontop(:,ineigh), vna_atom(:,ineigh) at 3*p
 *   per-atom 3-vectors   forces(i)%ftot(:) at 3*i
 * Neighbor indices returned to the caller are 1-based like the Fortran
 * arrays (neigh_j, neigh_back, neigh_self, iatom_common_j, jatom_common_j,
 * neigh_common); cell indices mbeta are 0-based as in the reference.
 *
 * Threading: one context per thread; calls on a context are ordered on its
 * CUDA stream and return after the work completes unless stated otherwise.
 */
#ifndef FBGPU_H
#define FBGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FB_OK 0
#define FB_ERR_ARG 1           /* bad argument */
#define FB_ERR_IO 2            /* Fdata file missing or unparsable */
#define FB_ERR_TABLE 3         /* interaction cell or ME map missing */
#define FB_ERR_X_NEGATIVE 4    /* getMEs: negative distance */
#define FB_ERR_X_TOO_LARGE 5   /* getMEs: x > xmax*(1+1e-5) */
#define FB_ERR_ATOMS_CLOSE 6   /* find_neighbors: two atoms < 0.5 A apart */
#define FB_ERR_NEIGH_SELF 7    /* neigh_self missing or found twice */
#define FB_ERR_NEIGH_BACK 8    /* neigh_back missing or found twice */
#define FB_ERR_CUDA 9          /* CUDA runtime error */
#define FB_ERR_WATCHDOG 10     /* a device wait ran out of its budget */
#define FB_ERR_STATE 11        /* call out of order (e.g. no neighbors yet) */
#define FB_ERR_CAPACITY 12     /* size beyond a stated maximum */
#define FB_ERR_UNSUPPORTED 13  /* basis or map this build does not handle */
#define FB_ERR_SOLVER 14       /* an eigen-decomposition did not converge */

/* assembly selection bits for fb_assemble / fb_dassemble */
#define FB_S 1u        /* overlap           (assemble_S / Dassemble_S) */
#define FB_T 2u        /* kinetic           (assemble_T / Dassemble_T) */
#define FB_VNA2C 4u    /* neutral atom 2c   (assemble_vna_2c / Dassemble_vna_2c) */
#define FB_VNA3C 8u    /* neutral atom 3c   (assemble_vna_3c / Dassemble_vna_3c) */
#define FB_ALL 15u
#define FB_KEEP_DBLOCKS 16u  /* fb_dassemble: also keep dS, dT Dblocks */
#define FB_FORCES 32u        /* fb_assemble_graph / fb_autotune: the force pass too */
#define FB_SVNL 128u         /* svnl blocks <basis i | projectors j> (assemble_svnl, M_assemble_PP_2c.f90:86) */
#define FB_VNL2C 256u        /* vnl 2c: atom, ontop left / right (assemble_vnl_2c, M_assemble_PP_2c.f90:232) */
#define FB_VNL3C 512u        /* vnl 3c (assemble_vnl_3c, M_assemble_PP_3c.f90:94); fb_dassemble: the vnl forces */
#define FB_EWALD 1024u       /* DOGS Ewald: the matrix (assemble_ewald) and the ewaldsr / ewaldlr blocks
                                (M_assemble_ewald_DOGS.f90:98, :404, :633); Harris: zero ewaldsr /
                                ewaldlr blocks and forces (M_assemble_ewald_Harris.f90:92-239) */
#define FB_VXC 2048u         /* McWEDA exchange-correlation, Harris (assemble_vxc,
                                M_assemble_vxc_McWEDA_Harris.f90:102): the input densities
                                (M_assemble_rho_McWEDA_Harris.f90) and the vxc blocks; reads the
                                overlap (FB_S in the same or an earlier call) */
#define FB_DIPOLE 64u        /* z-dipole blocks (assemble_dipole_z, M_assemble_2c_DOGS.f90:376-499);
                                with FB_THEORY_DOGS, FB_VNA2C computes them and FB_S as well */

/* block sets for fb_get_blocks / fb_device_blocks */
#define FB_BLOCK_S 0       /* s%overlap(i)%neighbors(k)%block */
#define FB_BLOCK_T 1       /* s%kinetic(i)%neighbors(k)%block */
#define FB_BLOCK_VNA 2     /* s%vna(i)%neighbors(k)%block  (atom + 3c) */
#define FB_BLOCK_VNAO 3    /* s%vna(i)%neighbors(k)%blocko (ontop L + R) */
#define FB_BLOCK_DS 4      /* s%overlap(i)%neighbors(k)%Dblock */
#define FB_BLOCK_DT 5      /* s%kinetic(i)%neighbors(k)%Dblock */
#define FB_BLOCK_RHO 6     /* s%denmat(i)%neighbors(k)%block (input) */
#define FB_BLOCK_CAPE 7    /* s%capemat(i)%neighbors(k)%block (input) */
#define FB_BLOCK_DIP 8     /* s%dipole_z(i)%neighbors(k)%block (FB_DIPOLE) */
#define FB_BLOCK_SVNL 9    /* s%svnl(i)%neighbors(k)%block over PP pairs, norb_i x norb_PP_j */
#define FB_BLOCK_VNL 10    /* s%vnl(i)%neighbors(k)%block over PPp pairs, norb_i x norb_j */
#define FB_BLOCK_DSVNL 11  /* s%svnl(i)%neighbors(k)%Dblock (after the vnl force pass) */
#define FB_BLOCK_RHO_PP 12 /* s%denmat_PP(i)%neighbors(k)%block (input, PPp pairs) */
#define FB_BLOCK_EWALDSR 13 /* s%ewaldsr(i)%neighbors(k)%block (FB_EWALD) */
#define FB_BLOCK_EWALDLR 14 /* s%ewaldlr(i)%neighbors(k)%block (FB_EWALD) */
#define FB_BLOCK_VXC 15       /* s%vxc(i)%neighbors(k)%block (FB_VXC) */
#define FB_BLOCK_RHO_IN 16    /* s%rho_in(i)%neighbors(k)%block (FB_VXC) */
#define FB_BLOCK_RHO_BOND 17  /* s%rho_bond(i)%neighbors(k)%block (FB_VXC) */
#define FB_BLOCK_WRHO_IN 18   /* s%rho_in_weighted(i)%neighbors(k)%block, nssh_i x nssh_j: 9 doubles
                                 per pair, (issh, jssh) at [9 p + issh + nssh_i jssh] (FB_VXC) */
#define FB_BLOCK_WRHO_BOND 19 /* s%rho_bond_weighted(i)%neighbors(k)%block, same layout (FB_VXC) */

/* force arrays for fb_get_forces */
#define FB_F_TOT 0         /* ftot: kinetic + vna + f3na(a+b+c) - pulay */
#define FB_F_KINETIC 1     /* forces(i)%kinetic */
#define FB_F_VNA 2         /* forces(i)%vna (atom + ontop pair sums) */
#define FB_F_PULAY 3       /* forces(i)%pulay */
#define FB_F_F3NAA 4       /* forces(i)%f3naa */
#define FB_F_F3NAB 5       /* forces(i)%f3nab */
#define FB_F_F3NAC 6       /* forces(i)%f3nac */
#define FB_F_VNA_ONTOP 7   /* forces(i)%vna_ontop(3, neighn), per pair */
#define FB_F_VNA_ATOM 8    /* forces(i)%vna_atom(3, neighn), per pair */
#define FB_F_VNL 9         /* forces(i)%vnl: the vnl atom and ontop pair sums */
#define FB_F_F3NLA 10      /* forces(i)%f3nla */
#define FB_F_F3NLB 11      /* forces(i)%f3nlb */
#define FB_F_F3NLC 12      /* forces(i)%f3nlc */
#define FB_F_VNL_ATOM 13   /* forces(i)%vnl_atom(3, neighn_PP), per PP pair */
#define FB_F_VNL_ONTOP 14  /* forces(i)%vnl_ontop(3, neighn_PPx), per PPx pair (ontop left) */
#define FB_F_EWALDSR 15    /* forces(i)%ewaldsr(3, neighn), per pair (DOGS, FB_EWALD) */
#define FB_F_EWALDLR 16    /* forces(i)%ewaldlr (DOGS, FB_EWALD) */
#define FB_F_EWALD 17      /* forces(i)%ewald, the Ewald energy force of Dassemble_ewald (DOGS, FB_EWALD) */
#define FB_F_VXC 18        /* forces(i)%vxc: the vxc_off_site + vxc_on_site pair sums (FB_VXC) */
#define FB_F_F3XCA 19      /* forces(i)%f3xca (FB_VXC) */
#define FB_F_F3XCB 20      /* forces(i)%f3xcb (FB_VXC) */
#define FB_F_F3XCC 21      /* forces(i)%f3xcc (FB_VXC) */
#define FB_F_VXC_OFF_SITE 22 /* forces(i)%vxc_off_site(3, neighn), per pair (FB_VXC) */
#define FB_F_VXC_ON_SITE 23  /* forces(i)%vxc_on_site(3, neighn), per pair (FB_VXC) */

typedef struct fb_ctx fb_ctx;

/* Create a context on CUDA device `device`.  Replaces the module state that
 * M_species, M_Fdata_2c/3c and the structure type hold in the reference. */
int fb_create(int device, fb_ctx **out);
void fb_destroy(fb_ctx *ctx);
const char *fb_last_error(const fb_ctx *ctx);
const char *fb_version(void);

/* Run the context's work on `stream` (a cudaStream_t, or NULL for the
 * context's own stream).  The caller keeps ownership of the stream. */
int fb_set_stream(fb_ctx *ctx, void *stream);

/* read_info (c.SYSTEM/M_species.f90:1057) + read_Fdata_2c
 * (e.FDATA/M_Fdata_2c.f90:149) + read_Fdata_3c (e.FDATA/M_Fdata_3c.f90:143):
 * parse the Fdata directory and stage every table in device memory.
 * nZ[k] is the atomic number of species k+1 (the Fdata.inp list). */
int fb_load_fdata(fb_ctx *ctx, const char *fdata_dir, int nspecies,
                  const int *nZ);
/* species layout after fb_load_fdata: norb_max of species isp (1-based) */
int fb_species_norb(const fb_ctx *ctx, int isp);

/* Structure: positions, species, lattice; make_cells
 * (c.SYSTEM/make_cells.f90:51).  icluster = 1 disables periodic images. */
int fb_set_structure(fb_ctx *ctx, int natoms, const double *ratom,
                     const int *imass, const double *lattice, int icluster);
/* Batch of independent structures (MD snapshots or unrelated
 * configurations of uneven size) assembled together.  No reference
 * counterpart: the reference handles one structure per process; each
 * structure here keeps the reference's per-structure semantics (its own
 * make_cells images, neighbor maps that never cross structures).
 * natoms[s] atoms of structure s follow one another in ratom (3 per atom)
 * and imass; lattice holds 9 doubles per structure (rows a1, a2, a3; may be
 * NULL when every structure is a cluster); icluster[s] = 1 marks a cluster
 * (NULL: all periodic).  fb_set_structure is the batch of one.  All later
 * calls act on the whole batch: block arrays, force arrays and pair lists
 * are the structures' arrays one after another, with the offsets of
 * fb_get_batch; atom numbers returned by fb_get_neighbors / fb_get_common
 * are 1-based within each structure, as the reference numbers them. */
int fb_set_batch(fb_ctx *ctx, int nstruct, const int *natoms,
                 const double *ratom, const int *imass, const double *lattice,
                 const int *icluster);
/* Per-structure offsets (nstruct + 1 entries each, 0-based, last = total):
 * first atom, first pair, first common-neighbor triplet and first block
 * element.  Any pointer may be NULL; pair, triplet and block offsets need
 * fb_neighbors first. */
int fb_get_batch(const fb_ctx *ctx, int *atom_off, int *pair_off,
                 int *trip_off, long long *block_off);
/* New positions for the same atoms (an MD step); neighbor maps must be
 * rebuilt by fb_neighbors before the next assembly. */
int fb_update_positions(fb_ctx *ctx, const double *ratom);

/* driver_neighbors (c.SYSTEM/M_neighbors.f90:93): find_neighbors,
 * neigh_self, neigh_back, find_common_neighbors, built on the GPU in the
 * reference order. */
int fb_neighbors(fb_ctx *ctx);
/* Adopt neighbor maps computed by the caller (e.g. read_NEIGHBORS,
 * M_neighbors.f90:171).  Arrays are 1-based as returned by
 * fb_get_neighbors; common-neighbor maps are rebuilt on the GPU. */
int fb_set_neighbors(fb_ctx *ctx, const int *neighn, const int *neigh_j,
                     const int *neigh_b);
int fb_get_sizes(const fb_ctx *ctx, int *npairs, int *ntriplets,
                 long long *nblock);
/* copy the maps out (any pointer may be NULL) */
int fb_get_neighbors(fb_ctx *ctx, int *neighn, int *neigh_j, int *neigh_b,
                     int *neigh_back, int *neigh_self, long long *blk_off);
int fb_get_common(fb_ctx *ctx, int *ncommon, int *iatom_common_j,
                  int *iatom_common_b, int *jatom_common_j,
                  int *jatom_common_b, int *neigh_common);

/* assemble_S/T/vna_2c (j.ASSEMBLERS/M_assemble_2c_Harris.f90:89,233,435)
 * and assemble_vna_3c (j.ASSEMBLERS/M_assemble_3c_Harris.f90:82), selected
 * by `what`.  Blocks stay in device memory until fetched. FB_VNA3C
 * accumulates onto the vna blocks, so it requires FB_VNA2C in the same call
 * or an earlier one (the reference's call order). */
int fb_assemble(fb_ctx *ctx, unsigned what);
/* copy one block set to the host (nblock doubles; 3*nblock for Dblocks) */
int fb_get_blocks(fb_ctx *ctx, int which, double *out);
/* device address of a block set (valid until the next fb_neighbors) */
int fb_device_blocks(fb_ctx *ctx, int which, void **dptr);

/* Density matrix and energy-weighted density matrix blocks (host, nblock
 * doubles each, layout as the blocks); cape may be NULL (zero Pulay). */
int fb_set_denmat(fb_ctx *ctx, const double *rho, const double *cape);

/* Same, from device memory (a GPU solver's output): device-to-device copy
 * on the context's stream; cape_dev may be NULL. */
int fb_set_denmat_device(fb_ctx *ctx, const void *rho_dev,
                         const void *cape_dev);

/* Dassemble_S/T/vna_2c (k.DASSEMBLERS/M_Dassemble_2c_Harris.f90:96,289,538),
 * Dassemble_vna_3c (k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136) and the
 * assembly terms of build_forces (c.SYSTEM/M_build_forces.f90:172). */
int fb_dassemble(fb_ctx *ctx, unsigned what);
/* copy one force array to the host (3*natoms, or 3*npairs for the per-pair
 * vna_ontop / vna_atom arrays) */
int fb_get_forces(fb_ctx *ctx, int which, double *out);

/* End-to-end H/S step through host buffers: upload positions, build the
 * neighbor maps, assemble S, T, vna (2c + 3c) and copy the four block sets
 * back.  Any output may be NULL. */
/* One step with forces through host buffers, the copies overlapped with the
 * kernels: upload the positions (ratom may be NULL: unchanged), build the
 * neighbor maps, then the value pass (assemble_S, assemble_T,
 * assemble_vna_2c/3c) while rho and cape (nblock doubles each, block layout
 * of the maps just built; cape may be NULL) travel on a copy stream, then the
 * force pass (Dassemble_S/T/vna_2c/vna_3c, build_forces) while S, T and vnao
 * travel back; vna and ftot (3*natoms) follow.  The two-center kernels run
 * on a second internal stream beside the common-neighbor search (unless
 * per-kernel timing is on or MLP-3c routes triplets); the call returns after
 * both internal streams and the context's stream are done.  Any output may
 * be NULL.  The
 * same results as fb_neighbors + fb_set_denmat + fb_assemble_graph(FB_ALL |
 * FB_FORCES) + fb_get_blocks + fb_get_forces; pinned host buffers let the
 * copies overlap.  Harris only.  Replaces one SCF/MD step's calls of
 * assemble_S/T/vna_2c/vna_3c (j.ASSEMBLERS/M_assemble_2c_Harris.f90:89-649,
 * M_assemble_3c_Harris.f90:82-227) and Dassemble_* + build_forces
 * (k.DASSEMBLERS/M_Dassemble_2c_Harris.f90:96-869,
 * M_Dassemble_3c_Harris.f90:136-408, c.SYSTEM/M_build_forces.f90:172-588). */
int fb_step_forces(fb_ctx *ctx, const double *ratom, const double *rho,
                   const double *cape, double *S, double *T, double *vna,
                   double *vnao, double *ftot);
int fb_assemble_step(fb_ctx *ctx, const double *ratom, double *S, double *T,
                     double *vna, double *vnao);

/* Value pass (what & FB_ALL) and, with FB_FORCES, the force pass of
 * fb_dassemble (same bits, FB_KEEP_DBLOCKS allowed) as ONE CUDA graph
 * launch on the context's stream.  The graph is captured on the first call
 * and replayed while the sizes (atoms, pairs, triplets, block elements),
 * device buffers, precision, launch shapes, stream and `what` stay the
 * same, so new positions and rebuilt neighbor maps of unchanged sizes reuse
 * it; anything else re-captures it.  For a batch (fb_set_batch) every kernel node is one launch over the
 * whole batch's concatenated pair or triplet list.  Results are the same as
 * fb_assemble(what & FB_ALL) followed by fb_dassemble(what).  The density
 * matrix must be set (fb_set_denmat / _device) before a call with
 * FB_FORCES; its contents may change between calls.  No reference
 * counterpart. */
int fb_assemble_graph(fb_ctx *ctx, unsigned what);

/* Launch shape of a tunable kernel ("assemble_2c", "assemble_3c",
 * "dassemble_2c", "dassemble_3c"): threads per CTA (32..256, a multiple of
 * 32), ctas_per_sm = 0 for a grid that covers the work (one triplet per
 * thread, one atom per warp), or > 0 for a persistent grid of
 * ctas_per_sm CTAs per SM whose warps take `chunk` groups of work (32
 * triplets, or one atom, per group) at a time from a device counter.  The
 * double-float three-center force kernels run at most 128 threads per CTA
 * (their register budget): a "dassemble_3c" shape of 256 threads runs them
 * with 128. */
int fb_set_launch(fb_ctx *ctx, const char *kernel, int threads,
                  int ctas_per_sm, int chunk);
int fb_get_launch(const fb_ctx *ctx, const char *kernel, int *threads,
                  int *ctas_per_sm, int *chunk);
/* Autotuner: times every candidate launch shape (covering grids of 64, 128
 * and 256 threads; persistent grids of 256..2048 threads per SM with chunks
 * of 1, 4 and 16) of the kernels `what` selects (FB_FORCES adds the force
 * kernels; they need the density matrix) on the current system with CUDA
 * events, `reps` launches per shape, and keeps the fastest.  best_ms (may be
 * NULL) receives 4 doubles: the best time per launch of assemble_2c,
 * assemble_3c, dassemble_2c, dassemble_3c (0 if not tuned).  The timed
 * launches overwrite the block and force arrays: assemble again before
 * reading them.  No reference counterpart. */
int fb_autotune(fb_ctx *ctx, unsigned what, int reps, double *best_ms);

/* ---- MLP-3c surrogate (no reference counterpart) ------------------------
 * A network that stands in for the three-center table interpolation of the
 * bcna integrals (getMEs_Fdata_3c, e.FDATA/M_Fdata_3c.f90:293-517): inputs
 * (2x/xmax - 1, 2y/ymax - 1, cos theta) of a triplet plus a 16-float
 * embedding of its species triple, three hidden layers of 128 with SiLU, 64
 * outputs of which output (itheta-1)*10 + ime (itheta = 1..5, ime = 0..9) is
 * the Legendre coefficient itheta of matrix element ime divided by its
 * scale (fb_mlp_scales).  BF16 weights and tensor-core inputs, FP32
 * accumulation.  Species triple index = (in1 * nspecies + in2) * nspecies +
 * indna, all 0-based.  The parameter vector (FP32) is laid out as
 * fb_mlp_layout describes: 10 offsets (embedding [ntriple][16], W1 [128][32],
 * b1, W2 [128][128], b2, W3, b3, W4 [64][128], b4 [64], end); W1 columns
 * 19..31 and W4 rows 50..63 are padding and stay zero. */
int fb_mlp_init(fb_ctx *ctx, unsigned long long seed);
long long fb_mlp_nparams(const fb_ctx *ctx);
int fb_mlp_layout(const fb_ctx *ctx, long long *offsets);
int fb_mlp_get_params(fb_ctx *ctx, float *out);
/* per-triple output scales, [ntriple][64] floats */
int fb_mlp_scales(fb_ctx *ctx, float *out);
/* Adam training on the GPU: nsamples points drawn uniformly over the table
 * domains (x in [0, xmax], y in [0, ymax], cos theta in [-1, 1], a species
 * triple with a table) and labelled by the FP64 table interpolator; `epochs`
 * passes in batches of `batch` (a multiple of 64), learning rate lr with
 * cosine decay; mean loss of each epoch into loss_per_epoch (may be NULL). */
int fb_mlp_train(fb_ctx *ctx, long long nsamples, int epochs, int batch,
                 double lr, unsigned long long seed, double *loss_per_epoch);
/* n training points as the trainer draws them: feat3 [n][3], triple [n],
 * normalized targets [n][64] */
int fb_mlp_samples(fb_ctx *ctx, int n, unsigned long long seed, float *feat3,
                   int *triple, float *target);
/* loss and gradient (FP32, the parameter layout) of one batch of n rows (a
 * multiple of 64): loss = sum (out - target)^2 / (50 n) over used outputs */
int fb_mlp_grad(fb_ctx *ctx, int n, const float *feat3, const int *triple,
                const float *target, float *grad, double *loss);
/* forward pass of n rows (a multiple of 64): normalized outputs [n][64] */
int fb_mlp_forward(fb_ctx *ctx, int n, const float *feat3, const int *triple,
                   float *out);
/* Validation against the FP64 table interpolator, per interpolation bin
 * (species triple x stencil node (ix, iy) of getMEs_Fdata_3c,
 * M_Fdata_3c.f90:367-376): the largest |network - tables| of a
 * Legendre-combined matrix element (table units, before the P_eq2 factor)
 * over samples_per_bin random points of the bin's region and random cos
 * theta.  max_err (may be NULL) receives the largest over all bins;
 * fb_mlp_bin_errors copies the per-bin values (out may be NULL to query
 * nbins). */
int fb_mlp_validate(fb_ctx *ctx, int samples_per_bin, unsigned long long seed,
                    double *max_err);
int fb_mlp_bin_errors(fb_ctx *ctx, float *out, long long *nbins);
/* Gate: a bin is given to the network only where its validated error keeps
 * every assembled vna block element of the current neighbor maps within
 * tol_ha Hartree in the worst case (all of a block's triplets erring the
 * same way): per-triplet bound tau = tol_ha * P_Hartree / (P_eq2 * 3 * n),
 * n the most triplets adding into one block.  Elsewhere the table path
 * runs.  Sets FB_MLP_GATED; tau (table units) and coverage (fraction of the
 * current triplets given to the network) may be NULL. */
int fb_mlp_gate(fb_ctx *ctx, double tol_ha, double *tau, double *coverage);
/* FB_MLP_OFF: tables only.  FB_MLP_GATED: approved bins through the
 * network (fb_mlp_gate).  FB_MLP_ALL: every three-center triplet through
 * the network, ungated (to measure the surrogate alone).  Applies to the
 * value and force passes of fb_assemble, fb_dassemble and
 * fb_assemble_graph; the network's results enter the same double-float
 * rotation and density contraction as the table values. */
#define FB_MLP_OFF 0
#define FB_MLP_GATED 1
#define FB_MLP_ALL 2
int fb_mlp_set_mode(fb_ctx *ctx, int mode);
/* The assembly's network evaluation at given points (n rows of pts =
 * (x, y, cos theta), x the neutral-atom and y the bond-charge distance in
 * Angstrom, and a species triple each): Legendre-combined matrix elements
 * out[n][10] (before the sin(theta) factor of the mvalue = 1 elements), or
 * with derivs out[n][4][10] = value, d/dcos, d/dx, d/dy. */
int fb_mlp_eval_points(fb_ctx *ctx, int n, const float *pts, const int *triple,
                       int derivs, float *out);
/* Tensor-core engine of the network evaluation in the assembly:
 * FB_MLP_ENGINE_MMA (warp-level mma.sync BF16) or FB_MLP_ENGINE_TC (tcgen05
 * UMMA with TMEM accumulators, one thread per triplet; the default).  Same
 * contract and results up to FP32 summation order. */
#define FB_MLP_ENGINE_MMA 0
#define FB_MLP_ENGINE_TC 1
int fb_mlp_set_engine(fb_ctx *ctx, int engine);
/* triplets the network takes in the current mode, and all triplets */
int fb_mlp_routed(const fb_ctx *ctx, int *n_mlp, int *n_total);

/* Bloch sums, the step after the assembly (h.SOLVESH/M_kspace_Lowdin.f90:
 * 680-708 for S, :796-853 for H): dense complex matrices
 *   M(jmu, jnu) = sum over pairs of phase(k . (xl(mbeta) + r_j - r_i)) *
 *                 block(imu, inu),  phase(dot) = cos(dot) + i sin(dot),
 * jmu / jnu the orbital's position in the structure (iblock_slot order),
 * for H the T + vna + vnao blocks (the Harris terms of build_Hmatrix,
 * :253-255) and for S the overlap blocks, one norbitals x norbitals
 * column-major complex matrix (re, im interleaved) per k-point (kpts: 3
 * doubles each, 1/Angstrom).  fb_bloch_device writes into device buffers
 * (either may be NULL) and adds extra_dev (NULL, or nblock doubles on the
 * device: the caller's other H terms, e.g. vxc) to H; fb_bloch copies to
 * host buffers.  Needs fb_assemble of the blocks; single structures. */
long long fb_norbitals(const fb_ctx *ctx);
int fb_bloch_device(fb_ctx *ctx, int nk, const double *kpts,
                    const void *extra_dev, void *Hk_dev, void *Sk_dev);
int fb_bloch(fb_ctx *ctx, int nk, const double *kpts, double *Hk, double *Sk);

/* k-point Lowdin solver after the Bloch sums.  Replaces kspace_Lowdin
 * (h.SOLVESH/M_kspace_Lowdin.f90:740-880) with diagonalize_S and
 * diagonalize_H_Lowdin (h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:
 * 145-403).  Per k-point (kpts: 3 doubles each, 1/Angstrom): the Bloch sums
 * S(k) and H(k) = T + vna + vnao (+ extra_dev, as fb_bloch_device) on the
 * device, the eigenpairs of S(k), the reference's linear-dependence rule
 * (overlap eigenvalues below 1e-4: the columns above them move down, the
 * trailing columns keep theirs), S^-1/2 from lambda^(-1/4)-scaled columns,
 * the eigenpairs of S^-1/2 H S^-1/2 and c = S^-1/2 c_Lowdin.
 *   eigen    host, nk * norbitals doubles: band energies, ascending (eV)
 *   c_dev    device or NULL: nk column-major norbitals x norbitals complex
 *            matrices (re, im interleaved), the eigenvectors c (the
 *            reference's s%kpoints(ik)%c)
 *   dropped  host or NULL: per k-point the number of overlap eigenvalues
 *            below 1e-4 (norbitals - norbitals_new)
 * The eigen-decompositions are cuSOLVER zheevd and the products cuBLAS
 * zgemm, opened at the first call (FB_ERR_UNSUPPORTED where absent); the
 * reference stops where zheev fails, this returns FB_ERR_SOLVER; it also
 * returns FB_ERR_SOLVER where more than half of the overlap eigenvalues
 * fall below 1e-4, where the reference's column shift leaves eigenvalues
 * below 1e-4 (negative ones among them) in S^-1/2 and its result is NaN.  Works in
 * four norbitals^2 complex device matrices the context keeps. */
int fb_solve_k(fb_ctx *ctx, int nk, const double *kpts, const void *extra_dev,
               double *eigen, void *c_dev, int *dropped);

/* Non-local pseudopotential (vnl).  fb_neighbors_pp replaces
 * driver_neighbors_PP (c.SYSTEM/M_neighbors_PP.f90:98-151): the PP map
 * (basis of i within rcA_i + rc_PP_j - 0.01 of the projectors of j), the PPx
 * map (projectors of i, basis of j), the PPp map (atoms sharing a projector
 * atom, in the reference's first-occurrence order) with the PP and PPx maps
 * into it and the PPx points into PP(j), and the PP common-neighbor triplets
 * (find_common_neighbors_PP with mpairnay's svnl indices).  Needs Fdata with
 * the vnl tables (interaction 6) and projector shells of s, sp or spd; single
 * structures.  fb_assemble with FB_SVNL / FB_VNL2C / FB_VNL3C assembles
 * svnl over PP pairs and vnl over PPp pairs; fb_set_denmat_pp gives
 * s%denmat_PP (PPp layout, FB_BLOCK_RHO_PP) and fb_dassemble with FB_VNL2C /
 * FB_VNL3C computes Dassemble_svnl, Dassemble_vnl_2c (vnl_atom, vnl_ontop;
 * the reference leaves the ontop-right force out, M_Dassemble_PP_2c.f90:
 * 737-738, and build_forces doubles the left one), Dassemble_vnl_3c
 * (f3nla/b/c) and the vnl terms of build_forces (M_build_forces.f90:395-461),
 * added into FB_F_TOT.  The maps are returned 1-based as the reference
 * numbers them: which = FB_PP_MAP (neighn, neigh_j, neigh_b, self, map into
 * PPp), FB_PPX_MAP (also point into PP(j)) or FB_PPP_MAP (no map / point). */
#define FB_PP_MAP 0
#define FB_PPX_MAP 1
#define FB_PPP_MAP 2
int fb_neighbors_pp(fb_ctx *ctx);
int fb_get_pp_sizes(fb_ctx *ctx, int *npp, int *nppx, int *nppp, int *ntrip,
                    long long *nsvnl, long long *nvnl);
int fb_get_pp_neighbors(fb_ctx *ctx, int which, int *neighn, int *neigh_j,
                        int *neigh_b, int *self, int *map, int *point);
int fb_get_pp_common(fb_ctx *ctx, int *ncommon, int *iatom_common_j,
                     int *iatom_common_b, int *jatom_common_j,
                     int *jatom_common_b, int *neigh_common, int *m31,
                     int *m32);
int fb_set_denmat_pp(fb_ctx *ctx, const double *rho_pp);
int fb_set_denmat_pp_device(fb_ctx *ctx, const void *rho_pp_dev);

/* Theory of the neutral-atom terms.  FB_THEORY_HARRIS (the default):
 * assemble_vna_2c / assemble_vna_3c of the Harris functional
 * (M_assemble_2c_Harris.f90, M_assemble_3c_Harris.f90).  FB_THEORY_DOGS:
 * the charge-weighted versions (j.ASSEMBLERS/M_assemble_2c_DOGS.f90:640-814,
 * M_assemble_3c_DOGS.f90:158-322): the vna ontop and atom terms add the
 * charged-shell sub-cells isorp = 1..nssh weighted by the shell charges
 * dQ = Qin - Qneutral, the atom and three-center terms smoothed into the
 * effective monopole of the overlap and z-dipole blocks.  DOGS needs Fdata
 * with the sub-cells and dipole_z tables (FB_ERR_TABLE otherwise) and
 * fb_set_charges; it runs the FP64 kernels and the tables only (no MLP-3c
 * routing).  fb_dassemble then computes the DOGS force pass
 * (k.DASSEMBLERS/M_Dassemble_2c_DOGS.f90:679-1199, M_Dassemble_3c_DOGS.f90:
 * 136-520): the charged ontop and atom derivatives with the smoother and
 * monopole terms, and the charged three-center terms from the overlap and
 * z-dipole blocks and their derivatives, into the same force arrays as
 * Harris (vna_ontop, vna_atom, f3na*, ftot).  fb_dassemble_noalloc stays
 * Harris-only (FB_ERR_UNSUPPORTED in DOGS). */
#define FB_THEORY_HARRIS 0
#define FB_THEORY_DOGS 1
int fb_set_theory(fb_ctx *ctx, int theory);

/* Shell charges of the DOGS terms, dq[i * nssh_max + k] = Qin(k+1, i+1) -
 * Qneutral(k+1, imass(i+1)), a row per atom (entries beyond the species'
 * nssh are ignored; nssh_max <= 3).  Stands for the reference's
 * s%atom(i)%shell(k)%dQ (M_assemble_2c_DOGS.f90:662, :806,
 * M_assemble_3c_DOGS.f90:313). */
int fb_set_charges(fb_ctx *ctx, const double *dq, int nssh_max);

/* The DOGS Ewald terms (j.ASSEMBLERS/M_assemble_ewald_DOGS.f90), assembled
 * with FB_EWALD in DOGS after (or with) FB_VNA2C: the long-range Coulomb
 * matrix s%ewald(i, j) of assemble_ewald (:633-918; reciprocal sum over the
 * reference's g box, erfc-screened lattice sum, -2 kappa/sqrt(pi) on the
 * diagonal; a cluster keeps only the bare 1/z of its own cell), the
 * short-range correction s%ewaldsr (:98-378: atom, ontop and three-center
 * terms from the overlap and z-dipole blocks and the atoms' total charges)
 * and the long-range blocks s%ewaldlr (:404-592, with sum_ewald = ewald dQ).
 * Single structures.  fb_get_ewald copies the N x N matrix (row-major).
 * fb_dassemble with FB_EWALD (after FB_EWALD was assembled, or in one
 * fb_assemble_graph with it) computes the force pass of
 * k.DASSEMBLERS/M_Dassemble_ewald_DOGS.f90: dewald and the Ewald energy
 * force FB_F_EWALD (Dassemble_ewald, :878-1236), the ewaldsr pair forces
 * FB_F_EWALDSR with their three-center terms added into f3na (:94-527),
 * the ewaldlr atom forces FB_F_EWALDLR (:553-837), and the build_forces
 * terms (ftot -= ewaldsr on i, += on j, += ewaldlr; M_build_forces.f90:
 * 367-386) added into FB_F_TOT.  dewald is 3 N^2 doubles. */
int fb_get_ewald(fb_ctx *ctx, double *ewald);

/* Arithmetic of the three-center kernels.  FB_PREC_DF (the default): the
 * table contractions, rotations, frame derivatives and density contractions
 * run in double-float arithmetic on the FP32 pipe (two floats per value,
 * 48-bit significand), while every grid-cell, stencil, cutoff and
 * interpolation-branch decision is still made in FP64 exactly as the
 * reference makes it; GB300 executes FP64 at 1/64 of its FP32 rate.
 * FB_PREC_FP64: every operation in FP64.  Systems with d shells always use
 * FP64.  No reference counterpart (the reference computes in FP64). */
#define FB_PREC_FP64 0
#define FB_PREC_DF 1
int fb_set_precision(fb_ctx *ctx, int mode);

/* Number of kernels this context launched since creation (diagnostics). */
long long fb_kernel_launches(const fb_ctx *ctx);

/* Per-kernel timing with CUDA events recorded on the context's stream
 * around every launch.  fb_set_timing(ctx, 1) resets and enables it;
 * fb_get_timing returns the accumulated device time and launch count of one
 * kernel: "neigh_count", "neigh_fill", "neigh_back", "common_count",
 * "common_fill", "assemble_2c", "assemble_3c", "dassemble_2c",
 * "dassemble_3c", "build_forces", "trip_bins", "split_rho", "mlp_eval",
 * "assemble_3c_mlp", "dassemble_3c_mlp", "bloch", "pp_pairs", "ppp", "pp_common",
 * "svnl", "vnl_2c", "vnl_3c", "dsvnl", "dvnl_2c", "dvnl_3c", "vnl_forces", "ewald",
 * "ewald_blocks", "rho_2c", "rho_3c", "vxc", "dvxc_2c", "dvxc_3c",
 * "vxc_forces".  No reference counterpart (the reference
 * has no timers on this path). */
int fb_set_timing(fb_ctx *ctx, int enable);
int fb_get_timing(fb_ctx *ctx, const char *kernel, double *total_ms,
                  long long *launches);

/* Allocation-free force pass.  No counterpart in the reference: it exists
 * for callers that cannot allocate GPU memory while they run the force pass,
 * for example a driver that hands the whole GPU to a pre-sized memory pool,
 * or an MD loop that must not call the CUDA allocator between steps (an
 * allocation synchronizes the device and can fail once memory fragments).
 *
 * Computes the Harris forces that fb_dassemble(ctx, FB_ALL) +
 * fb_get_forces(ctx, FB_F_TOT) compute, for the structure and neighbor maps
 * already on the context, from the density matrices passed here (not the
 * ones fb_set_denmat stored on the context):
 *   rho_dev, cape_dev  device pointers, nblock doubles each, block layout;
 *                      cape_dev may be NULL (no Pulay term)
 *   ftot_dev           device pointer, 3*natoms doubles, written
 * It always runs the FP64 three-center kernel from the tables, whatever
 * fb_set_precision and the MLP-3c mode say (on GB300 that kernel is about
 * 2.7x slower than the double-float one that fb_dassemble runs by default).
 * The call makes no cudaMalloc, cudaFree or other allocating call.  Its
 * intermediate per-pair and per-atom terms live in one statically sized
 * device array of the library, which every GPU that loads the library holds
 * until the process exits (8.25 MiB); systems with more than
 * FB_NOALLOC_MAX_PAIRS pairs or FB_NOALLOC_MAX_ATOMS atoms are rejected with
 * FB_ERR_CAPACITY.  fb_create looks up that array's device address for its
 * device, so the module that holds the array is loaded then, not inside
 * this call.  All calls share the array and it keeps the last call's
 * contents (the call clears what it accumulates), so calls that overlap on
 * the GPU (two streams, two contexts on one device) race and must be
 * serialized by the caller.  Returns after the work completes. */
#define FB_NOALLOC_MAX_PAIRS 65536
#define FB_NOALLOC_MAX_ATOMS 16384
int fb_dassemble_noalloc(fb_ctx *ctx, const double *rho_dev,
                         const double *cape_dev, double *ftot_dev);

/* Measured FP64 FMA throughput of this GPU in TFLOP/s (a DFMA-chain kernel,
 * about 0.1 s); the denominator of the FP64 roofline.  No reference
 * counterpart. */
int fb_probe_fp64(fb_ctx *ctx, double *tflops);
/* Measured FP32 FMA throughput in TFLOP/s (FFMA chains); the denominator of
 * the FP32-pipe roofline of the double-float kernels.  No reference
 * counterpart. */
int fb_probe_fp32(fb_ctx *ctx, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
