// fb_api.cu -- context, memory and the C ABI of libfbgpu (include/fbgpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fbgpu.h"
#include "fb_fdata.h"
#include "fb_launch.h"
#include "fb_pp.h"
#include "fb_ewald.h"
#include "fb_vxc.h"
#include "fb_devbuf.h"
#include "fb_mlp.h"
#include "fb_solve.h"

using namespace fb;

namespace fb {
std::atomic<long long> g_alloc_gen{0};
}

// kernels timed by fb_set_timing / fb_get_timing
enum { KT_NEIGH_COUNT, KT_NEIGH_FILL, KT_NEIGH_BACK, KT_COMMON_COUNT, KT_COMMON_FILL, KT_ASM2C, KT_ASM3C,
       KT_DASM2C, KT_DASM3C, KT_FORCES, KT_TRIP_BINS, KT_SPLIT_RHO, KT_MLP_EVAL, KT_ASM3C_MLP, KT_DASM3C_MLP,
       KT_BLOCH, KT_PP_PAIRS, KT_PPP, KT_PPC, KT_SVNL, KT_VNL2C, KT_VNL3C, KT_DSVNL, KT_DVNL2C, KT_DVNL3C,
       KT_VNLF, KT_EWALD, KT_EWALD_BLOCKS, KT_RHO2C, KT_RHO3C, KT_VXC, KT_DVXC2C, KT_DVXC3C, KT_VXCF, KT_N };
static const char *kt_names[KT_N] = {"neigh_count", "neigh_fill", "neigh_back", "common_count", "common_fill",
                                     "assemble_2c", "assemble_3c", "dassemble_2c", "dassemble_3c",
                                     "build_forces", "trip_bins", "split_rho", "mlp_eval", "assemble_3c_mlp",
                                     "dassemble_3c_mlp", "bloch", "pp_pairs", "ppp", "pp_common", "svnl",
                                     "vnl_2c", "vnl_3c", "dsvnl", "dvnl_2c", "dvnl_3c", "vnl_forces", "ewald",
                                     "ewald_blocks", "rho_2c", "rho_3c", "vxc", "dvxc_2c", "dvxc_3c",
                                     "vxc_forces"};
// kernels with a tunable launch shape
enum { TK_A2C, TK_A3C, TK_D2C, TK_D3C, TK_N };
static const char *tk_names[TK_N] = {"assemble_2c", "assemble_3c", "dassemble_2c", "dassemble_3c"};

struct fb_ctx {
  int device = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  // fb_step_forces: a copy stream and its events (host <-> device copies
  // overlapped with the kernels)
  cudaStream_t cstream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_val = nullptr, ev_frc = nullptr;
  // and a second kernel stream: the two-center kernels run on it while the
  // common-neighbor stage runs on the main stream
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_nb = nullptr, ev_2c = nullptr;
  // set while a graph of a value + force pass is captured: the force pass's
  // three-center table kernel also adds the value-pass vna terms, and the
  // value pass skips its three-center table kernel
  bool fuse3c = false;
  std::string err;
  long long launches = 0;
  // Fdata
  bool have_fdata = false;
  FdataHost fdh;
  DevBuf d_fd, d_tab2, d_tab3, d_tab3df, d_lin, d_gxy;
  int prec = FB_PREC_DF;
  // structure
  // structures: a batch of nstruct concatenated systems (one structure is a
  // batch of one); structure s holds atoms h_satom_off[s] .. h_satom_off[s+1]-1
  int N = 0, nstruct = 0;
  std::vector<int> h_satom_off, h_sid, h_icl, h_simg_off, h_isp, h_imgs;
  std::vector<long long> h_img_off;  // per structure: first (atom, image) entry of d_img_start / d_img_orb
  std::vector<double> h_lat;   // 9 per structure, rows a1, a2, a3
  std::vector<double> h_xl;    // XL_STRIDE per structure
  std::vector<float4> h_sbbox; // lo, hi per structure
  std::vector<float4> h_cbox;  // lo, hi per chunk of 32 consecutive atoms of a structure
  std::vector<int> h_cb_off;   // first chunk of each structure
  float rcmax = 0.0f;
  DevBuf d_ratom, d_pos4, d_isp, d_xl, d_xlf, d_imgs, d_sid, d_satom_off, d_simg_off, d_sbbox, d_speriodic;
  DevBuf d_img_off, d_img_start, d_img_orb;
  DevBuf d_cbox, d_cb_off;
  // neighbors
  bool have_neigh = false;
  int P = 0, T = 0;
  long long nblock = 0;
  std::vector<int> h_pair_off, h_trip_off;
  std::vector<long long> h_blk_base;  // first block element of each atom's pairs (+ total)
  DevBuf d_bsum, d_blk_base;
  DevBuf d_cnt, d_pair_off, d_neigh_j, d_neigh_b, d_neigh_self, d_neigh_back, d_pair_owner, d_r3v, d_r3f,
      d_blk_off, d_tcnt, d_trip_off, d_ci_j, d_ci_b, d_cj_j, d_cj_b, d_cneigh, d_tdst, d_talpha;
  DevBuf d_tkey, d_trank, d_tperm, d_thist;
  // the triplet lists in the binned order (6 x T ints) for the table
  // kernels, valid for tbin_T triplets
  DevBuf d_tbin;
  DevBuf d_mlp_pts, d_mlp_ptrip;  // network inputs per routed triplet (tensor-core engine)
  int tbin_T = -1;
  DevBuf d_slot_off, d_slot_nn, d_slot_found, d_rcnt;
  DevBuf d_orb_slot;  // first orbital of each atom (iblock_slot)
  // k-point Lowdin solver (fb_solve_k): handles and n x n work matrices
  SolverHandles solver;
  DevBuf d_sol_S, d_sol_H, d_sol_W, d_sol_T, d_sol_lam, d_sol_eps, d_sol_work, d_sol_info;
  DevBuf d_status, d_errinfo;
  // blocks
  DevBuf d_S, d_T, d_vb, d_vbo, d_rho, d_cape, d_dS, d_dT, d_rho_df, d_dip;
  // theory of the neutral-atom terms (FB_THEORY_HARRIS / FB_THEORY_DOGS) and
  // the DOGS shell charges dq[atom][MAXSUB]
  int theory = FB_THEORY_HARRIS;
  DevBuf d_dq, d_dogs_ps;
  // non-local pseudopotential: maps (driver_neighbors_PP), blocks, forces
  bool have_pp_neigh = false, have_rho_pp = false;
  int npp = 0, nppx = 0, nppp = 0, ntrip_pp = 0;
  long long nsvnl = 0, nvnl = 0;
  std::vector<int> h_pp_off, h_ppx_off, h_ppp_off, h_ppc_off;
  std::vector<long long> h_svnl_base, h_vnl_base;
  DevBuf d_pp_cnt, d_pp_off, d_pp_j, d_pp_b, d_pp_self, d_pp_map, d_svnl_sum, d_svnl_base, d_svnl_off;
  DevBuf d_ppx_cnt, d_ppx_off, d_ppx_j, d_ppx_b, d_ppx_self, d_ppx_map, d_ppx_point;
  DevBuf d_ub, d_pslot_off, d_pslot_j, d_pslot_b, d_ppp_cnt, d_vnl_sum, d_ppp_off, d_vnl_base, d_ppp_j, d_ppp_b,
      d_ppp_self, d_vnl_off;
  DevBuf d_ppc_cnt, d_ppc_off, d_t_alpha, d_t_i, d_t_ib, d_t_j, d_t_jb, d_t_m, d_t_m31, d_t_m32;
  DevBuf d_svnl, d_dsvnl, d_vnl, d_rho_pp, d_vnl_atom, d_vnl_ontop, d_f3nla, d_f3nlb, d_f3nlc, d_fvnl;
  // DOGS Ewald: the N x N matrix, its g / L lists, atom charges, sr / lr blocks
  bool have_ewald = false;
  bool ewald_matrix = false;  // the DOGS Ewald matrix (Harris assembles zero blocks only)
  int ew_ng = 0, ew_nl = 0;
  double ew_kappa = 0.0;
  DevBuf d_ewald, d_ew_g, d_ew_stuff, d_ew_l, d_dqa, d_sum_ewald, d_ewsr, d_ewlr, d_ew_sfc, d_ew_sfs, d_ew_ldf;
  DevBuf d_q0a, d_dewald, d_ew_w, d_sum_dewald, d_ew_cw, d_fewald, d_fsr, d_flr;
  // McWEDA exchange-correlation (Harris): input densities and vxc blocks
  DevBuf d_rho_in, d_rho_bond, d_wrho_in, d_wrho_bond, d_vxc;
  DevBuf d_vxc_off, d_vxc_on, d_vxc_wd, d_vxc_gd, d_f3xa, d_f3xb, d_f3xc, d_fvxc;
  bool have_charges = false, have_dip = false;
  bool have_vna2c = false, have_rho = false, have_cape = false, have_dblocks = false;
  unsigned assembled = 0, dassembled = 0;
  // forces
  DevBuf d_sumT, d_sumS, d_ontop, d_atomf, d_f3a, d_f3b, d_f3c, d_kin, d_vna, d_pul, d_ftot;
  // launch shapes of the tunable kernels and their persistent work counters
  int nsm = 0;
  KCfg cfg[TK_N];
  DevBuf d_queue;
  // CUDA graph of assembly + force pass (fb_assemble_graph).  Its kernel
  // arguments hold device pointers and the sizes N, P, T, nblock; it stays
  // valid while none of them changes (new positions and rebuilt neighbor
  // maps of the same sizes reuse it).
  cudaGraphExec_t gexec = nullptr;
  unsigned g_what = 0;
  int g_npp = -1, g_nppx = -1, g_nppp = -1, g_ntrip_pp = -1;
  int g_theory = -1, g_prec = -1, g_N = -1, g_P = -1, g_T = -1, g_have_d = -1, g_mlp_n = -1, g_mlp_mode = -1, g_mlp_engine = -1;
  long long g_nblock = -1, g_alloc = -1, g_launches = 0;
  cudaStream_t g_stream = nullptr;
  KCfg g_cfg[TK_N];
  // MLP-3c surrogate: mode, per-bin validation errors and approval, the
  // number of triplets routed to the network (the first mlp_n of tperm)
  MlpState mlp;
  int mlp_mode = FB_MLP_OFF;
  int mlp_cells = 0;
  std::vector<float> h_bin_err;
  DevBuf d_binok, d_mlpF;
  int mlp_n = 0;
  double mlp_tau = 0.0;
  int mlp_engine = FB_MLP_ENGINE_TC;
  // per-kernel CUDA-event timing (fb_set_timing)
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> evpool;
  std::vector<std::pair<int, int>> pending;  // (kernel id, event index)
  double kt_ms[KT_N] = {0};
  long long kt_n[KT_N] = {0};
};

static PPArgs pp_args(fb_ctx *ctx);
static EwaldArgs ewald_args(fb_ctx *ctx);
static int ewald_setup(fb_ctx *ctx);
template <typename T>
static int host_scan(fb_ctx *ctx, const DevBuf &cnt, int n, std::vector<T> &off, DevBuf &d_off);

static int fail(fb_ctx *c, int code, const char *fmt, ...) {
  char b[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(b, sizeof b, fmt, ap);
  va_end(ap);
  if (c) c->err = b;
  return code;
}

#define CU(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(ctx, FB_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
#define CHK(call)                                                               \
  do {                                                                          \
    int st_ = (call);                                                           \
    if (st_) return st_ == FB_ERR_CUDA ? fail(ctx, FB_ERR_CUDA, "allocation failed: %s", #call) : st_; \
  } while (0)
static int timing_begin(fb_ctx *ctx) {
  size_t k = ctx->pending.size();
  if (k >= ctx->evpool.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1;
    ctx->evpool.push_back({a, b});
  }
  cudaEventRecord(ctx->evpool[k].first, ctx->stream);
  return (int)k;
}

static void timing_end(fb_ctx *ctx, int kid, int ev) {
  if (ev < 0) return;
  cudaEventRecord(ctx->evpool[ev].second, ctx->stream);
  ctx->pending.push_back({kid, ev});
}

// fold finished launches into the per-kernel totals (after a stream sync)
static void timing_drain(fb_ctx *ctx) {
  for (auto &pe : ctx->pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->evpool[pe.second].first, ctx->evpool[pe.second].second) == cudaSuccess) {
      ctx->kt_ms[pe.first] += ms;
      ctx->kt_n[pe.first] += 1;
    }
  }
  ctx->pending.clear();
}

#define KL(kid, call)                                                                                   \
  do {                                                                                                  \
    int ev_ = ctx->timing ? timing_begin(ctx) : -1;                                                     \
    int e_ = (call);                                                                                    \
    ctx->launches++;                                                                                    \
    timing_end(ctx, kid, ev_);                                                                          \
    if (e_) return fail(ctx, FB_ERR_CUDA, "launch %s: %s", #call, cudaGetErrorString((cudaError_t)e_)); \
  } while (0)

static int sync_status(fb_ctx *ctx, unsigned *st) {
  CU(cudaMemcpyAsync(st, ctx->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (ctx->timing) timing_drain(ctx);
  return FB_OK;
}

static int status_error(fb_ctx *ctx, unsigned st) {
  if (st & DEVERR_CLOSE) {
    int info[3] = {0, 0, 0};
    cudaMemcpy(info, ctx->d_errinfo.p, sizeof info, cudaMemcpyDeviceToHost);
    return fail(ctx, FB_ERR_ATOMS_CLOSE, "atoms dangerously close: iatom %d jatom %d mbeta %d", info[0] + 1,
                info[1] + 1, info[2]);
  }
  if (st & DEVERR_CAP) {
    int info[3] = {0, 0, 0};
    cudaMemcpy(info, ctx->d_errinfo.p, sizeof info, cudaMemcpyDeviceToHost);
    return fail(ctx, FB_ERR_CAPACITY, "PPp: the image of atom %d seen from atom %d lies outside the 9x9x9 image box",
                info[1] + 1, info[0] + 1);
  }
  if (st & DEVERR_SELF) return fail(ctx, FB_ERR_NEIGH_SELF, "neigh_self missing");
  if (st & DEVERR_BACK) return fail(ctx, FB_ERR_NEIGH_BACK, "neigh_back missing or found twice");
  if (st & DEVERR_XLARGE) return fail(ctx, FB_ERR_X_TOO_LARGE, "interaction distance beyond table range");
  if (st & DEVERR_TABLE) return fail(ctx, FB_ERR_TABLE, "table missing");
  if (st & DEVERR_WATCHDOG) return fail(ctx, FB_ERR_WATCHDOG, "a tensor-core product did not complete in time");
  return FB_OK;
}

static int noalloc_scratch(fb_ctx *ctx, double **out);

extern "C" {

const char *fb_version(void) { return "fbgpu 0.1 sm_103a fp64"; }

int fb_create(int device, fb_ctx **out) {
  if (!out) return FB_ERR_ARG;
  *out = nullptr;
  fb_ctx *ctx = new fb_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return FB_ERR_CUDA;
  }
  ctx->stream = ctx->own;
  if (ctx->d_status.ensure(sizeof(unsigned)) || ctx->d_errinfo.ensure(4 * sizeof(int))) {
    delete ctx;
    return FB_ERR_CUDA;
  }
  cudaMemset(ctx->d_status.p, 0, sizeof(unsigned));
  if (cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      ctx->d_queue.ensure(TK_N * sizeof(int))) {
    fb_destroy(ctx);
    return FB_ERR_CUDA;
  }
  for (int k = 0; k < TK_N; k++) ctx->cfg[k] = KCfg{128, 0, 1, ctx->nsm};
  // the device address of fb_dassemble_noalloc's static scratch, looked up
  // here so that the entry point itself never loads a module or reserves
  // memory
  double *scr = nullptr;
  if (noalloc_scratch(ctx, &scr) != FB_OK) {
    fb_destroy(ctx);
    return FB_ERR_CUDA;
  }
  *out = ctx;
  return FB_OK;
}

void fb_destroy(fb_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  DevBuf *bufs[] = {&ctx->d_fd, &ctx->d_tab2, &ctx->d_tab3, &ctx->d_lin, &ctx->d_gxy, &ctx->d_ratom,
                    &ctx->d_pos4, &ctx->d_isp, &ctx->d_xl, &ctx->d_xlf, &ctx->d_imgs, &ctx->d_cnt,
                    &ctx->d_pair_off, &ctx->d_neigh_j, &ctx->d_neigh_b, &ctx->d_neigh_self, &ctx->d_neigh_back,
                    &ctx->d_pair_owner, &ctx->d_r3v, &ctx->d_r3f, &ctx->d_blk_off, &ctx->d_tcnt,
                    &ctx->d_trip_off, &ctx->d_ci_j, &ctx->d_ci_b, &ctx->d_cj_j, &ctx->d_cj_b, &ctx->d_cneigh,
                    &ctx->d_tdst, &ctx->d_talpha, &ctx->d_status, &ctx->d_errinfo, &ctx->d_S, &ctx->d_T,
                    &ctx->d_vb, &ctx->d_vbo, &ctx->d_rho, &ctx->d_cape, &ctx->d_dS, &ctx->d_dT, &ctx->d_sumT,
                    &ctx->d_sumS, &ctx->d_ontop, &ctx->d_atomf, &ctx->d_f3a, &ctx->d_f3b, &ctx->d_f3c,
                    &ctx->d_kin, &ctx->d_vna, &ctx->d_pul, &ctx->d_ftot, &ctx->d_bsum, &ctx->d_blk_base, &ctx->d_tab3df, &ctx->d_rho_df, &ctx->d_tkey, &ctx->d_trank, &ctx->d_tperm, &ctx->d_tbin, &ctx->d_mlp_pts, &ctx->d_mlp_ptrip,
                    &ctx->d_thist, &ctx->d_slot_off, &ctx->d_slot_nn, &ctx->d_slot_found, &ctx->d_rcnt, &ctx->d_sid, &ctx->d_satom_off, &ctx->d_simg_off, &ctx->d_sbbox,
                    &ctx->d_img_off, &ctx->d_img_start, &ctx->d_img_orb,
                    &ctx->d_cbox, &ctx->d_cb_off,
                    &ctx->d_speriodic};
  for (DevBuf *b : bufs) b->release();
  ctx->d_queue.release();
  solver_destroy(ctx->solver);
  DevBuf *sb[] = {&ctx->d_sol_S, &ctx->d_sol_H, &ctx->d_sol_W, &ctx->d_sol_T, &ctx->d_sol_lam, &ctx->d_sol_eps,
                  &ctx->d_sol_work, &ctx->d_sol_info, &ctx->d_orb_slot};
  for (DevBuf *b : sb) b->release();
  ctx->d_binok.release();
  ctx->d_mlpF.release();
  DevBuf *mb[] = {&ctx->mlp.params, &ctx->mlp.grad, &ctx->mlp.adam_m, &ctx->mlp.adam_v, &ctx->mlp.wbf,
                  &ctx->mlp.scale, &ctx->mlp.tmeta, &ctx->mlp.dX, &ctx->mlp.dXt, &ctx->mlp.dY, &ctx->mlp.dTrip,
                  &ctx->mlp.Z, &ctx->mlp.H, &ctx->mlp.Ht, &ctx->mlp.O, &ctx->mlp.dO, &ctx->mlp.dOt,
                  &ctx->mlp.dZ, &ctx->mlp.dZt, &ctx->mlp.dXg, &ctx->mlp.part};
  for (DevBuf *b : mb) b->release();
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  for (auto &e : ctx->evpool) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  if (ctx->own) cudaStreamDestroy(ctx->own);
  if (ctx->cstream) cudaStreamDestroy(ctx->cstream);
  if (ctx->s2) cudaStreamDestroy(ctx->s2);
  cudaEvent_t evs[] = {ctx->ev_in, ctx->ev_val, ctx->ev_frc, ctx->ev_nb, ctx->ev_2c};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  delete ctx;
}

const char *fb_last_error(const fb_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long fb_kernel_launches(const fb_ctx *ctx) { return ctx ? ctx->launches : 0; }

int fb_set_stream(fb_ctx *ctx, void *stream) {
  if (!ctx) return FB_ERR_ARG;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
  return FB_OK;
}

int fb_load_fdata(fb_ctx *ctx, const char *fdata_dir, int nspecies, const int *nZ) {
  if (!ctx || !fdata_dir || !nZ) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = fdata_read(fdata_dir, nspecies, nZ, ctx->fdh, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  FdataHost &f = ctx->fdh;
  CHK(ctx->d_fd.ensure(sizeof(FdataDev)));
  CHK(ctx->d_tab2.ensure(f.table2c.size() * sizeof(double)));
  CHK(ctx->d_tab3.ensure(f.table3c.size() * sizeof(double)));
  CHK(ctx->d_tab3df.ensure(f.table3c_df.size() * sizeof(float)));
  CHK(ctx->d_lin.ensure(f.lin.size()));
  CHK(ctx->d_gxy.ensure(f.gxy.size() * sizeof(double)));
  CU(cudaMemcpy(ctx->d_fd.p, &f.dev, sizeof(FdataDev), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_tab2.p, f.table2c.data(), f.table2c.size() * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_tab3.p, f.table3c.data(), f.table3c.size() * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_tab3df.p, f.table3c_df.data(), f.table3c_df.size() * sizeof(float), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_lin.p, f.lin.data(), f.lin.size(), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_gxy.p, f.gxy.data(), f.gxy.size() * sizeof(double), cudaMemcpyHostToDevice));
  ctx->have_fdata = true;
  ctx->have_neigh = false;
  ctx->have_pp_neigh = ctx->have_rho_pp = ctx->have_ewald = ctx->ewald_matrix = false;
  return FB_OK;
}

int fb_species_norb(const fb_ctx *ctx, int isp) {
  if (!ctx || !ctx->have_fdata || isp < 1 || isp > ctx->fdh.nspecies) return -1;
  return ctx->fdh.sp[isp - 1].norb;
}

// image list of structure s: every cell mbeta whose translation can bring
// some atom within range of another; kept in increasing mbeta (the
// reference loop order)
static void make_images(fb_ctx *ctx, int s, const double *ratom) {
  if (ctx->h_icl[s] == 1) {
    ctx->h_imgs.push_back(0);
    return;
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = ctx->h_satom_off[s]; i < ctx->h_satom_off[s + 1]; i++)
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], ratom[3 * i + k]);
      hi[k] = std::max(hi[k], ratom[3 * i + k]);
    }
  double D = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                       (hi[2] - lo[2]) * (hi[2] - lo[2]));
  double rmax = 0.0;
  for (int k = 0; k < ctx->fdh.nspecies; k++)
    rmax = std::max(rmax, std::max(ctx->fdh.sp[k].rcA, ctx->fdh.sp[k].rc_pp));
  double reach = std::max(2.0 * rmax, 0.5) + D + 1.0;
  const double *X = &ctx->h_xl[(size_t)s * XL_STRIDE];
  for (int mb = 0; mb < NIMG; mb++) {
    const double *L = X + 3 * mb;
    double l = std::sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    if (l < reach) ctx->h_imgs.push_back(mb);
  }
}

int fb_set_batch(fb_ctx *ctx, int nstruct, const int *natoms, const double *ratom, const int *imass,
                 const double *lattice, const int *icluster) {
  if (!ctx || nstruct < 1 || !natoms || !ratom || !imass) return FB_ERR_ARG;
  if (!ctx->have_fdata) return fail(ctx, FB_ERR_STATE, "fb_load_fdata first");
  long long total = 0;
  for (int s = 0; s < nstruct; s++) {
    if (natoms[s] < 1) return fail(ctx, FB_ERR_ARG, "structure %d has %d atoms", s + 1, natoms[s]);
    if ((!icluster || icluster[s] != 1) && !lattice)
      return fail(ctx, FB_ERR_ARG, "structure %d is periodic but no lattice was given", s + 1);
    total += natoms[s];
  }
  if (total > (1LL << 30)) return fail(ctx, FB_ERR_ARG, "%lld atoms in the batch", total);
  CU(cudaSetDevice(ctx->device));
  int N = (int)total;
  if (N != ctx->N) ctx->have_charges = false;
  ctx->N = N;
  ctx->nstruct = nstruct;
  ctx->h_isp.resize(N);
  for (int i = 0; i < N; i++) {
    if (imass[i] < 1 || imass[i] > ctx->fdh.nspecies)
      return fail(ctx, FB_ERR_ARG, "imass(%d) = %d out of range", i + 1, imass[i]);
    ctx->h_isp[i] = imass[i] - 1;
  }
  ctx->h_satom_off.assign(nstruct + 1, 0);
  ctx->h_sid.resize(N);
  ctx->h_icl.assign(nstruct, 0);
  ctx->h_lat.assign((size_t)9 * nstruct, 0.0);
  ctx->h_xl.assign((size_t)XL_STRIDE * nstruct, 0.0);
  for (int s = 0; s < nstruct; s++) {
    ctx->h_satom_off[s + 1] = ctx->h_satom_off[s] + natoms[s];
    for (int i = ctx->h_satom_off[s]; i < ctx->h_satom_off[s + 1]; i++) ctx->h_sid[i] = s;
    ctx->h_icl[s] = icluster ? icluster[s] : 0;
    if (ctx->h_icl[s] == 1) continue;  // a cluster has mbeta = 0 only
    double *lat = &ctx->h_lat[(size_t)9 * s];
    std::memcpy(lat, lattice + (size_t)9 * s, 9 * sizeof(double));
    // make_cells (c.SYSTEM/make_cells.f90:112-144)
    double *X = &ctx->h_xl[(size_t)s * XL_STRIDE];
    int mb = 1;
    for (int iz = -P_mbox; iz <= P_mbox; iz++)
      for (int iy = -P_mbox; iy <= P_mbox; iy++)
        for (int ix = -P_mbox; ix <= P_mbox; ix++)
          if (!(ix == 0 && iy == 0 && iz == 0)) {
            for (int k = 0; k < 3; k++)
              X[3 * mb + k] = (double)ix * lat[k] + (double)iy * lat[3 + k] + (double)iz * lat[6 + k];
            mb++;
          }
  }
  std::vector<float> xlf(ctx->h_xl.begin(), ctx->h_xl.end());
  std::vector<int> per(nstruct);
  for (int s = 0; s < nstruct; s++) per[s] = ctx->h_icl[s] != 1;
  CHK(ctx->d_xl.ensure(ctx->h_xl.size() * sizeof(double)));
  CHK(ctx->d_xlf.ensure(xlf.size() * sizeof(float)));
  CHK(ctx->d_isp.ensure(N * sizeof(int)));
  CHK(ctx->d_sid.ensure(N * sizeof(int)));
  CHK(ctx->d_satom_off.ensure((nstruct + 1) * sizeof(int)));
  CHK(ctx->d_speriodic.ensure(nstruct * sizeof(int)));
  CU(cudaMemcpy(ctx->d_xl.p, ctx->h_xl.data(), ctx->h_xl.size() * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_xlf.p, xlf.data(), xlf.size() * sizeof(float), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_isp.p, ctx->h_isp.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_sid.p, ctx->h_sid.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_satom_off.p, ctx->h_satom_off.data(), (nstruct + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ctx->d_speriodic.p, per.data(), nstruct * sizeof(int), cudaMemcpyHostToDevice));
  ctx->have_neigh = false;
  ctx->have_pp_neigh = ctx->have_rho_pp = ctx->have_ewald = ctx->ewald_matrix = false;
  return fb_update_positions(ctx, ratom);
}

int fb_set_structure(fb_ctx *ctx, int natoms, const double *ratom, const int *imass, const double *lattice,
                     int icluster) {
  if (!ctx || natoms < 1 || !ratom || !imass || (!lattice && icluster != 1)) return FB_ERR_ARG;
  return fb_set_batch(ctx, 1, &natoms, ratom, imass, lattice, &icluster);
}

int fb_update_positions(fb_ctx *ctx, const double *ratom) {
  if (!ctx || !ratom) return FB_ERR_ARG;
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  CU(cudaSetDevice(ctx->device));
  int N = ctx->N, ns = ctx->nstruct;
  ctx->h_imgs.clear();
  ctx->h_simg_off.assign(ns + 1, 0);
  ctx->h_img_off.assign(ns + 1, 0);
  for (int s = 0; s < ns; s++) {
    make_images(ctx, s, ratom);
    ctx->h_simg_off[s + 1] = (int)ctx->h_imgs.size();
    long long na = ctx->h_satom_off[s + 1] - ctx->h_satom_off[s];
    ctx->h_img_off[s + 1] = ctx->h_img_off[s] + na * (ctx->h_simg_off[s + 1] - ctx->h_simg_off[s]);
  }
  // float positions with the species cutoff in .w, and the bounding boxes
  std::vector<float4> p4(N);
  float rcmax = 0.0f;
  for (int k = 0; k < ctx->fdh.nspecies; k++) rcmax = std::max(rcmax, (float)ctx->fdh.sp[k].rcA);
  ctx->rcmax = rcmax;
  ctx->h_sbbox.assign(2 * (size_t)ns, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  for (int s = 0; s < ns; s++) {
    float4 lo = make_float4(1e30f, 1e30f, 1e30f, 0.0f), hi = make_float4(-1e30f, -1e30f, -1e30f, 0.0f);
    for (int i = ctx->h_satom_off[s]; i < ctx->h_satom_off[s + 1]; i++) {
      p4[i] = make_float4((float)ratom[3 * i], (float)ratom[3 * i + 1], (float)ratom[3 * i + 2],
                          (float)ctx->fdh.sp[ctx->h_isp[i]].rcA);
      lo.x = std::min(lo.x, p4[i].x);
      lo.y = std::min(lo.y, p4[i].y);
      lo.z = std::min(lo.z, p4[i].z);
      hi.x = std::max(hi.x, p4[i].x);
      hi.y = std::max(hi.y, p4[i].y);
      hi.z = std::max(hi.z, p4[i].z);
    }
    ctx->h_sbbox[2 * s] = lo;
    ctx->h_sbbox[2 * s + 1] = hi;
  }
  // bounding boxes of the chunks of 32 consecutive atoms the neighbor sweep
  // takes per warp step: a chunk whose shifted box lies beyond reach of atom
  // i is skipped whole, which keeps the (mbeta, jatom) order
  ctx->h_cb_off.assign(ns + 1, 0);
  for (int s = 0; s < ns; s++) {
    int na = ctx->h_satom_off[s + 1] - ctx->h_satom_off[s];
    ctx->h_cb_off[s + 1] = ctx->h_cb_off[s] + (na + 31) / 32;
  }
  ctx->h_cbox.assign(2 * (size_t)ctx->h_cb_off[ns], make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  for (int s = 0; s < ns; s++) {
    int a0 = ctx->h_satom_off[s], a1 = ctx->h_satom_off[s + 1];
    for (int k = 0; a0 + 32 * k < a1; k++) {
      float4 lo = make_float4(1e30f, 1e30f, 1e30f, 0.0f), hi = make_float4(-1e30f, -1e30f, -1e30f, 0.0f);
      for (int i = a0 + 32 * k; i < std::min(a1, a0 + 32 * k + 32); i++) {
        lo.x = std::min(lo.x, p4[i].x);
        lo.y = std::min(lo.y, p4[i].y);
        lo.z = std::min(lo.z, p4[i].z);
        hi.x = std::max(hi.x, p4[i].x);
        hi.y = std::max(hi.y, p4[i].y);
        hi.z = std::max(hi.z, p4[i].z);
      }
      ctx->h_cbox[2 * (size_t)(ctx->h_cb_off[s] + k)] = lo;
      ctx->h_cbox[2 * (size_t)(ctx->h_cb_off[s] + k) + 1] = hi;
    }
  }
  CHK(ctx->d_ratom.ensure(3 * (size_t)N * sizeof(double)));
  CHK(ctx->d_pos4.ensure(N * sizeof(float4)));
  CHK(ctx->d_imgs.ensure(ctx->h_imgs.size() * sizeof(int)));
  CHK(ctx->d_simg_off.ensure((ns + 1) * sizeof(int)));
  CHK(ctx->d_sbbox.ensure(2 * (size_t)ns * sizeof(float4)));
  CHK(ctx->d_cbox.ensure(ctx->h_cbox.size() * sizeof(float4)));
  CHK(ctx->d_cb_off.ensure((ns + 1) * sizeof(int)));
  CHK(ctx->d_img_off.ensure((ns + 1) * sizeof(long long)));
  CHK(ctx->d_img_start.ensure((size_t)ctx->h_img_off[ns] * sizeof(int) + 4));
  CHK(ctx->d_img_orb.ensure((size_t)ctx->h_img_off[ns] * sizeof(long long) + 8));
  CU(cudaMemcpyAsync(ctx->d_img_off.p, ctx->h_img_off.data(), (ns + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_ratom.p, ratom, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_pos4.p, p4.data(), N * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_imgs.p, ctx->h_imgs.data(), ctx->h_imgs.size() * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_simg_off.p, ctx->h_simg_off.data(), (ns + 1) * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_sbbox.p, ctx->h_sbbox.data(), 2 * (size_t)ns * sizeof(float4), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_cbox.p, ctx->h_cbox.data(), ctx->h_cbox.size() * sizeof(float4), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_cb_off.p, ctx->h_cb_off.data(), (ns + 1) * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_neigh = false;
  ctx->have_pp_neigh = ctx->have_rho_pp = ctx->have_ewald = ctx->ewald_matrix = false;
  return FB_OK;
}

static NeighArgs neigh_args(fb_ctx *ctx) {
  NeighArgs a{};
  a.N = ctx->N;
  a.P = ctx->P;
  a.ratom = ctx->d_ratom.as<double>();
  a.pos4 = ctx->d_pos4.as<float4>();
  a.sid = ctx->d_sid.as<int>();
  a.satom_off = ctx->d_satom_off.as<int>();
  a.simg_off = ctx->d_simg_off.as<int>();
  a.sbbox = ctx->d_sbbox.as<float4>();
  a.cbox = ctx->d_cbox.as<float4>();
  a.cb_off = ctx->d_cb_off.as<int>();
  a.speriodic = ctx->d_speriodic.as<int>();
  a.rcmax = ctx->rcmax;
  a.isp = ctx->d_isp.as<int>();
  a.fd = ctx->d_fd.as<FdataDev>();
  a.xl = ctx->d_xl.as<double>();
  a.xlf = ctx->d_xlf.as<float>();
  a.imgs = ctx->d_imgs.as<int>();
  a.img_off = ctx->d_img_off.as<long long>();
  a.img_start = ctx->d_img_start.as<int>();
  a.img_orb = ctx->d_img_orb.as<long long>();
  a.cnt = ctx->d_cnt.as<int>();
  a.bsum = ctx->d_bsum.as<long long>();
  a.blk_base = ctx->d_blk_base.as<long long>();
  a.pair_owner_w = ctx->d_pair_owner.as<int>();
  a.blk_off_w = ctx->d_blk_off.as<long long>();
  a.talpha = ctx->d_talpha.as<int>();
  a.pair_off = ctx->d_pair_off.as<int>();
  a.neigh_j = ctx->d_neigh_j.as<int>();
  a.neigh_b = ctx->d_neigh_b.as<int>();
  a.neigh_self = ctx->d_neigh_self.as<int>();
  a.neigh_back = ctx->d_neigh_back.as<int>();
  a.pair_owner = ctx->d_pair_owner.as<int>();
  a.r3v = ctx->d_r3v.as<double>();
  a.r3f = ctx->d_r3f.as<float4>();
  a.tcnt = ctx->d_tcnt.as<int>();
  a.rcnt = ctx->d_rcnt.as<int>();
  a.trip_off = ctx->d_trip_off.as<int>();
  a.ci_j = ctx->d_ci_j.as<int>();
  a.ci_b = ctx->d_ci_b.as<int>();
  a.cj_j = ctx->d_cj_j.as<int>();
  a.cj_b = ctx->d_cj_b.as<int>();
  a.cneigh = ctx->d_cneigh.as<int>();
  a.tdst = ctx->d_tdst.as<int>();
  a.slot_off = ctx->d_slot_off.as<long long>();
  a.slot_nn = ctx->d_slot_nn.as<unsigned>();
  a.slot_found = ctx->d_slot_found.as<int>();
  a.status = ctx->d_status.as<unsigned>();
  a.errinfo = ctx->d_errinfo.as<int>();
  return a;
}

// grid nodes of the largest 3c cell (the bin count per species triple)
static int trip_cells(const fb_ctx *ctx) {
  int nsp = ctx->fdh.nspecies, cells = 1;
  for (int x = 0; x < nsp; x++)
    for (int y = 0; y < nsp; y++)
      for (int z = 0; z < nsp; z++) cells = std::max(cells, ctx->fdh.dev.c3[x][y][z].nx * ctx->fdh.dev.c3[x][y][z].ny);
  return cells;
}

static bool mlp_routes(const fb_ctx *ctx) {
  return ctx->mlp.ready && ctx->mlp_mode != FB_MLP_OFF && !ctx->fdh.have_d && ctx->theory == FB_THEORY_HARRIS;
}

// counting sort of the triplets by interpolation bin, approved MLP-3c bins
// first; mlp_n = triplets the network takes
// the three-center table kernels' view of list positions nm .. T-1: the
// binned copies of the triplet lists, read in order
static AsmArgs table3c_view(const fb_ctx *ctx, const AsmArgs &a, int nm) {
  AsmArgs at = a;
  int T = ctx->T;
  at.ntrip = T - nm;
  if (ctx->tbin_T == T && ctx->d_tbin.p) {
    const int *b = ctx->d_tbin.as<int>();
    long long n = T;
    at.trip_alpha = b + nm;
    at.ci_j = b + n + nm;
    at.ci_b = b + 2 * n + nm;
    at.cj_j = b + 3 * n + nm;
    at.cj_b = b + 4 * n + nm;
    at.tdst = b + 5 * n + nm;
    at.tperm = nullptr;
  } else {
    at.tperm = a.tperm ? a.tperm + nm : nullptr;
  }
  return at;
}

static int bin_triplets(fb_ctx *ctx) {
  int T = ctx->T, nsp = ctx->fdh.nspecies, cells = trip_cells(ctx);
  size_t nbins = (size_t)nsp * nsp * nsp * cells;
  size_t tb = (size_t)T * sizeof(int) + 4;
  CHK(ctx->d_tkey.ensure(tb));
  CHK(ctx->d_trank.ensure(tb));
  CHK(ctx->d_tperm.ensure(tb));
  CHK(ctx->d_thist.ensure(2 * nbins * sizeof(int)));
  CHK(ctx->d_tbin.ensure(6 * (size_t)T * sizeof(int) + 4));
  bool gated = mlp_routes(ctx) && ctx->mlp_mode == FB_MLP_GATED && ctx->d_binok.p;
  NeighArgs a = neigh_args(ctx);
  KL(KT_TRIP_BINS, launch_trip_bins(a, T, nsp, cells, gated ? ctx->d_binok.as<unsigned char>() : nullptr,
                                    ctx->d_tkey.as<int>(), ctx->d_trank.as<int>(), ctx->d_thist.as<int>(),
                                    ctx->d_tperm.as<int>(), ctx->d_tbin.as<int>(), ctx->stream));
  ctx->tbin_T = T;
  ctx->mlp_n = 0;
  if (mlp_routes(ctx) && ctx->mlp_mode == FB_MLP_ALL) ctx->mlp_n = T;
  if (gated && T > 0) {
    CU(cudaMemcpyAsync(&ctx->mlp_n, ctx->d_thist.as<int>() + nbins, sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
  }
  return FB_OK;
}

// after the pair lists exist on the device: neigh_back and the block storage
static int finish_pairs(fb_ctx *ctx) {
  int P = ctx->P;
  CHK(ctx->d_neigh_back.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_r3v.ensure(3 * P * sizeof(double) + 8));
  CHK(ctx->d_r3f.ensure(P * sizeof(float4) + 16));
  NeighArgs a = neigh_args(ctx);
  KL(KT_NEIGH_BACK, launch_neigh_back(a, ctx->stream));
  size_t bb = (size_t)ctx->nblock * sizeof(double) + 8;
  CHK(ctx->d_S.ensure(bb));
  CHK(ctx->d_T.ensure(bb));
  CHK(ctx->d_vb.ensure(bb));
  CHK(ctx->d_vbo.ensure(bb));
  return FB_OK;
}

// after neigh_back: the common neighbors and the triplet binning (one host
// synchronization with ctx->stream for the triplet count)
static int finish_common(fb_ctx *ctx) {
  int N = ctx->N, P = ctx->P;
  NeighArgs a = neigh_args(ctx);
  // common neighbors: slots for every ordered pair of ialpha's non-self
  // neighbors, one row of n - 1 per non-self neighbor (n of them)
  std::vector<long long> soff(N + 1, 0);
  for (int i = 0; i < N; i++) {
    long long n = ctx->h_pair_off[i + 1] - ctx->h_pair_off[i] - 1;  // non-self neighbors
    if (n > 65535) return fail(ctx, FB_ERR_CAPACITY, "atom %d has %lld neighbors (at most 65536)", i + 1, n + 1);
    soff[i + 1] = soff[i] + (n > 1 ? n * (n - 1) : 0);
  }
  CHK(ctx->d_tcnt.ensure(N * sizeof(int)));
  CHK(ctx->d_rcnt.ensure((size_t)P * sizeof(int) + 4));
  CHK(ctx->d_slot_off.ensure((N + 1) * sizeof(long long)));
  CHK(ctx->d_slot_nn.ensure((size_t)soff[N] * sizeof(unsigned) + 4));
  CHK(ctx->d_slot_found.ensure((size_t)soff[N] * sizeof(int) + 4));
  CU(cudaMemcpyAsync(ctx->d_slot_off.p, soff.data(), (N + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                     ctx->stream));
  a = neigh_args(ctx);
  KL(KT_COMMON_COUNT, launch_common(a, ctx->stream));
  std::vector<int> tc(N);
  CU(cudaMemcpyAsync(tc.data(), ctx->d_tcnt.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  ctx->h_trip_off.assign(N + 1, 0);
  for (int i = 0; i < N; i++) ctx->h_trip_off[i + 1] = ctx->h_trip_off[i] + tc[i];
  int T = ctx->h_trip_off[N];
  ctx->T = T;
  size_t tb = (size_t)T * sizeof(int) + 4;
  CHK(ctx->d_trip_off.ensure((N + 1) * sizeof(int)));
  CHK(ctx->d_ci_j.ensure(tb));
  CHK(ctx->d_ci_b.ensure(tb));
  CHK(ctx->d_cj_j.ensure(tb));
  CHK(ctx->d_cj_b.ensure(tb));
  CHK(ctx->d_cneigh.ensure(tb));
  CHK(ctx->d_tdst.ensure(tb));
  CHK(ctx->d_talpha.ensure(tb));
  CU(cudaMemcpyAsync(ctx->d_trip_off.p, ctx->h_trip_off.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  a = neigh_args(ctx);
  KL(KT_COMMON_FILL, launch_common_compact(a, ctx->stream));
  ctx->mlp_cells = trip_cells(ctx);
  // triplet processing order, binned by (species triple, 3c grid cell)
  CHK(bin_triplets(ctx));
  ctx->have_neigh = true;
  ctx->have_vna2c = ctx->have_rho = ctx->have_cape = ctx->have_dblocks = ctx->have_dip = false;
  ctx->assembled = ctx->dassembled = 0;
  return FB_OK;
}

static int finish_neighbors(fb_ctx *ctx) {
  CHK(finish_pairs(ctx));
  return finish_common(ctx);
}

// the pair stage of fb_neighbors: counts, pair lists, neigh_back, block storage
static int neighbors_pairs(fb_ctx *ctx) {
  int N = ctx->N;
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  CHK(ctx->d_cnt.ensure(N * sizeof(int)));
  CHK(ctx->d_bsum.ensure(N * sizeof(long long)));
  NeighArgs a = neigh_args(ctx);
  KL(KT_NEIGH_COUNT, launch_neigh(a, false, ctx->stream));
  std::vector<int> cnt(N);
  std::vector<long long> bsum(N), bbase(N);
  CU(cudaMemcpyAsync(cnt.data(), ctx->d_cnt.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaMemcpyAsync(bsum.data(), ctx->d_bsum.p, N * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  ctx->h_pair_off.assign(N + 1, 0);
  ctx->h_blk_base.assign(N + 1, 0);
  long long nb = 0;
  for (int i = 0; i < N; i++) {
    ctx->h_pair_off[i + 1] = ctx->h_pair_off[i] + cnt[i];
    bbase[i] = nb;
    ctx->h_blk_base[i] = nb;
    nb += bsum[i];
  }
  ctx->h_blk_base[N] = nb;
  int P = ctx->h_pair_off[N];
  ctx->P = P;
  ctx->nblock = nb;
  CHK(ctx->d_pair_off.ensure((N + 1) * sizeof(int)));
  CHK(ctx->d_blk_base.ensure(N * sizeof(long long)));
  CHK(ctx->d_neigh_j.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_neigh_b.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_neigh_self.ensure(N * sizeof(int)));
  CHK(ctx->d_pair_owner.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_blk_off.ensure((P + 1) * sizeof(long long)));
  CU(cudaMemcpyAsync(ctx->d_pair_off.p, ctx->h_pair_off.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_blk_base.p, bbase.data(), N * sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_blk_off.as<long long>() + P, &ctx->nblock, sizeof(long long), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemsetAsync(ctx->d_neigh_self.p, 0xff, N * sizeof(int), ctx->stream));
  a = neigh_args(ctx);
  KL(KT_NEIGH_FILL, launch_neigh(a, true, ctx->stream));
  return finish_pairs(ctx);
}

int fb_neighbors(fb_ctx *ctx) {
  if (!ctx) return FB_ERR_ARG;
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  CU(cudaSetDevice(ctx->device));
  CHK(neighbors_pairs(ctx));
  return finish_common(ctx);
}

int fb_set_neighbors(fb_ctx *ctx, const int *neighn, const int *neigh_j, const int *neigh_b) {
  if (!ctx || !neighn || !neigh_j || !neigh_b) return FB_ERR_ARG;
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  CU(cudaSetDevice(ctx->device));
  int N = ctx->N;
  ctx->h_pair_off.assign(N + 1, 0);
  for (int i = 0; i < N; i++) {
    if (neighn[i] < 0) return fail(ctx, FB_ERR_ARG, "neighn(%d) < 0", i + 1);
    ctx->h_pair_off[i + 1] = ctx->h_pair_off[i] + neighn[i];
  }
  int P = ctx->h_pair_off[N];
  ctx->P = P;
  // neigh_j is numbered within the atom's own structure (1-based)
  std::vector<int> nj(P), self(N, -1);
  for (int i = 0; i < N; i++) {
    int s = ctx->h_sid[i], a0 = ctx->h_satom_off[s], ns = ctx->h_satom_off[s + 1] - a0;
    int bmax = ctx->h_icl[s] == 1 ? 0 : NIMG - 1;
    for (int p = ctx->h_pair_off[i]; p < ctx->h_pair_off[i + 1]; p++) {
      if (neigh_j[p] < 1 || neigh_j[p] > ns || neigh_b[p] < 0 || neigh_b[p] > bmax)
        return fail(ctx, FB_ERR_ARG, "neighbor %d of atom %d out of range", p - ctx->h_pair_off[i] + 1, i + 1);
      nj[p] = a0 + neigh_j[p] - 1;
      if (nj[p] == i && neigh_b[p] == 0) {
        if (self[i] >= 0) return fail(ctx, FB_ERR_NEIGH_SELF, "neigh_self found twice for atom %d", i + 1);
        self[i] = p - ctx->h_pair_off[i];
      }
    }
  }
  CHK(ctx->d_pair_off.ensure((N + 1) * sizeof(int)));
  CHK(ctx->d_neigh_j.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_neigh_b.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_neigh_self.ensure(N * sizeof(int)));
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_pair_off.p, ctx->h_pair_off.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_neigh_j.p, nj.data(), P * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_neigh_b.p, neigh_b, P * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_neigh_self.p, self.data(), N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  std::vector<int> owner(P);
  std::vector<long long> blk(P + 1);
  long long off = 0;
  ctx->h_blk_base.assign(N + 1, 0);
  for (int i = 0; i < N; i++) {
    if (self[i] < 0) return fail(ctx, FB_ERR_NEIGH_SELF, "no neigh_self for atom %d", i + 1);
    ctx->h_blk_base[i] = off;
    int ni = ctx->fdh.sp[ctx->h_isp[i]].norb;
    for (int p = ctx->h_pair_off[i]; p < ctx->h_pair_off[i + 1]; p++) {
      owner[p] = i;
      blk[p] = off;
      off += (long long)ni * ctx->fdh.sp[ctx->h_isp[nj[p]]].norb;
    }
  }
  blk[P] = off;
  ctx->h_blk_base[N] = off;
  ctx->nblock = off;
  CHK(ctx->d_pair_owner.ensure(P * sizeof(int) + 4));
  CHK(ctx->d_blk_off.ensure((P + 1) * sizeof(long long)));
  CU(cudaMemcpyAsync(ctx->d_pair_owner.p, owner.data(), P * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(ctx->d_blk_off.p, blk.data(), (P + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return finish_neighbors(ctx);
}

int fb_get_sizes(const fb_ctx *ctx, int *npairs, int *ntriplets, long long *nblock) {
  if (!ctx || !ctx->have_neigh) return FB_ERR_STATE;
  if (npairs) *npairs = ctx->P;
  if (ntriplets) *ntriplets = ctx->T;
  if (nblock) *nblock = ctx->nblock;
  return FB_OK;
}

static int d2h_int(fb_ctx *ctx, int *dst, const DevBuf &src, size_t n, int add) {
  if (!dst) return FB_OK;
  CU(cudaMemcpyAsync(dst, src.p, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (add)
    for (size_t k = 0; k < n; k++) dst[k] += add;
  return FB_OK;
}

// atom numbers of a per-item list, made 1-based within the structure of the
// item's owner atom (off[owner] .. off[owner+1]-1 are the owner's items)
static void local_atoms(const fb_ctx *ctx, int *dst, const std::vector<int> &off) {
  if (!dst || ctx->nstruct < 2) return;
  for (int i = 0; i < ctx->N; i++) {
    int a0 = ctx->h_satom_off[ctx->h_sid[i]];
    for (int k = off[i]; k < off[i + 1]; k++) dst[k] -= a0;
  }
}

int fb_get_neighbors(fb_ctx *ctx, int *neighn, int *neigh_j, int *neigh_b, int *neigh_back, int *neigh_self,
                     long long *blk_off) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if (neighn)
    for (int i = 0; i < ctx->N; i++) neighn[i] = ctx->h_pair_off[i + 1] - ctx->h_pair_off[i];
  CHK(d2h_int(ctx, neigh_j, ctx->d_neigh_j, ctx->P, 1));
  local_atoms(ctx, neigh_j, ctx->h_pair_off);
  CHK(d2h_int(ctx, neigh_b, ctx->d_neigh_b, ctx->P, 0));
  CHK(d2h_int(ctx, neigh_back, ctx->d_neigh_back, ctx->P, 1));
  CHK(d2h_int(ctx, neigh_self, ctx->d_neigh_self, ctx->N, 1));
  if (blk_off) {
    CU(cudaMemcpy(blk_off, ctx->d_blk_off.p, (ctx->P + 1) * sizeof(long long), cudaMemcpyDeviceToHost));
  }
  return FB_OK;
}

// driver_neighbors_PP (c.SYSTEM/M_neighbors_PP.f90:98-151) on the device
int fb_neighbors_pp(fb_ctx *ctx) {
  if (!ctx) return FB_ERR_ARG;
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  if (!ctx->fdh.dev.have_pp)
    return fail(ctx, FB_ERR_TABLE, "vnl: the Fdata lacks a vnl table or a projector basis of s, sp or spd shells");
  if (ctx->nstruct != 1) return fail(ctx, FB_ERR_UNSUPPORTED, "vnl maps: single structures (a batch of one)");
  CU(cudaSetDevice(ctx->device));
  int N = ctx->N;
  ctx->have_pp_neigh = ctx->have_rho_pp = ctx->have_ewald = ctx->ewald_matrix = false;
  ctx->assembled &= ~(unsigned)(FB_SVNL | FB_VNL2C | FB_VNL3C);
  ctx->dassembled &= ~(unsigned)(FB_VNL2C | FB_VNL3C);
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  size_t ib = (size_t)N * sizeof(int) + 4, lb = (size_t)N * sizeof(long long) + 8;
  DevBuf *ibufs[] = {&ctx->d_pp_cnt, &ctx->d_ppx_cnt, &ctx->d_ub, &ctx->d_ppp_cnt, &ctx->d_ppc_cnt, &ctx->d_pp_self,
                     &ctx->d_ppx_self, &ctx->d_ppp_self};
  for (DevBuf *b : ibufs) CHK(b->ensure(ib));
  CHK(ctx->d_svnl_sum.ensure(lb));
  CHK(ctx->d_vnl_sum.ensure(lb));
  PPArgs a = pp_args(ctx);
  // PP and PPx pairs: count, offsets, fill
  KL(KT_PP_PAIRS, launch_pp_pairs(a, 0, false, ctx->stream));
  KL(KT_PP_PAIRS, launch_pp_pairs(a, 1, false, ctx->stream));
  CHK(host_scan<int>(ctx, ctx->d_pp_cnt, N, ctx->h_pp_off, ctx->d_pp_off));
  CHK(host_scan<int>(ctx, ctx->d_ppx_cnt, N, ctx->h_ppx_off, ctx->d_ppx_off));
  CHK(host_scan<long long>(ctx, ctx->d_svnl_sum, N, ctx->h_svnl_base, ctx->d_svnl_base));
  ctx->npp = ctx->h_pp_off[N];
  ctx->nppx = ctx->h_ppx_off[N];
  ctx->nsvnl = ctx->h_svnl_base[N];
  size_t pb = (size_t)ctx->npp * sizeof(int) + 4, xb = (size_t)ctx->nppx * sizeof(int) + 4;
  CHK(ctx->d_pp_j.ensure(pb));
  CHK(ctx->d_pp_b.ensure(pb));
  CHK(ctx->d_pp_map.ensure(pb));
  CHK(ctx->d_svnl_off.ensure((size_t)ctx->npp * sizeof(long long) + 8));
  CHK(ctx->d_ppx_j.ensure(xb));
  CHK(ctx->d_ppx_b.ensure(xb));
  CHK(ctx->d_ppx_map.ensure(xb));
  CHK(ctx->d_ppx_point.ensure(xb));
  CU(cudaMemsetAsync(ctx->d_pp_self.p, 0xff, N * sizeof(int), ctx->stream));
  CU(cudaMemsetAsync(ctx->d_ppx_self.p, 0xff, N * sizeof(int), ctx->stream));
  a = pp_args(ctx);
  KL(KT_PP_PAIRS, launch_pp_pairs(a, 0, true, ctx->stream));
  KL(KT_PP_PAIRS, launch_pp_pairs(a, 1, true, ctx->stream));
  // PPp: candidate bounds, first occurrences into slots, compaction + maps
  KL(KT_PPP, launch_ppp_bounds(a, ctx->stream));
  {
    std::vector<int> ub(N);
    CU(cudaMemcpyAsync(ub.data(), ctx->d_ub.p, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    std::vector<long long> so(N + 1, 0);
    for (int i = 0; i < N; i++) so[i + 1] = so[i] + ub[i];
    CHK(ctx->d_pslot_off.ensure((N + 1) * sizeof(long long)));
    CHK(ctx->d_pslot_j.ensure((size_t)so[N] * sizeof(int) + 4));
    CHK(ctx->d_pslot_b.ensure((size_t)so[N] * sizeof(int) + 4));
    CU(cudaMemcpyAsync(ctx->d_pslot_off.p, so.data(), (N + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  a = pp_args(ctx);
  KL(KT_PPP, launch_ppp(a, ctx->stream));
  CHK(host_scan<int>(ctx, ctx->d_ppp_cnt, N, ctx->h_ppp_off, ctx->d_ppp_off));
  CHK(host_scan<long long>(ctx, ctx->d_vnl_sum, N, ctx->h_vnl_base, ctx->d_vnl_base));
  ctx->nppp = ctx->h_ppp_off[N];
  ctx->nvnl = ctx->h_vnl_base[N];
  size_t kb = (size_t)ctx->nppp * sizeof(int) + 4;
  CHK(ctx->d_ppp_j.ensure(kb));
  CHK(ctx->d_ppp_b.ensure(kb));
  CHK(ctx->d_vnl_off.ensure((size_t)ctx->nppp * sizeof(long long) + 8));
  CU(cudaMemsetAsync(ctx->d_ppp_self.p, 0xff, N * sizeof(int), ctx->stream));
  a = pp_args(ctx);
  KL(KT_PPP, launch_ppp_compact(a, ctx->npp, ctx->nppx, ctx->stream));
  ctx->launches++;  // compaction + maps
  // common PP triplets: count, offsets, fill
  KL(KT_PPC, launch_ppc(a, false, ctx->stream));
  CHK(host_scan<int>(ctx, ctx->d_ppc_cnt, N, ctx->h_ppc_off, ctx->d_ppc_off));
  ctx->ntrip_pp = ctx->h_ppc_off[N];
  size_t tb = (size_t)ctx->ntrip_pp * sizeof(int) + 4;
  DevBuf *tbufs[] = {&ctx->d_t_alpha, &ctx->d_t_i, &ctx->d_t_ib, &ctx->d_t_j, &ctx->d_t_jb, &ctx->d_t_m,
                     &ctx->d_t_m31, &ctx->d_t_m32};
  for (DevBuf *b : tbufs) CHK(b->ensure(tb));
  a = pp_args(ctx);
  KL(KT_PPC, launch_ppc(a, true, ctx->stream));
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  ctx->have_pp_neigh = true;
  return FB_OK;
}

int fb_get_pp_sizes(fb_ctx *ctx, int *npp, int *nppx, int *nppp, int *ntrip, long long *nsvnl, long long *nvnl) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors_pp first");
  if (npp) *npp = ctx->npp;
  if (nppx) *nppx = ctx->nppx;
  if (nppp) *nppp = ctx->nppp;
  if (ntrip) *ntrip = ctx->ntrip_pp;
  if (nsvnl) *nsvnl = ctx->nsvnl;
  if (nvnl) *nvnl = ctx->nvnl;
  return FB_OK;
}

int fb_get_pp_neighbors(fb_ctx *ctx, int which, int *neighn, int *neigh_j, int *neigh_b, int *self, int *map,
                        int *point) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors_pp first");
  if (which < FB_PP_MAP || which > FB_PPP_MAP) return fail(ctx, FB_ERR_ARG, "unknown PP map %d", which);
  const std::vector<int> &off = which == FB_PP_MAP ? ctx->h_pp_off : which == FB_PPX_MAP ? ctx->h_ppx_off
                                                                                              : ctx->h_ppp_off;
  DevBuf &J = which == FB_PP_MAP ? ctx->d_pp_j : which == FB_PPX_MAP ? ctx->d_ppx_j : ctx->d_ppp_j;
  DevBuf &B = which == FB_PP_MAP ? ctx->d_pp_b : which == FB_PPX_MAP ? ctx->d_ppx_b : ctx->d_ppp_b;
  DevBuf &S = which == FB_PP_MAP ? ctx->d_pp_self : which == FB_PPX_MAP ? ctx->d_ppx_self : ctx->d_ppp_self;
  int n = off[ctx->N];
  if (neighn)
    for (int i = 0; i < ctx->N; i++) neighn[i] = off[i + 1] - off[i];
  CHK(d2h_int(ctx, neigh_j, J, n, 1));
  CHK(d2h_int(ctx, neigh_b, B, n, 0));
  CHK(d2h_int(ctx, self, S, ctx->N, 1));
  if (which == FB_PP_MAP) CHK(d2h_int(ctx, map, ctx->d_pp_map, n, 1));
  if (which == FB_PPX_MAP) {
    CHK(d2h_int(ctx, map, ctx->d_ppx_map, n, 1));
    CHK(d2h_int(ctx, point, ctx->d_ppx_point, n, 1));
  }
  return FB_OK;
}

int fb_get_pp_common(fb_ctx *ctx, int *ncommon, int *iatom_common_j, int *iatom_common_b, int *jatom_common_j,
                     int *jatom_common_b, int *neigh_common, int *m31, int *m32) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors_pp first");
  int T = ctx->ntrip_pp;
  if (ncommon)
    for (int i = 0; i < ctx->N; i++) ncommon[i] = ctx->h_ppc_off[i + 1] - ctx->h_ppc_off[i];
  CHK(d2h_int(ctx, iatom_common_j, ctx->d_t_i, T, 1));
  CHK(d2h_int(ctx, iatom_common_b, ctx->d_t_ib, T, 0));
  CHK(d2h_int(ctx, jatom_common_j, ctx->d_t_j, T, 1));
  CHK(d2h_int(ctx, jatom_common_b, ctx->d_t_jb, T, 0));
  CHK(d2h_int(ctx, neigh_common, ctx->d_t_m, T, 1));
  CHK(d2h_int(ctx, m31, ctx->d_t_m31, T, 1));
  CHK(d2h_int(ctx, m32, ctx->d_t_m32, T, 1));
  return FB_OK;
}

int fb_get_ewald(fb_ctx *ctx, double *ewald) {
  if (!ctx || !ewald) return FB_ERR_ARG;
  if (!ctx->have_ewald) return fail(ctx, FB_ERR_STATE, "fb_assemble with FB_EWALD first");
  if (!ctx->ewald_matrix)
    return fail(ctx, FB_ERR_STATE, "no Ewald matrix: the Harris assemble_ewald only allocates zero ewaldsr / ewaldlr blocks");
  CU(cudaMemcpyAsync(ewald, ctx->d_ewald.p, (size_t)ctx->N * ctx->N * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FB_OK;
}

int fb_set_denmat_pp(fb_ctx *ctx, const double *rho_pp) {
  if (!ctx || !rho_pp) return FB_ERR_ARG;
  if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors_pp first");
  CU(cudaSetDevice(ctx->device));
  size_t bb = (size_t)ctx->nvnl * sizeof(double);
  CHK(ctx->d_rho_pp.ensure(bb + 8));
  CU(cudaMemcpyAsync(ctx->d_rho_pp.p, rho_pp, bb, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_rho_pp = true;
  return FB_OK;
}

int fb_set_denmat_pp_device(fb_ctx *ctx, const void *rho_pp_dev) {
  if (!ctx || !rho_pp_dev) return FB_ERR_ARG;
  if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors_pp first");
  CU(cudaSetDevice(ctx->device));
  size_t bb = (size_t)ctx->nvnl * sizeof(double);
  CHK(ctx->d_rho_pp.ensure(bb + 8));
  CU(cudaMemcpyAsync(ctx->d_rho_pp.p, rho_pp_dev, bb, cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->have_rho_pp = true;
  return FB_OK;
}

int fb_get_common(fb_ctx *ctx, int *ncommon, int *iatom_common_j, int *iatom_common_b, int *jatom_common_j,
                  int *jatom_common_b, int *neigh_common) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if (ncommon)
    for (int i = 0; i < ctx->N; i++) ncommon[i] = ctx->h_trip_off[i + 1] - ctx->h_trip_off[i];
  CHK(d2h_int(ctx, iatom_common_j, ctx->d_ci_j, ctx->T, 1));
  local_atoms(ctx, iatom_common_j, ctx->h_trip_off);
  CHK(d2h_int(ctx, iatom_common_b, ctx->d_ci_b, ctx->T, 0));
  CHK(d2h_int(ctx, jatom_common_j, ctx->d_cj_j, ctx->T, 1));
  local_atoms(ctx, jatom_common_j, ctx->h_trip_off);
  CHK(d2h_int(ctx, jatom_common_b, ctx->d_cj_b, ctx->T, 0));
  CHK(d2h_int(ctx, neigh_common, ctx->d_cneigh, ctx->T, 1));
  return FB_OK;
}

int fb_get_batch(const fb_ctx *ctx, int *atom_off, int *pair_off, int *trip_off, long long *block_off) {
  if (!ctx) return FB_ERR_ARG;
  if (ctx->nstruct < 1) return FB_ERR_STATE;
  if ((pair_off || trip_off || block_off) && !ctx->have_neigh) return FB_ERR_STATE;
  for (int s = 0; s <= ctx->nstruct; s++) {
    int a = ctx->h_satom_off[s];
    if (atom_off) atom_off[s] = a;
    if (pair_off) pair_off[s] = ctx->h_pair_off[a];
    if (trip_off) trip_off[s] = ctx->h_trip_off[a];
  }
  if (block_off)
    for (int s = 0; s <= ctx->nstruct; s++) block_off[s] = ctx->h_blk_base[ctx->h_satom_off[s]];
  return FB_OK;
}

static AsmArgs asm_args(fb_ctx *ctx) {
  AsmArgs a{};
  a.N = ctx->N;
  a.ntrip = ctx->T;
  a.have_d = ctx->fdh.have_d;
  a.P = ctx->P;
  a.pair_owner = ctx->d_pair_owner.as<int>();
  a.ratom = ctx->d_ratom.as<double>();
  a.sid = ctx->d_sid.as<int>();
  a.isp = ctx->d_isp.as<int>();
  a.fd = ctx->d_fd.as<FdataDev>();
  a.table2c = ctx->d_tab2.as<double>();
  a.table3c = ctx->d_tab3.as<double>();
  a.lin = ctx->d_lin.as<unsigned char>();
  a.gxy = ctx->d_gxy.as<double>();
  a.xl = ctx->d_xl.as<double>();
  a.pair_off = ctx->d_pair_off.as<int>();
  a.neigh_j = ctx->d_neigh_j.as<int>();
  a.neigh_b = ctx->d_neigh_b.as<int>();
  a.neigh_self = ctx->d_neigh_self.as<int>();
  a.neigh_back = ctx->d_neigh_back.as<int>();
  a.blk_off = ctx->d_blk_off.as<long long>();
  a.trip_alpha = ctx->d_talpha.as<int>();
  a.ci_j = ctx->d_ci_j.as<int>();
  a.ci_b = ctx->d_ci_b.as<int>();
  a.cj_j = ctx->d_cj_j.as<int>();
  a.cj_b = ctx->d_cj_b.as<int>();
  a.tdst = ctx->d_tdst.as<int>();
  a.tperm = ctx->d_tperm.as<int>();
  a.S = ctx->d_S.as<double>();
  a.T = ctx->d_T.as<double>();
  a.vb = ctx->d_vb.as<double>();
  a.vbo = ctx->d_vbo.as<double>();
  a.rho = ctx->d_rho.as<double>();
  a.cape = ctx->d_cape.as<double>();
  a.dS = ctx->d_dS.as<double>();
  a.dT = ctx->d_dT.as<double>();
  a.sumT = ctx->d_sumT.as<double>();
  a.sumS = ctx->d_sumS.as<double>();
  a.ontop = ctx->d_ontop.as<double>();
  a.atomf = ctx->d_atomf.as<double>();
  a.f3naa = ctx->d_f3a.as<double>();
  a.f3nab = ctx->d_f3b.as<double>();
  a.f3nac = ctx->d_f3c.as<double>();
  a.kin = ctx->d_kin.as<double>();
  a.vna = ctx->d_vna.as<double>();
  a.pul = ctx->d_pul.as<double>();
  a.ftot = ctx->d_ftot.as<double>();
  a.status = ctx->d_status.as<unsigned>();
  a.table3c_df = ctx->d_tab3df.as<float2>();
  a.rho_df = ctx->d_rho_df.as<float2>();
  a.cfg_a2c = ctx->cfg[TK_A2C];
  a.cfg_a3c = ctx->cfg[TK_A3C];
  a.cfg_d2c = ctx->cfg[TK_D2C];
  a.cfg_d3c = ctx->cfg[TK_D3C];
  a.queue = ctx->d_queue.as<int>();
  a.dogs = ctx->theory == FB_THEORY_DOGS;
  a.dq = ctx->d_dq.as<double>();
  a.dip = ctx->d_dip.as<double>();
  a.dogs_ps = ctx->d_dogs_ps.as<double>();
  return a;
}

static VxcArgs vxc_args(fb_ctx *ctx) {
  VxcArgs v{};
  v.a = asm_args(ctx);
  v.rho_in = ctx->d_rho_in.as<double>();
  v.rho_bond = ctx->d_rho_bond.as<double>();
  v.wrho_in = ctx->d_wrho_in.as<double>();
  v.wrho_bond = ctx->d_wrho_bond.as<double>();
  v.vxc = ctx->d_vxc.as<double>();
  v.off = ctx->d_vxc_off.as<double>();
  v.on = ctx->d_vxc_on.as<double>();
  v.wd = ctx->d_vxc_wd.as<double>();
  v.gd = ctx->d_vxc_gd.as<double>();
  v.f3a = ctx->d_f3xa.as<double>();
  v.f3b = ctx->d_f3xb.as<double>();
  v.f3c = ctx->d_f3xc.as<double>();
  v.fvxc = ctx->d_fvxc.as<double>();
  v.qsum_all = ctx->fdh.dev.vxc_qsum_all;
  return v;
}

extern "C++" {
// device arguments of the vnl kernels
static PPArgs pp_args(fb_ctx *ctx) {
  PPArgs a{};
  a.N = ctx->N;
  a.ratom = ctx->d_ratom.as<double>();
  a.pos4 = ctx->d_pos4.as<float4>();
  a.sid = ctx->d_sid.as<int>();
  a.isp = ctx->d_isp.as<int>();
  a.fd = ctx->d_fd.as<FdataDev>();
  a.table2c = ctx->d_tab2.as<double>();
  a.xl = ctx->d_xl.as<double>();
  a.xlf = ctx->d_xlf.as<float>();
  a.satom_off = ctx->d_satom_off.as<int>();
  a.simg_off = ctx->d_simg_off.as<int>();
  a.imgs = ctx->d_imgs.as<int>();
  a.sbbox = ctx->d_sbbox.as<float4>();
  double ra = 0.0, rp = 0.0;
  int have_d = ctx->fdh.have_d;
  for (int k = 0; k < ctx->fdh.nspecies; k++) {
    ra = std::max(ra, ctx->fdh.sp[k].rcA);
    rp = std::max(rp, ctx->fdh.sp[k].rc_pp);
    if (ctx->fdh.sp[k].pattern_pp() == PAT_SPD) have_d = 1;
  }
  a.reach = (float)(ra + rp);
  a.have_d = have_d;
  a.pp_cnt = ctx->d_pp_cnt.as<int>();
  a.svnl_sum = ctx->d_svnl_sum.as<long long>();
  a.pp_off = ctx->d_pp_off.as<int>();
  a.svnl_base = ctx->d_svnl_base.as<long long>();
  a.pp_j = ctx->d_pp_j.as<int>();
  a.pp_b = ctx->d_pp_b.as<int>();
  a.pp_self = ctx->d_pp_self.as<int>();
  a.pp_map = ctx->d_pp_map.as<int>();
  a.svnl_off = ctx->d_svnl_off.as<long long>();
  a.ppx_cnt = ctx->d_ppx_cnt.as<int>();
  a.ppx_off = ctx->d_ppx_off.as<int>();
  a.ppx_j = ctx->d_ppx_j.as<int>();
  a.ppx_b = ctx->d_ppx_b.as<int>();
  a.ppx_self = ctx->d_ppx_self.as<int>();
  a.ppx_map = ctx->d_ppx_map.as<int>();
  a.ppx_point = ctx->d_ppx_point.as<int>();
  a.ub = ctx->d_ub.as<int>();
  a.slot_off = ctx->d_pslot_off.as<long long>();
  a.slot_j = ctx->d_pslot_j.as<int>();
  a.slot_b = ctx->d_pslot_b.as<int>();
  a.ppp_cnt = ctx->d_ppp_cnt.as<int>();
  a.vnl_sum = ctx->d_vnl_sum.as<long long>();
  a.ppp_off = ctx->d_ppp_off.as<int>();
  a.vnl_base = ctx->d_vnl_base.as<long long>();
  a.ppp_j = ctx->d_ppp_j.as<int>();
  a.ppp_b = ctx->d_ppp_b.as<int>();
  a.ppp_self = ctx->d_ppp_self.as<int>();
  a.vnl_off = ctx->d_vnl_off.as<long long>();
  a.ppc_cnt = ctx->d_ppc_cnt.as<int>();
  a.ppc_off = ctx->d_ppc_off.as<int>();
  a.t_alpha = ctx->d_t_alpha.as<int>();
  a.t_i = ctx->d_t_i.as<int>();
  a.t_ib = ctx->d_t_ib.as<int>();
  a.t_j = ctx->d_t_j.as<int>();
  a.t_jb = ctx->d_t_jb.as<int>();
  a.t_m = ctx->d_t_m.as<int>();
  a.t_m31 = ctx->d_t_m31.as<int>();
  a.t_m32 = ctx->d_t_m32.as<int>();
  a.svnl = ctx->d_svnl.as<double>();
  a.dsvnl = ctx->d_dsvnl.as<double>();
  a.vnl = ctx->d_vnl.as<double>();
  a.rho_pp = ctx->d_rho_pp.as<double>();
  a.vnl_atom = ctx->d_vnl_atom.as<double>();
  a.vnl_ontop = ctx->d_vnl_ontop.as<double>();
  a.f3nla = ctx->d_f3nla.as<double>();
  a.f3nlb = ctx->d_f3nlb.as<double>();
  a.f3nlc = ctx->d_f3nlc.as<double>();
  a.fvnl = ctx->d_fvnl.as<double>();
  a.ftot = ctx->d_ftot.as<double>();
  a.status = ctx->d_status.as<unsigned>();
  a.errinfo = ctx->d_errinfo.as<int>();
  return a;
}
}  // extern "C++"

extern "C++" {
extern "C++" {
// the reciprocal and lattice sums of assemble_ewald (M_assemble_ewald_DOGS.f90:
// 640-700), built on the host exactly as the reference builds them: the cell
// volume and reciprocal vectors, kappa = (gmin^2 / (4 rmin^2))^(1/4), the
// g box (g != 0) with stuff = 4 pi exp(-g^2 / 4 kappa^2) / (g^2 V), and the L
// box; a cluster has no g terms, only L = 0 and kappa = 0.
static int ewald_setup(fb_ctx *ctx) {
  const double pi = 3.141592653589793238462643;
  const double *lat = &ctx->h_lat[0];
  double a1[3] = {lat[0], lat[1], lat[2]}, a2[3] = {lat[3], lat[4], lat[5]}, a3[3] = {lat[6], lat[7], lat[8]};
  auto cross = [](const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  auto mag2 = [](const double *a) {
    double m = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    return m * m;
  };
  double c[3], g1[3], g2[3], g3[3];
  cross(a2, a3, c);
  double volume = a1[0] * c[0] + a1[1] * c[1] + a1[2] * c[2];
  for (int k = 0; k < 3; k++) g1[k] = 2.0 * pi * c[k] / volume;
  cross(a3, a1, c);
  for (int k = 0; k < 3; k++) g2[k] = 2.0 * pi * c[k] / volume;
  cross(a1, a2, c);
  for (int k = 0; k < 3; k++) g3[k] = 2.0 * pi * c[k] / volume;
  volume = std::fabs(volume);
  std::vector<double> gv, st, lv;
  double kappa = 0.0;
  if (ctx->h_icl[0] == 1) {
    lv = {0.0, 0.0, 0.0};
  } else {
    double gmax = 5.0, rmax = 5.0;
    double g1m2 = mag2(g1), g2m2 = mag2(g2), g3m2 = mag2(g3), r1m2 = mag2(a1), r2m2 = mag2(a2), r3m2 = mag2(a3);
    double rmin2 = std::min(r1m2, std::min(r2m2, r3m2)), gmin2 = std::min(g1m2, std::min(g2m2, g3m2));
    kappa = std::sqrt(std::sqrt(gmin2 / (4.0 * rmin2)));
    auto box = [](double v) {
      int n = (int)(v + 1.0);
      return n <= 1 ? 2 : n;
    };
    int ig1 = box(gmax * std::sqrt(4.0 * kappa * kappa / g1m2)), ig2 = box(gmax * std::sqrt(4.0 * kappa * kappa / g2m2)),
        ig3 = box(gmax * std::sqrt(4.0 * kappa * kappa / g3m2));
    int il1 = box(rmax * std::sqrt(1.0 / (kappa * kappa * r1m2))), il2 = box(rmax * std::sqrt(1.0 / (kappa * kappa * r2m2))),
        il3 = box(rmax * std::sqrt(1.0 / (kappa * kappa * r3m2)));
    for (int n1 = -ig1; n1 <= ig1; n1++)
      for (int n2 = -ig2; n2 <= ig2; n2++)
        for (int n3 = -ig3; n3 <= ig3; n3++) {
          if (n1 == 0 && n2 == 0 && n3 == 0) continue;
          double g[3];
          for (int k = 0; k < 3; k++) g[k] = n1 * g1[k] + n2 * g2[k] + n3 * g3[k];
          double gm2 = mag2(g);
          gv.insert(gv.end(), g, g + 3);
          st.push_back(4.0 * pi * std::exp(-gm2 / (4.0 * kappa * kappa)) / (gm2 * volume));
        }
    for (int n1 = -il1; n1 <= il1; n1++)
      for (int n2 = -il2; n2 <= il2; n2++)
        for (int n3 = -il3; n3 <= il3; n3++)
          for (int k = 0; k < 3; k++) lv.push_back(n1 * a1[k] + n2 * a2[k] + n3 * a3[k]);
  }
  ctx->ew_ng = (int)st.size();
  ctx->ew_nl = (int)(lv.size() / 3);
  ctx->ew_kappa = kappa;
  CHK(ctx->d_ew_sfc.ensure((size_t)ctx->N * ctx->ew_ng * sizeof(double) + 8));
  CHK(ctx->d_ew_sfs.ensure((size_t)ctx->N * ctx->ew_ng * sizeof(double) + 8));
  CHK(ctx->d_ew_g.ensure(gv.size() * sizeof(double) + 8));
  CHK(ctx->d_ew_stuff.ensure(st.size() * sizeof(double) + 8));
  CHK(ctx->d_ew_l.ensure(lv.size() * sizeof(double) + 8));
  if (!gv.empty()) {
    CU(cudaMemcpy(ctx->d_ew_g.p, gv.data(), gv.size() * sizeof(double), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(ctx->d_ew_stuff.p, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  CU(cudaMemcpy(ctx->d_ew_l.p, lv.data(), lv.size() * sizeof(double), cudaMemcpyHostToDevice));
  // hi/lo float pairs of the lattice vectors for the double-float sums
  std::vector<float> lf(2 * lv.size());
  for (size_t q = 0; q < lv.size(); q++) {
    float hi = (float)lv[q];
    lf[2 * q] = hi;
    lf[2 * q + 1] = (float)(lv[q] - (double)hi);
  }
  CHK(ctx->d_ew_ldf.ensure(lf.size() * sizeof(float) + 8));
  CU(cudaMemcpy(ctx->d_ew_ldf.p, lf.data(), lf.size() * sizeof(float), cudaMemcpyHostToDevice));
  return FB_OK;
}

static EwaldArgs ewald_args(fb_ctx *ctx) {
  EwaldArgs e{};
  e.N = ctx->N;
  e.T = ctx->T;
  e.ratom = ctx->d_ratom.as<double>();
  e.sid = ctx->d_sid.as<int>();
  e.isp = ctx->d_isp.as<int>();
  e.fd = ctx->d_fd.as<FdataDev>();
  e.xl = ctx->d_xl.as<double>();
  e.ng = ctx->ew_ng;
  e.nl = ctx->ew_nl;
  e.df = ctx->prec == FB_PREC_DF;
  e.lvec_df = ctx->d_ew_ldf.as<float2>();
  e.gvec = ctx->d_ew_g.as<double>();
  e.stuff = ctx->d_ew_stuff.as<double>();
  e.lvec = ctx->d_ew_l.as<double>();
  e.kappa = ctx->ew_kappa;
  e.pair_off = ctx->d_pair_off.as<int>();
  e.neigh_j = ctx->d_neigh_j.as<int>();
  e.neigh_b = ctx->d_neigh_b.as<int>();
  e.neigh_self = ctx->d_neigh_self.as<int>();
  e.blk_off = ctx->d_blk_off.as<long long>();
  e.trip_alpha = ctx->d_talpha.as<int>();
  e.ci_j = ctx->d_ci_j.as<int>();
  e.ci_b = ctx->d_ci_b.as<int>();
  e.cj_j = ctx->d_cj_j.as<int>();
  e.cj_b = ctx->d_cj_b.as<int>();
  e.tdst = ctx->d_tdst.as<int>();
  e.dq = ctx->d_dq.as<double>();
  e.dqa = ctx->d_dqa.as<double>();
  e.sfc = ctx->d_ew_sfc.as<double>();
  e.sfs = ctx->d_ew_sfs.as<double>();
  e.ewald = ctx->d_ewald.as<double>();
  e.sum_ewald = ctx->d_sum_ewald.as<double>();
  e.S = ctx->d_S.as<double>();
  e.dip = ctx->d_dip.as<double>();
  e.sr = ctx->d_ewsr.as<double>();
  e.lr = ctx->d_ewlr.as<double>();
  e.dogs_ps = ctx->d_dogs_ps.as<double>();
  e.q0a = ctx->d_q0a.as<double>();
  e.dewald = ctx->d_dewald.as<double>();
  e.w = ctx->d_ew_w.as<double>();
  e.sum_dewald = ctx->d_sum_dewald.as<double>();
  e.cw = ctx->d_ew_cw.as<double>();
  e.fewald = ctx->d_fewald.as<double>();
  e.fsr = ctx->d_fsr.as<double>();
  e.flr = ctx->d_flr.as<double>();
  e.f3naa = ctx->d_f3a.as<double>();
  e.f3nab = ctx->d_f3b.as<double>();
  e.f3nac = ctx->d_f3c.as<double>();
  e.ftot = ctx->d_ftot.as<double>();
  e.pair_owner = ctx->d_pair_owner.as<int>();
  e.P = ctx->P;
  return e;
}

}  // extern "C++"

// count -> host prefix sum -> offsets on the device (n + 1 entries)
template <typename T>
static int host_scan(fb_ctx *ctx, const DevBuf &cnt, int n, std::vector<T> &off, DevBuf &d_off) {
  std::vector<T> c(n);
  CU(cudaMemcpyAsync(c.data(), cnt.p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  off.assign(n + 1, 0);
  for (int i = 0; i < n; i++) off[i + 1] = off[i] + c[i];
  CHK(d_off.ensure((n + 1) * sizeof(T)));
  CU(cudaMemcpyAsync(d_off.p, off.data(), (n + 1) * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return FB_OK;
}
}  // extern "C++"

// the double-float kernels carry the Harris terms only; DOGS runs in FP64
static bool use_df(const fb_ctx *ctx) {
  return ctx->prec == FB_PREC_DF && !ctx->fdh.have_d && ctx->theory == FB_THEORY_HARRIS;
}
// the DOGS three-center kernels in double-float
static bool use_df_dogs(const fb_ctx *ctx) {
  return ctx->prec == FB_PREC_DF && !ctx->fdh.have_d && ctx->theory == FB_THEORY_DOGS;
}

int fb_set_theory(fb_ctx *ctx, int theory) {
  if (!ctx || (theory != FB_THEORY_HARRIS && theory != FB_THEORY_DOGS)) return FB_ERR_ARG;
  if (theory == FB_THEORY_DOGS && (!ctx->have_fdata || !ctx->fdh.dev.have_dogs))
    return fail(ctx, FB_ERR_TABLE, "DOGS: the Fdata has no charged-shell sub-cells or no z-dipole table");
  if (theory != ctx->theory) {
    ctx->theory = theory;
    // vna blocks and forces of the other theory are stale
    ctx->have_vna2c = false;
    ctx->assembled &= ~(unsigned)(FB_VNA2C | FB_VNA3C);
    ctx->dassembled = 0;
  }
  return FB_OK;
}

int fb_set_charges(fb_ctx *ctx, const double *dq, int nssh_max) {
  if (!ctx || !dq || nssh_max < 1) return FB_ERR_ARG;
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  if (nssh_max > MAXSUB) return fail(ctx, FB_ERR_CAPACITY, "nssh_max = %d > %d", nssh_max, MAXSUB);
  CU(cudaSetDevice(ctx->device));
  int N = ctx->N;
  std::vector<double> h((size_t)N * MAXSUB, 0.0);
  for (int i = 0; i < N; i++) {
    int nssh = ctx->fdh.dev.sp[ctx->h_isp[i]].nssh;
    for (int k = 0; k < nssh_max; k++) {
      double v = dq[(size_t)i * nssh_max + k];
      if (!std::isfinite(v)) return fail(ctx, FB_ERR_ARG, "dQ(%d, %d) is not finite", k + 1, i + 1);
      if (k < nssh) h[(size_t)i * MAXSUB + k] = v;
    }
  }
  CHK(ctx->d_dq.ensure(h.size() * sizeof(double)));
  CU(cudaMemcpyAsync(ctx->d_dq.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_charges = true;
  return FB_OK;
}

int fb_set_precision(fb_ctx *ctx, int mode) {
  if (!ctx || (mode != FB_PREC_FP64 && mode != FB_PREC_DF)) return FB_ERR_ARG;
  ctx->prec = mode;
  return FB_OK;
}

// MLP-3c evaluation arguments for the first mlp_n triplets of tperm
static MlpEvalArgs mlp_eval_args(fb_ctx *ctx) {
  MlpEvalArgs m{};
  const MlpState &s = ctx->mlp;
  m.n = ctx->mlp_n;
  m.list = ctx->d_tperm.as<int>();
  m.wbf = s.wbf.as<__nv_bfloat16>();
  m.params = s.params.as<float>();
  m.o_emb = s.o_emb;
  m.o_b1 = s.o_b1;
  m.o_b2 = s.o_b2;
  m.o_b3 = s.o_b3;
  m.o_b4 = s.o_b4;
  m.scale = s.scale.as<float>();
  m.nsp = s.nsp;
  m.out = ctx->d_mlpF.as<float>();
  m.pts = nullptr;
  m.ptrip = nullptr;
  return m;
}

static int mlp_launch(fb_ctx *ctx, const MlpEvalArgs &m, const AsmArgs &a, bool tangents) {
  if (ctx->mlp_engine == FB_MLP_ENGINE_TC && !m.pts) {
    // inputs first, at full occupancy; the tensor-core kernel reads them
    MlpEvalArgs mp = m;
    mp.pts = ctx->d_mlp_pts.as<float>();
    mp.ptrip = ctx->d_mlp_ptrip.as<int>();
    int e = launch_mlp_points(m, a, ctx->d_pos4.as<float4>(), ctx->d_xlf.as<float>(), ctx->d_mlp_pts.as<float>(),
                              ctx->d_mlp_ptrip.as<int>(), ctx->stream);
    if (e) return e;
    ctx->launches++;
    return launch_mlp_tc(mp, a, tangents, ctx->nsm, ctx->stream);
  }
  if (ctx->mlp_engine == FB_MLP_ENGINE_TC) return launch_mlp_tc(m, a, tangents, ctx->nsm, ctx->stream);
  return launch_mlp_eval(m, a, tangents, ctx->nsm, ctx->stream);
}

static int prepare_mlp(fb_ctx *ctx, bool forces) {
  if (mlp_routes(ctx) && ctx->mlp_n > 0) {
    CHK(ctx->d_mlpF.ensure((size_t)ctx->mlp_n * (forces ? 4 : 1) * MLP_ME_STRIDE * sizeof(float)));
    CHK(ctx->d_mlp_pts.ensure((size_t)ctx->mlp_n * 3 * sizeof(float) + 16));
    CHK(ctx->d_mlp_ptrip.ensure((size_t)ctx->mlp_n * sizeof(int) + 16));
  }
  return FB_OK;
}

// launches of the value pass (no synchronization)
static int enqueue_assemble(fb_ctx *ctx, unsigned what) {
  AsmArgs a = asm_args(ctx);
  unsigned w2 = what & (FB_S | FB_T | FB_VNA2C | FB_DIPOLE);
  // DOGS: the vna 2c pass also writes the overlap and z-dipole blocks the
  // three-center terms read
  if (a.dogs && (w2 & FB_VNA2C)) w2 |= FB_S | FB_DIPOLE;
  if (w2) KL(KT_ASM2C, launch_assemble_2c(a, w2, ctx->stream));
  if (what & (FB_SVNL | FB_VNL2C | FB_VNL3C)) {
    PPArgs pa = pp_args(ctx);
    if (what & FB_SVNL) KL(KT_SVNL, launch_svnl(pa, ctx->npp, false, ctx->stream));
    if (what & FB_VNL2C) KL(KT_VNL2C, launch_vnl_2c(pa, ctx->stream));
    if (what & FB_VNL3C) KL(KT_VNL3C, launch_vnl_3c(pa, ctx->ntrip_pp, ctx->stream));
  }
  if (what & FB_VXC) {
    VxcArgs v = vxc_args(ctx);
    KL(KT_RHO2C, launch_rho_2c(v, ctx->stream));
    if (a.ntrip > 0) {
      if (use_df(ctx)) KL(KT_RHO3C, launch_rho_3c_df(v, ctx->stream));
      else KL(KT_RHO3C, launch_rho_3c(v, ctx->stream));
      if (!v.qsum_all) ctx->launches++;  // the triples without summed cells
    }
    KL(KT_VXC, launch_vxc(v, ctx->stream));
  }
  if ((what & FB_EWALD) && !a.dogs) {
    // Harris: assemble_ewaldsr / assemble_ewaldlr allocate zero blocks
    // (j.ASSEMBLERS/M_assemble_ewald_Harris.f90:92-239)
    size_t nb = (size_t)ctx->nblock * sizeof(double);
    CU(cudaMemsetAsync(ctx->d_ewsr.p, 0, nb, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_ewlr.p, 0, nb, ctx->stream));
  } else if (what & FB_EWALD) {
    EwaldArgs e = ewald_args(ctx);
    KL(KT_EWALD, launch_ewald_matrix(e, ctx->stream));
    if (e.ng > 0) ctx->launches++;  // structure factors + tiles
    KL(KT_EWALD_BLOCKS, launch_ewald_blocks(e, ctx->fdh.have_d, ctx->stream));
    ctx->launches += e.T > 0 ? 3 : 2;
  }
  if (what & FB_VNA3C) {
    // triplets of approved bins through the network, the rest through the tables
    int nm = mlp_routes(ctx) ? ctx->mlp_n : 0;
    AsmArgs at = table3c_view(ctx, a, nm);
    if (ctx->fuse3c) {
      // the force pass adds these triplets' value terms (enqueue_dassemble)
    } else if (use_df(ctx)) KL(KT_ASM3C, launch_assemble_3c_df(at, ctx->stream));
    else if (use_df_dogs(ctx)) KL(KT_ASM3C, launch_assemble_3c_dogs_df(at, ctx->stream));
    else KL(KT_ASM3C, launch_assemble_3c(at, ctx->stream));
    if (nm > 0 && !ctx->fuse3c) {
      // (fused step: the force pass's network evaluation gives the values
      // too, and its tail adds the value terms)
      KL(KT_MLP_EVAL, mlp_launch(ctx, mlp_eval_args(ctx), a, false));
      AsmArgs am = a;
      am.ntrip = nm;
      am.mlpF = ctx->d_mlpF.as<float>();
      KL(KT_ASM3C_MLP, launch_assemble_3c_mlp(am, ctx->stream));
    }
  }
  return FB_OK;
}

// state checks and the storage of the value pass (allocations happen here,
// never while a graph is being captured)
static int check_assemble(fb_ctx *ctx, unsigned what) {
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if ((what & FB_VNA3C) && !(what & FB_VNA2C) && !ctx->have_vna2c)
    return fail(ctx, FB_ERR_STATE, "assemble_vna_3c accumulates onto assemble_vna_2c blocks: assemble FB_VNA2C first");
  bool dogs = ctx->theory == FB_THEORY_DOGS;
  if (dogs && (what & (FB_VNA2C | FB_VNA3C)) && !ctx->have_charges)
    return fail(ctx, FB_ERR_STATE, "DOGS: fb_set_charges first");
  if ((what & FB_DIPOLE) && !ctx->fdh.dev.have_dogs)
    return fail(ctx, FB_ERR_TABLE, "FB_DIPOLE: the Fdata has no z-dipole table (dipole_z)");
  if ((what & FB_DIPOLE) || (dogs && (what & FB_VNA2C)))
    CHK(ctx->d_dip.ensure((size_t)ctx->nblock * sizeof(double) + 8));
  if ((what & FB_EWALD) && !dogs) {
    size_t nb = (size_t)ctx->nblock * sizeof(double) + 8;
    CHK(ctx->d_ewsr.ensure(nb));
    CHK(ctx->d_ewlr.ensure(nb));
  } else if (what & FB_EWALD) {
    if (!ctx->have_charges) return fail(ctx, FB_ERR_STATE, "Ewald: fb_set_charges first");
    if (ctx->nstruct != 1) return fail(ctx, FB_ERR_UNSUPPORTED, "Ewald: single structures (a batch of one)");
    if (!(what & FB_VNA2C) && !(ctx->have_dip && (ctx->assembled & FB_S)))
      return fail(ctx, FB_ERR_STATE, "Ewald reads the overlap and dipole blocks: assemble FB_VNA2C (DOGS) first");
    size_t nb = (size_t)ctx->nblock * sizeof(double) + 8, n = (size_t)ctx->N;
    CHK(ctx->d_ewald.ensure(n * n * sizeof(double) + 8));
    CHK(ctx->d_dqa.ensure(n * sizeof(double) + 8));
    CHK(ctx->d_sum_ewald.ensure(n * sizeof(double) + 8));
    CHK(ctx->d_ewsr.ensure(nb));
    CHK(ctx->d_ewlr.ensure(nb));
    CHK(ewald_setup(ctx));
  }
  if (what & FB_VXC) {
    if (dogs) return fail(ctx, FB_ERR_UNSUPPORTED, "vxc: this build assembles the McWEDA Harris exchange-correlation only");
    if (!ctx->fdh.dev.have_vxc)
      return fail(ctx, FB_ERR_TABLE, "vxc: the Fdata lacks McWEDA tables (vxc_ontop, den_*, denS_*, den3, denS3, vxc_1c)");
    if (!(what & FB_S) && !(ctx->assembled & FB_S))
      return fail(ctx, FB_ERR_STATE, "assemble_vxc reads the overlap blocks: assemble FB_S first");
    size_t nb = (size_t)ctx->nblock * sizeof(double) + 8, nw = (size_t)VXC_WSH * ctx->P * sizeof(double) + 8;
    CHK(ctx->d_rho_in.ensure(nb));
    CHK(ctx->d_rho_bond.ensure(nb));
    CHK(ctx->d_vxc.ensure(nb));
    CHK(ctx->d_wrho_in.ensure(nw));
    CHK(ctx->d_wrho_bond.ensure(nw));
  }
  if (what & (FB_SVNL | FB_VNL2C | FB_VNL3C)) {
    if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "vnl: fb_neighbors_pp first");
    if ((what & (FB_VNL2C | FB_VNL3C)) && !(what & FB_SVNL) && !(ctx->assembled & FB_SVNL))
      return fail(ctx, FB_ERR_STATE, "assemble_vnl reads the svnl blocks: assemble FB_SVNL first");
    if ((what & FB_VNL3C) && !(what & FB_VNL2C) && !(ctx->assembled & FB_VNL2C))
      return fail(ctx, FB_ERR_STATE, "assemble_vnl_3c accumulates onto assemble_vnl_2c blocks: assemble FB_VNL2C first");
    CHK(ctx->d_svnl.ensure((size_t)ctx->nsvnl * sizeof(double) + 8));
    CHK(ctx->d_vnl.ensure((size_t)ctx->nvnl * sizeof(double) + 8));
  }
  return FB_OK;
}

static void assemble_done(fb_ctx *ctx, unsigned what) {
  if (what & FB_VNA2C) ctx->have_vna2c = true;
  if ((what & FB_DIPOLE) || (ctx->theory == FB_THEORY_DOGS && (what & FB_VNA2C))) ctx->have_dip = true;
  ctx->assembled |= what & (FB_ALL | FB_DIPOLE | FB_SVNL | FB_VNL2C | FB_VNL3C | FB_VXC);
  if (what & FB_EWALD) {
    ctx->have_ewald = true;
    ctx->ewald_matrix = ctx->theory == FB_THEORY_DOGS;
  }
}

int fb_assemble(fb_ctx *ctx, unsigned what) {
  if (!ctx) return FB_ERR_ARG;
  CHK(check_assemble(ctx, what));
  CU(cudaSetDevice(ctx->device));
  if (what & FB_VNA3C) CHK(prepare_mlp(ctx, false));
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  CHK(enqueue_assemble(ctx, what));
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  assemble_done(ctx, what);
  return FB_OK;
}

static DevBuf *block_buf(fb_ctx *ctx, int which, size_t *n) {
  *n = (size_t)ctx->nblock;
  switch (which) {
    case FB_BLOCK_S: return &ctx->d_S;
    case FB_BLOCK_T: return &ctx->d_T;
    case FB_BLOCK_VNA: return &ctx->d_vb;
    case FB_BLOCK_VNAO: return &ctx->d_vbo;
    case FB_BLOCK_DS: *n *= 3; return ctx->have_dblocks ? &ctx->d_dS : nullptr;
    case FB_BLOCK_DT: *n *= 3; return ctx->have_dblocks ? &ctx->d_dT : nullptr;
    case FB_BLOCK_RHO: return ctx->have_rho ? &ctx->d_rho : nullptr;
    case FB_BLOCK_CAPE: return ctx->have_rho ? &ctx->d_cape : nullptr;
    case FB_BLOCK_DIP: return ctx->have_dip ? &ctx->d_dip : nullptr;
    case FB_BLOCK_SVNL: *n = (size_t)ctx->nsvnl; return (ctx->assembled & FB_SVNL) ? &ctx->d_svnl : nullptr;
    case FB_BLOCK_VNL: *n = (size_t)ctx->nvnl; return (ctx->assembled & FB_VNL2C) ? &ctx->d_vnl : nullptr;
    case FB_BLOCK_DSVNL: *n = (size_t)3 * ctx->nsvnl; return (ctx->dassembled & (FB_VNL2C | FB_VNL3C)) ? &ctx->d_dsvnl : nullptr;
    case FB_BLOCK_RHO_PP: *n = (size_t)ctx->nvnl; return ctx->have_rho_pp ? &ctx->d_rho_pp : nullptr;
    case FB_BLOCK_EWALDSR: return ctx->have_ewald ? &ctx->d_ewsr : nullptr;
    case FB_BLOCK_EWALDLR: return ctx->have_ewald ? &ctx->d_ewlr : nullptr;
    case FB_BLOCK_VXC: return (ctx->assembled & FB_VXC) ? &ctx->d_vxc : nullptr;
    case FB_BLOCK_RHO_IN: return (ctx->assembled & FB_VXC) ? &ctx->d_rho_in : nullptr;
    case FB_BLOCK_RHO_BOND: return (ctx->assembled & FB_VXC) ? &ctx->d_rho_bond : nullptr;
    case FB_BLOCK_WRHO_IN: *n = (size_t)VXC_WSH * ctx->P; return (ctx->assembled & FB_VXC) ? &ctx->d_wrho_in : nullptr;
    case FB_BLOCK_WRHO_BOND: *n = (size_t)VXC_WSH * ctx->P; return (ctx->assembled & FB_VXC) ? &ctx->d_wrho_bond : nullptr;
  }
  return nullptr;
}

int fb_get_blocks(fb_ctx *ctx, int which, double *out) {
  if (!ctx || !out) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  size_t n;
  DevBuf *b = block_buf(ctx, which, &n);
  if (!b) return fail(ctx, FB_ERR_STATE, "block set %d not available", which);
  CU(cudaMemcpyAsync(out, b->p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FB_OK;
}

int fb_device_blocks(fb_ctx *ctx, int which, void **dptr) {
  if (!ctx || !dptr) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  size_t n;
  DevBuf *b = block_buf(ctx, which, &n);
  if (!b) return fail(ctx, FB_ERR_STATE, "block set %d not available", which);
  *dptr = b->p;
  return FB_OK;
}

int fb_set_denmat(fb_ctx *ctx, const double *rho, const double *cape) {
  if (!ctx || !rho) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  CU(cudaSetDevice(ctx->device));
  size_t bb = (size_t)ctx->nblock * sizeof(double);
  CHK(ctx->d_rho.ensure(bb + 8));
  CHK(ctx->d_cape.ensure(bb + 8));
  CU(cudaMemcpyAsync(ctx->d_rho.p, rho, bb, cudaMemcpyHostToDevice, ctx->stream));
  if (cape) CU(cudaMemcpyAsync(ctx->d_cape.p, cape, bb, cudaMemcpyHostToDevice, ctx->stream));
  else CU(cudaMemsetAsync(ctx->d_cape.p, 0, bb, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_rho = true;
  return FB_OK;
}

int fb_set_denmat_device(fb_ctx *ctx, const void *rho_dev, const void *cape_dev) {
  if (!ctx || !rho_dev) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  CU(cudaSetDevice(ctx->device));
  size_t bb = (size_t)ctx->nblock * sizeof(double);
  CHK(ctx->d_rho.ensure(bb + 8));
  CHK(ctx->d_cape.ensure(bb + 8));
  CU(cudaMemcpyAsync(ctx->d_rho.p, rho_dev, bb, cudaMemcpyDeviceToDevice, ctx->stream));
  if (cape_dev) CU(cudaMemcpyAsync(ctx->d_cape.p, cape_dev, bb, cudaMemcpyDeviceToDevice, ctx->stream));
  else CU(cudaMemsetAsync(ctx->d_cape.p, 0, bb, ctx->stream));
  ctx->have_rho = true;
  return FB_OK;
}

// device storage of the force pass (allocations happen here, never while
// a graph is being captured)
static int prepare_dassemble(fb_ctx *ctx, unsigned what, bool graph_values = false, bool pairs_only = false) {
  // (pairs_only: the pair lists exist, the common-neighbor stage is still to
  // come; the storage allocated here depends on the pairs only)
  if (!ctx->have_neigh && !pairs_only) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if ((what & FB_ALL) && !ctx->have_rho) return fail(ctx, FB_ERR_STATE, "fb_set_denmat first");
  if (what & (FB_VNL2C | FB_VNL3C)) {
    if (!ctx->have_pp_neigh) return fail(ctx, FB_ERR_STATE, "vnl: fb_neighbors_pp first");
    if (!ctx->have_rho_pp) return fail(ctx, FB_ERR_STATE, "vnl: fb_set_denmat_pp first");
    // the svnl blocks: assembled before, or by the same graph's value pass
    if (!(what & FB_SVNL) && !(ctx->assembled & FB_SVNL))
      return fail(ctx, FB_ERR_STATE, "Dassemble_vnl reads the svnl blocks: assemble FB_SVNL first");
    size_t a3 = (size_t)3 * ctx->N * sizeof(double);
    CHK(ctx->d_dsvnl.ensure((size_t)3 * ctx->nsvnl * sizeof(double) + 8));
    CHK(ctx->d_vnl_atom.ensure((size_t)3 * ctx->npp * sizeof(double) + 8));
    CHK(ctx->d_vnl_ontop.ensure((size_t)3 * ctx->nppx * sizeof(double) + 8));
    DevBuf *bufs[] = {&ctx->d_f3nla, &ctx->d_f3nlb, &ctx->d_f3nlc, &ctx->d_fvnl};
    for (DevBuf *b : bufs) CHK(b->ensure(a3));
  }
  bool dogs = ctx->theory == FB_THEORY_DOGS;
  if (dogs && (what & (FB_VNA2C | FB_VNA3C)) && !ctx->have_charges)
    return fail(ctx, FB_ERR_STATE, "DOGS: fb_set_charges first");
  int N = ctx->N, P = ctx->P;
  size_t pb = (size_t)3 * P * sizeof(double) + 8, ab = (size_t)3 * N * sizeof(double);
  CHK(ctx->d_sumT.ensure(pb));
  CHK(ctx->d_sumS.ensure(pb));
  CHK(ctx->d_ontop.ensure(pb));
  CHK(ctx->d_atomf.ensure(pb));
  DevBuf *ab_bufs[] = {&ctx->d_f3a, &ctx->d_f3b, &ctx->d_f3c, &ctx->d_kin, &ctx->d_vna, &ctx->d_pul, &ctx->d_ftot};
  for (DevBuf *b : ab_bufs) CHK(b->ensure(ab));
  if (what & FB_KEEP_DBLOCKS) {
    size_t db = (size_t)3 * ctx->nblock * sizeof(double) + 8;
    CHK(ctx->d_dS.ensure(db));
    CHK(ctx->d_dT.ensure(db));
  }
  if ((what & FB_VNA3C) && (use_df(ctx) || use_df_dogs(ctx) || mlp_routes(ctx)))
    CHK(ctx->d_rho_df.ensure((size_t)ctx->nblock * sizeof(float2) + 16));
  if (what & FB_VNA3C) CHK(prepare_mlp(ctx, true));
  if (dogs && (what & (FB_VNA3C | FB_EWALD))) CHK(ctx->d_dogs_ps.ensure((size_t)8 * P * sizeof(double) + 8));
  if (what & FB_VXC) {
    if (dogs) return fail(ctx, FB_ERR_UNSUPPORTED, "vxc forces: this build assembles the McWEDA Harris exchange-correlation only");
    if (!ctx->have_rho) return fail(ctx, FB_ERR_STATE, "fb_set_denmat first");
    if (!(ctx->assembled & FB_VXC) && !(graph_values && (what & FB_VXC)))
      return fail(ctx, FB_ERR_STATE, "Dassemble_vxc reads the value pass: assemble FB_VXC first");
    CHK(ctx->d_vxc_off.ensure(pb));
    CHK(ctx->d_vxc_on.ensure(pb));
    CHK(ctx->d_vxc_wd.ensure((size_t)ctx->nblock * sizeof(double) + 8));
    CHK(ctx->d_vxc_gd.ensure((size_t)VXC_WSH * P * sizeof(double) + 8));
    DevBuf *b3[] = {&ctx->d_f3xa, &ctx->d_f3xb, &ctx->d_f3xc, &ctx->d_fvxc};
    for (DevBuf *b : b3) CHK(b->ensure(ab + 8));
  }
  if ((what & FB_EWALD) && !dogs) {
    // Harris: Dassemble_ewaldsr allocates zero pair forces, Dassemble_ewaldlr
    // does nothing (k.DASSEMBLERS/M_Dassemble_ewald_Harris.f90:94-160)
    CHK(ctx->d_fsr.ensure((size_t)3 * P * sizeof(double) + 8));
    CHK(ctx->d_flr.ensure((size_t)3 * N * sizeof(double) + 8));
    CHK(ctx->d_fewald.ensure((size_t)3 * N * sizeof(double) + 8));
  } else if (what & FB_EWALD) {
    if (!ctx->have_ewald && !(graph_values && (what & FB_EWALD)))
      return fail(ctx, FB_ERR_STATE, "Ewald forces read the Ewald matrix: assemble FB_EWALD first");
    size_t n = (size_t)N;
    CHK(ctx->d_q0a.ensure(n * sizeof(double) + 8));
    CHK(ctx->d_dewald.ensure(3 * n * n * sizeof(double) + 8));
    CHK(ctx->d_ew_w.ensure(n * sizeof(double) + 8));
    DevBuf *b3[] = {&ctx->d_sum_dewald, &ctx->d_ew_cw, &ctx->d_fewald, &ctx->d_flr};
    for (DevBuf *b : b3) CHK(b->ensure(3 * n * sizeof(double) + 8));
    CHK(ctx->d_fsr.ensure((size_t)3 * P * sizeof(double) + 8));
  }
  return FB_OK;
}

// clears and launches of the force pass (no synchronization).  phase 1 is
// the clears and the two-center kernel, which read the pair lists only;
// phase 2 the rest; phase 0 both.
static int enqueue_dassemble(fb_ctx *ctx, unsigned what, int phase = 0) {
  int N = ctx->N, P = ctx->P;
  size_t pb = (size_t)3 * P * sizeof(double) + 8, ab = (size_t)3 * N * sizeof(double);
  AsmArgs a = asm_args(ctx);
  a.keep_dblocks = (what & FB_KEEP_DBLOCKS) != 0;
  if (phase != 2) {
    CU(cudaMemsetAsync(ctx->d_f3a.p, 0, ab, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3b.p, 0, ab, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3c.p, 0, ab, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_sumT.p, 0, pb, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_sumS.p, 0, pb, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_ontop.p, 0, pb, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_atomf.p, 0, pb, ctx->stream));
    unsigned w2 = what & (FB_S | FB_T | FB_VNA2C);
    // DOGS: the 2c kernel also leaves the per-pair sums the 3c and Ewald kernels read
    if (a.dogs && (what & (FB_VNA3C | FB_EWALD))) w2 |= 8u;
    if (w2) KL(KT_DASM2C, launch_dassemble_2c(a, w2, ctx->stream));
  }
  if (phase == 1) return FB_OK;
  if ((what & FB_EWALD) && !a.dogs) {
    CU(cudaMemsetAsync(ctx->d_fsr.p, 0, (size_t)3 * P * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->d_flr.p, 0, (size_t)3 * N * sizeof(double), ctx->stream));
    CU(cudaMemsetAsync(ctx->d_fewald.p, 0, (size_t)3 * N * sizeof(double), ctx->stream));
  }
  if ((what & FB_EWALD) && a.dogs) {
    // Dassemble_ewald (dewald, the Ewald energy force, the katom sums) and
    // the ewaldsr three-center terms into f3na, before build_forces sums them
    EwaldArgs e = ewald_args(ctx);
    CU(cudaMemsetAsync(ctx->d_ew_w.p, 0, (size_t)N * sizeof(double), ctx->stream));
    KL(KT_EWALD, launch_dewald(e, ctx->stream));
    ctx->launches += e.ng > 0 ? 4 : 3;
    KL(KT_EWALD_BLOCKS, launch_ewald_f3c(e, ctx->stream));
  }
  if (what & FB_VNA3C) {
    int nm = mlp_routes(ctx) ? ctx->mlp_n : 0;
    AsmArgs at = table3c_view(ctx, a, nm);
    at.fuse_value = ctx->fuse3c;
    if (use_df(ctx) || use_df_dogs(ctx) || nm > 0) KL(KT_SPLIT_RHO, launch_split_rho(a, ctx->nblock, ctx->stream));
    if (use_df(ctx)) KL(KT_DASM3C, launch_dassemble_3c_df(at, ctx->stream));
    else if (use_df_dogs(ctx)) KL(KT_DASM3C, launch_dassemble_3c_dogs_df(at, ctx->stream));
    else KL(KT_DASM3C, launch_dassemble_3c(at, ctx->stream));
    if (nm > 0) {
      KL(KT_MLP_EVAL, mlp_launch(ctx, mlp_eval_args(ctx), a, true));
      AsmArgs am = a;
      am.ntrip = nm;
      am.mlpF = ctx->d_mlpF.as<float>();
      am.fuse_value = ctx->fuse3c;
      KL(KT_DASM3C_MLP, launch_dassemble_3c_mlp(am, ctx->stream));
    }
  }
  KL(KT_FORCES, launch_build_forces(a, what & FB_ALL, ctx->stream));
  if (what & (FB_VNL2C | FB_VNL3C)) {
    // vnl force pass (M_Dassemble_PP_2c.f90, M_Dassemble_PP_3c.f90) and its
    // build_forces terms, added into ftot
    PPArgs pa = pp_args(ctx);
    size_t a3 = (size_t)3 * N * sizeof(double);
    CU(cudaMemsetAsync(ctx->d_f3nla.p, 0, a3, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3nlb.p, 0, a3, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3nlc.p, 0, a3, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_fvnl.p, 0, a3, ctx->stream));
    KL(KT_DSVNL, launch_svnl(pa, ctx->npp, true, ctx->stream));
    if (what & FB_VNL2C) {
      KL(KT_DVNL2C, launch_dvnl_2c(pa, ctx->npp, ctx->nppx, ctx->stream));
    } else {
      CU(cudaMemsetAsync(ctx->d_vnl_atom.p, 0, (size_t)3 * ctx->npp * sizeof(double), ctx->stream));
      CU(cudaMemsetAsync(ctx->d_vnl_ontop.p, 0, (size_t)3 * ctx->nppx * sizeof(double), ctx->stream));
    }
    if (what & FB_VNL3C) KL(KT_DVNL3C, launch_dvnl_3c(pa, ctx->ntrip_pp, ctx->stream));
    KL(KT_VNLF, launch_pp_forces(pa, ctx->npp, ctx->nppx, ctx->stream));
    ctx->launches++;  // two kernels
  }
  if (what & FB_VXC) {
    // Dassemble_vxc (2c pair terms, then the three-center terms with the
    // per-pair weights the 2c kernel leaves) and its build_forces terms,
    // added into ftot
    VxcArgs v = vxc_args(ctx);
    v.a = a;
    KL(KT_DVXC2C, launch_dvxc_2c(v, ctx->stream));
    size_t a3 = (size_t)3 * N * sizeof(double);
    CU(cudaMemsetAsync(ctx->d_f3xa.p, 0, a3, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3xb.p, 0, a3, ctx->stream));
    CU(cudaMemsetAsync(ctx->d_f3xc.p, 0, a3, ctx->stream));
    if (a.ntrip > 0) {
      if (use_df(ctx)) KL(KT_DVXC3C, launch_dvxc_3c_df(v, ctx->stream));
      else KL(KT_DVXC3C, launch_dvxc_3c(v, ctx->stream));
      if (!v.qsum_all) ctx->launches++;
    }
    KL(KT_VXCF, launch_vxc_forces(v, ctx->stream));
  }
  if ((what & FB_EWALD) && a.dogs) {
    // Dassemble_ewaldsr / ewaldlr pair and atom forces and their
    // build_forces terms, added into ftot
    EwaldArgs e = ewald_args(ctx);
    KL(KT_EWALD_BLOCKS, launch_ewald_forces(e, ctx->stream));
    ctx->launches++;
  }
  return FB_OK;
}

static void dassemble_done(fb_ctx *ctx, unsigned what) {
  bool keep = (what & FB_KEEP_DBLOCKS) != 0;
  ctx->have_dblocks = keep && (what & FB_S) && (what & FB_T);
  ctx->dassembled = what & (FB_ALL | FB_VNL2C | FB_VNL3C | FB_EWALD | FB_VXC);
}

int fb_dassemble(fb_ctx *ctx, unsigned what) {
  if (!ctx) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  CHK(prepare_dassemble(ctx, what & ~FB_SVNL));
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  CHK(enqueue_dassemble(ctx, what));
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  dassemble_done(ctx, what);
  return FB_OK;
}

static bool same_cfg(const KCfg *a, const KCfg *b) {
  for (int k = 0; k < TK_N; k++)
    if (a[k].threads != b[k].threads || a[k].ctas_per_sm != b[k].ctas_per_sm || a[k].chunk != b[k].chunk)
      return false;
  return true;
}

// capture of the value pass (+ force pass) into one CUDA graph
static int capture_graph(fb_ctx *ctx, unsigned what) {
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  bool timing = ctx->timing;
  ctx->timing = false;  // no timing events inside the graph
  long long l0 = ctx->launches;
  CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int st = FB_OK;
  if (cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream) != cudaSuccess)
    st = fail(ctx, FB_ERR_CUDA, "graph capture: status clear");
  // one interpolation per triplet when the step computes values and forces
  ctx->fuse3c = (what & FB_VNA3C) && (what & FB_FORCES) && ctx->theory == FB_THEORY_HARRIS;
  if (!st && (what & (FB_ALL | FB_DIPOLE | FB_SVNL | FB_VNL2C | FB_VNL3C | FB_EWALD | FB_VXC))) st = enqueue_assemble(ctx, what);
  if (!st && (what & FB_FORCES)) st = enqueue_dassemble(ctx, what);
  ctx->fuse3c = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->timing = timing;
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return fail(ctx, FB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ctx->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    ctx->gexec = nullptr;
    return fail(ctx, FB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  ctx->g_launches = ctx->launches - l0;
  ctx->launches = l0;
  ctx->g_what = what;
  ctx->g_npp = ctx->npp;
  ctx->g_nppx = ctx->nppx;
  ctx->g_nppp = ctx->nppp;
  ctx->g_ntrip_pp = ctx->ntrip_pp;
  ctx->g_theory = ctx->theory;
  ctx->g_prec = ctx->prec;
  ctx->g_N = ctx->N;
  ctx->g_P = ctx->P;
  ctx->g_T = ctx->T;
  ctx->g_nblock = ctx->nblock;
  ctx->g_have_d = ctx->fdh.have_d;
  ctx->g_mlp_n = ctx->mlp_n;
  ctx->g_mlp_mode = ctx->mlp_mode;
  ctx->g_mlp_engine = ctx->mlp_engine;
  ctx->g_alloc = g_alloc_gen.load();
  ctx->g_stream = ctx->stream;
  for (int k = 0; k < TK_N; k++) ctx->g_cfg[k] = ctx->cfg[k];
  return FB_OK;
}

int fb_assemble_graph(fb_ctx *ctx, unsigned what) {
  if (!ctx) return FB_ERR_ARG;
  const unsigned vals = FB_ALL | FB_DIPOLE | FB_SVNL | FB_VNL2C | FB_VNL3C | FB_EWALD | FB_VXC;
  if (!(what & (vals | FB_FORCES))) return fail(ctx, FB_ERR_ARG, "nothing to assemble");
  CU(cudaSetDevice(ctx->device));
  if (what & vals) CHK(check_assemble(ctx, what));
  if (what & FB_VNA3C) CHK(prepare_mlp(ctx, (what & FB_FORCES) != 0));
  if (what & FB_FORCES) CHK(prepare_dassemble(ctx, what, true));
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  bool fresh = ctx->gexec && ctx->g_what == what && ctx->g_theory == ctx->theory && ctx->g_prec == ctx->prec &&
               ctx->g_npp == ctx->npp && ctx->g_nppx == ctx->nppx && ctx->g_nppp == ctx->nppp &&
               ctx->g_ntrip_pp == ctx->ntrip_pp && ctx->g_N == ctx->N &&
               ctx->g_P == ctx->P && ctx->g_T == ctx->T && ctx->g_nblock == ctx->nblock &&
               ctx->g_have_d == ctx->fdh.have_d && ctx->g_alloc == g_alloc_gen.load() &&
               ctx->g_mlp_n == ctx->mlp_n && ctx->g_mlp_mode == ctx->mlp_mode &&
               ctx->g_mlp_engine == ctx->mlp_engine &&
               ctx->g_stream == ctx->stream && same_cfg(ctx->g_cfg, ctx->cfg);
  if (!fresh) CHK(capture_graph(ctx, what));
  CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
  ctx->launches += ctx->g_launches;
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (st) return status_error(ctx, st);
  assemble_done(ctx, what);
  if (what & FB_FORCES) dassemble_done(ctx, what);
  return FB_OK;
}

// ---------------------------------------------------------------------------
// launch shapes and the autotuner
// ---------------------------------------------------------------------------
static int tk_index(const char *kernel) {
  if (!kernel) return -1;
  for (int k = 0; k < TK_N; k++)
    if (std::strcmp(kernel, tk_names[k]) == 0) return k;
  return -1;
}

int fb_set_launch(fb_ctx *ctx, const char *kernel, int threads, int ctas_per_sm, int chunk) {
  if (!ctx) return FB_ERR_ARG;
  int k = tk_index(kernel);
  if (k < 0) return fail(ctx, FB_ERR_ARG, "no tunable kernel named %s", kernel ? kernel : "(null)");
  if (threads < 32 || threads > 256 || threads % 32 || ctas_per_sm < 0 || ctas_per_sm > 64 || chunk < 1 ||
      chunk > 4096)
    return fail(ctx, FB_ERR_ARG, "launch shape (%d threads, %d CTAs/SM, chunk %d) out of range", threads,
                ctas_per_sm, chunk);
  ctx->cfg[k] = KCfg{threads, ctas_per_sm, chunk, ctx->nsm};
  return FB_OK;
}

int fb_get_launch(const fb_ctx *ctx, const char *kernel, int *threads, int *ctas_per_sm, int *chunk) {
  if (!ctx) return FB_ERR_ARG;
  int k = tk_index(kernel);
  if (k < 0) return FB_ERR_ARG;
  if (threads) *threads = ctx->cfg[k].threads;
  if (ctas_per_sm) *ctas_per_sm = ctx->cfg[k].ctas_per_sm;
  if (chunk) *chunk = ctx->cfg[k].chunk;
  return FB_OK;
}

// one launch of tunable kernel k with shape c
static int tune_launch(fb_ctx *ctx, int k, const KCfg &c, unsigned what) {
  AsmArgs a = asm_args(ctx);
  a.keep_dblocks = false;
  switch (k) {
    case TK_A2C: {
      a.cfg_a2c = c;
      unsigned w2 = what & (FB_S | FB_T | FB_VNA2C);
      if (a.dogs && (w2 & FB_VNA2C)) w2 |= FB_S | FB_DIPOLE;
      return launch_assemble_2c(a, w2, ctx->stream);
    }
    case TK_A3C:
      a = table3c_view(ctx, a, 0);
      a.cfg_a3c = c;
      return use_df(ctx) ? launch_assemble_3c_df(a, ctx->stream) : launch_assemble_3c(a, ctx->stream);
    case TK_D2C: {
      a.cfg_d2c = c;
      unsigned w2 = what & (FB_S | FB_T | FB_VNA2C);
      if (a.dogs && (what & FB_VNA3C)) w2 |= 8u;
      return launch_dassemble_2c(a, w2, ctx->stream);
    }
    case TK_D3C:
      a = table3c_view(ctx, a, 0);
      a.cfg_d3c = c;
      return use_df(ctx) ? launch_dassemble_3c_df(a, ctx->stream) : launch_dassemble_3c(a, ctx->stream);
  }
  return 0;
}

int fb_autotune(fb_ctx *ctx, unsigned what, int reps, double *best_ms) {
  if (!ctx) return FB_ERR_ARG;
  if (reps < 1) reps = 1;
  CU(cudaSetDevice(ctx->device));
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  bool forces = (what & FB_FORCES) != 0;
  if (what & FB_ALL) CHK(check_assemble(ctx, (what & FB_ALL) | FB_VNA2C));
  if (forces) CHK(prepare_dassemble(ctx, what | FB_ALL));
  if (forces && (what & FB_VNA3C) && use_df(ctx)) {
    AsmArgs a = asm_args(ctx);
    KL(KT_SPLIT_RHO, launch_split_rho(a, ctx->nblock, ctx->stream));
  }
  if (best_ms)
    for (int k = 0; k < TK_N; k++) best_ms[k] = 0.0;
  bool tune[TK_N] = {(what & (FB_S | FB_T | FB_VNA2C)) != 0, (what & FB_VNA3C) != 0,
                     forces && (what & (FB_S | FB_T | FB_VNA2C)) != 0, forces && (what & FB_VNA3C) != 0};
  // candidates: a grid that covers the work, and persistent grids filling
  // 256 .. 2048 threads per SM, each at several chunk sizes
  std::vector<KCfg> cand;
  const int ths[3] = {64, 128, 256}, per_sm[4] = {256, 512, 1024, 2048}, chunks[3] = {1, 4, 16};
  for (int t : ths) {
    cand.push_back(KCfg{t, 0, 1, ctx->nsm});
    for (int ps : per_sm)
      for (int ch : chunks)
        if (ps >= t) cand.push_back(KCfg{t, ps / t, ch, ctx->nsm});
  }
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  int rc = FB_OK;
  for (int k = 0; k < TK_N && rc == FB_OK; k++) {
    if (!tune[k]) continue;
    float best = 3.0e38f;
    KCfg bestc = ctx->cfg[k];
    for (const KCfg &c : cand) {
      int e = tune_launch(ctx, k, c, what);  // warm-up
      for (int r = 0; r < reps && !e; r++) {
        if (r == 0) cudaEventRecord(e0, ctx->stream);
        e = tune_launch(ctx, k, c, what);
      }
      if (e) {
        rc = fail(ctx, FB_ERR_CUDA, "autotune %s: %s", tk_names[k], cudaGetErrorString((cudaError_t)e));
        break;
      }
      cudaEventRecord(e1, ctx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = fail(ctx, FB_ERR_CUDA, "autotune %s: synchronize", tk_names[k]);
        break;
      }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      ctx->launches += reps + 1;
      if (ms < best) {
        best = ms;
        bestc = c;
      }
    }
    ctx->cfg[k] = bestc;
    if (best_ms) best_ms[k] = best / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the timed launches accumulated into the outputs: they must be recomputed
  ctx->assembled = ctx->dassembled = 0;
  ctx->have_vna2c = ctx->have_dblocks = false;
  unsigned st = 0;
  CHK(sync_status(ctx, &st));
  if (rc) return rc;
  return FB_OK;
}

int fb_get_forces(fb_ctx *ctx, int which, double *out) {
  if (!ctx || !out) return FB_ERR_ARG;
  if (!ctx->dassembled) return fail(ctx, FB_ERR_STATE, "fb_dassemble first");
  DevBuf *b = nullptr;
  size_t n = (size_t)3 * ctx->N;
  switch (which) {
    case FB_F_TOT: b = &ctx->d_ftot; break;
    case FB_F_KINETIC: b = &ctx->d_kin; break;
    case FB_F_VNA: b = &ctx->d_vna; break;
    case FB_F_PULAY: b = &ctx->d_pul; break;
    case FB_F_F3NAA: b = &ctx->d_f3a; break;
    case FB_F_F3NAB: b = &ctx->d_f3b; break;
    case FB_F_F3NAC: b = &ctx->d_f3c; break;
    case FB_F_VNA_ONTOP: b = &ctx->d_ontop; n = (size_t)3 * ctx->P; break;
    case FB_F_VNA_ATOM: b = &ctx->d_atomf; n = (size_t)3 * ctx->P; break;
    case FB_F_VNL: b = &ctx->d_fvnl; break;
    case FB_F_F3NLA: b = &ctx->d_f3nla; break;
    case FB_F_F3NLB: b = &ctx->d_f3nlb; break;
    case FB_F_F3NLC: b = &ctx->d_f3nlc; break;
    case FB_F_VNL_ATOM: b = &ctx->d_vnl_atom; n = (size_t)3 * ctx->npp; break;
    case FB_F_VNL_ONTOP: b = &ctx->d_vnl_ontop; n = (size_t)3 * ctx->nppx; break;
    case FB_F_EWALDSR: b = &ctx->d_fsr; n = (size_t)3 * ctx->P; break;
    case FB_F_EWALDLR: b = &ctx->d_flr; break;
    case FB_F_EWALD: b = &ctx->d_fewald; break;
    case FB_F_VXC: b = &ctx->d_fvxc; break;
    case FB_F_F3XCA: b = &ctx->d_f3xa; break;
    case FB_F_F3XCB: b = &ctx->d_f3xb; break;
    case FB_F_F3XCC: b = &ctx->d_f3xc; break;
    case FB_F_VXC_OFF_SITE: b = &ctx->d_vxc_off; n = (size_t)3 * ctx->P; break;
    case FB_F_VXC_ON_SITE: b = &ctx->d_vxc_on; n = (size_t)3 * ctx->P; break;
    default: return fail(ctx, FB_ERR_ARG, "unknown force array %d", which);
  }
  if (which >= FB_F_VXC && !(ctx->dassembled & FB_VXC))
    return fail(ctx, FB_ERR_STATE, "vxc forces: fb_dassemble with FB_VXC first");
  if (which >= FB_F_EWALDSR && which <= FB_F_EWALD && !(ctx->dassembled & FB_EWALD))
    return fail(ctx, FB_ERR_STATE, "Ewald forces: fb_dassemble with FB_EWALD first");
  if (which >= FB_F_VNL && which <= FB_F_VNL_ONTOP && !(ctx->dassembled & (FB_VNL2C | FB_VNL3C)))
    return fail(ctx, FB_ERR_STATE, "vnl forces: fb_dassemble with FB_VNL2C / FB_VNL3C first");
  CU(cudaMemcpyAsync(out, b->p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FB_OK;
}

int fb_assemble_step(fb_ctx *ctx, const double *ratom, double *S, double *T, double *vna, double *vnao) {
  if (!ctx) return FB_ERR_ARG;
  int st;
  if (ratom && (st = fb_update_positions(ctx, ratom))) return st;
  if ((st = fb_neighbors(ctx))) return st;
  if ((st = fb_assemble(ctx, FB_ALL))) return st;
  if (S && (st = fb_get_blocks(ctx, FB_BLOCK_S, S))) return st;
  if (T && (st = fb_get_blocks(ctx, FB_BLOCK_T, T))) return st;
  if (vna && (st = fb_get_blocks(ctx, FB_BLOCK_VNA, vna))) return st;
  if (vnao && (st = fb_get_blocks(ctx, FB_BLOCK_VNAO, vnao))) return st;
  return FB_OK;
}

// the overlapped form of fb_step_forces: after the pair stage of the
// neighbor build, the two-center value and force kernels (which read the
// pair lists only) run on a second stream while the main stream runs the
// common-neighbor stage and its host synchronization; the fused three-center
// kernel and build_forces wait for both
static int step_overlapped(fb_ctx *ctx, const double *rho, const double *cape, unsigned what) {
  size_t bb = (size_t)ctx->nblock * sizeof(double);
  cudaStream_t main = ctx->stream;
  // (the status word keeps the pair stage's flags: finish_common checks them)
  CU(cudaEventRecord(ctx->ev_nb, main));
  // the density matrices travel on the copy stream
  CU(cudaMemcpyAsync(ctx->d_rho.p, rho, bb, cudaMemcpyHostToDevice, ctx->cstream));
  if (cape) CU(cudaMemcpyAsync(ctx->d_cape.p, cape, bb, cudaMemcpyHostToDevice, ctx->cstream));
  else CU(cudaMemsetAsync(ctx->d_cape.p, 0, bb, ctx->cstream));
  CU(cudaEventRecord(ctx->ev_in, ctx->cstream));
  // second stream: two-center value pass, then (with rho) the two-center
  // force kernel and the clears of the force accumulators
  ctx->stream = ctx->s2;
  int st = cudaStreamWaitEvent(ctx->s2, ctx->ev_nb, 0) == cudaSuccess ? FB_OK : fail(ctx, FB_ERR_CUDA, "event wait");
  if (!st) st = enqueue_assemble(ctx, what & (FB_S | FB_T | FB_VNA2C));
  if (!st && cudaEventRecord(ctx->ev_val, ctx->s2) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event record");
  if (!st && cudaStreamWaitEvent(ctx->s2, ctx->ev_in, 0) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event wait");
  if (!st) st = enqueue_dassemble(ctx, what, 1);
  if (!st && cudaEventRecord(ctx->ev_2c, ctx->s2) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event record");
  ctx->stream = main;
  // main stream: common neighbors and triplet bins, then the three-center
  // force kernel (with the value-pass terms) and build_forces
  if (!st) st = finish_common(ctx);
  ctx->have_rho = true;
  if (!st) st = check_assemble(ctx, what);
  if (!st && cudaStreamWaitEvent(main, ctx->ev_2c, 0) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event wait");
  ctx->fuse3c = true;
  if (!st) st = enqueue_dassemble(ctx, what, 2);
  ctx->fuse3c = false;
  if (st) {
    cudaStreamSynchronize(ctx->s2);
    cudaStreamSynchronize(ctx->cstream);
    cudaStreamSynchronize(main);
  }
  return st;
}

int fb_step_forces(fb_ctx *ctx, const double *ratom, const double *rho, const double *cape, double *S, double *T,
                   double *vna, double *vnao, double *ftot) {
  if (!ctx || !rho) return FB_ERR_ARG;
  if (ctx->theory != FB_THEORY_HARRIS) return fail(ctx, FB_ERR_UNSUPPORTED, "fb_step_forces: Harris only");
  if (ctx->N < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  CU(cudaSetDevice(ctx->device));
  if (!ctx->cstream) CU(cudaStreamCreateWithFlags(&ctx->cstream, cudaStreamNonBlocking));
  if (!ctx->s2) CU(cudaStreamCreateWithFlags(&ctx->s2, cudaStreamNonBlocking));
  cudaEvent_t *evs[] = {&ctx->ev_in, &ctx->ev_val, &ctx->ev_frc, &ctx->ev_nb, &ctx->ev_2c};
  for (cudaEvent_t *e : evs)
    if (!*e) CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  int st;
  if (ratom && (st = fb_update_positions(ctx, ratom))) return st;
  const unsigned what = FB_ALL;
  // per-kernel timing drains its events at each host synchronization of the
  // main stream, and the network routing sizes its storage from the triplet
  // bins: both take the serial order
  bool overlap = !ctx->timing && !mlp_routes(ctx);
  if (overlap) {
    if ((st = neighbors_pairs(ctx))) return st;
  } else if ((st = fb_neighbors(ctx))) {
    return st;
  }
  size_t bb = (size_t)ctx->nblock * sizeof(double);
  CHK(ctx->d_rho.ensure(bb + 8));
  CHK(ctx->d_cape.ensure(bb + 8));
  ctx->have_rho = true;
  if (overlap) {
    CHK(prepare_dassemble(ctx, what, true, true));
    if ((st = step_overlapped(ctx, rho, cape, what))) return st;
  } else {
    CHK(check_assemble(ctx, what));
    CHK(prepare_mlp(ctx, true));
    CHK(prepare_dassemble(ctx, what, true));
    // the density matrices travel on the copy stream while the value pass runs
    CU(cudaMemcpyAsync(ctx->d_rho.p, rho, bb, cudaMemcpyHostToDevice, ctx->cstream));
    if (cape) CU(cudaMemcpyAsync(ctx->d_cape.p, cape, bb, cudaMemcpyHostToDevice, ctx->cstream));
    else CU(cudaMemsetAsync(ctx->d_cape.p, 0, bb, ctx->cstream));
    CU(cudaEventRecord(ctx->ev_in, ctx->cstream));
    CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
    ctx->fuse3c = true;  // one interpolation per triplet, as in the graph step
    st = enqueue_assemble(ctx, what);
    if (!st && cudaEventRecord(ctx->ev_val, ctx->stream) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event record");
    if (!st && cudaStreamWaitEvent(ctx->stream, ctx->ev_in, 0) != cudaSuccess) st = fail(ctx, FB_ERR_CUDA, "event wait");
    if (!st) st = enqueue_dassemble(ctx, what);
    ctx->fuse3c = false;
    if (st) {
      cudaStreamSynchronize(ctx->cstream);
      cudaStreamSynchronize(ctx->stream);
      return st;
    }
  }
  CU(cudaEventRecord(ctx->ev_frc, ctx->stream));
  // S, T and vnao are final after the value pass: they travel back while
  // the force pass runs; vna (2c + 3c) and ftot after it
  CU(cudaStreamWaitEvent(ctx->cstream, ctx->ev_val, 0));
  if (S) CU(cudaMemcpyAsync(S, ctx->d_S.p, bb, cudaMemcpyDeviceToHost, ctx->cstream));
  if (T) CU(cudaMemcpyAsync(T, ctx->d_T.p, bb, cudaMemcpyDeviceToHost, ctx->cstream));
  if (vnao) CU(cudaMemcpyAsync(vnao, ctx->d_vbo.p, bb, cudaMemcpyDeviceToHost, ctx->cstream));
  CU(cudaStreamWaitEvent(ctx->cstream, ctx->ev_frc, 0));
  if (vna) CU(cudaMemcpyAsync(vna, ctx->d_vb.p, bb, cudaMemcpyDeviceToHost, ctx->cstream));
  if (ftot)
    CU(cudaMemcpyAsync(ftot, ctx->d_ftot.p, (size_t)3 * ctx->N * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->cstream));
  CU(cudaStreamSynchronize(ctx->cstream));
  unsigned stt = 0;
  CHK(sync_status(ctx, &stt));
  if (stt) return status_error(ctx, stt);
  assemble_done(ctx, what);
  dassemble_done(ctx, what);
  return FB_OK;
}

int fb_set_timing(fb_ctx *ctx, int enable) {
  if (!ctx) return FB_ERR_ARG;
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->pending.clear();
  ctx->timing = enable != 0;
  for (int k = 0; k < KT_N; k++) {
    ctx->kt_ms[k] = 0.0;
    ctx->kt_n[k] = 0;
  }
  return FB_OK;
}

int fb_get_timing(fb_ctx *ctx, const char *kernel, double *total_ms, long long *launches) {
  if (!ctx || !kernel) return FB_ERR_ARG;
  CU(cudaStreamSynchronize(ctx->stream));
  timing_drain(ctx);
  for (int k = 0; k < KT_N; k++)
    if (std::strcmp(kernel, kt_names[k]) == 0) {
      if (total_ms) *total_ms = ctx->kt_ms[k];
      if (launches) *launches = ctx->kt_n[k];
      return FB_OK;
    }
  return fail(ctx, FB_ERR_ARG, "unknown kernel name %s", kernel);
}

int fb_probe_fp32(fb_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  double ms = 0.0, flops = 0.0;
  int st = fb::probe_ffma(ctx->stream, &ms, &flops);
  if (st) return fail(ctx, FB_ERR_CUDA, "fp32 probe: %s", cudaGetErrorString((cudaError_t)st));
  ctx->launches += 2;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return FB_OK;
}

int fb_probe_fp64(fb_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  double ms = 0.0, flops = 0.0;
  int st = fb::probe_dfma(ctx->stream, &ms, &flops);
  if (st) return fail(ctx, FB_ERR_CUDA, "fp64 probe: %s", cudaGetErrorString((cudaError_t)st));
  ctx->launches += 2;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return FB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free force pass (fb_dassemble_noalloc).  Its scratch is this
// file-scope device array: per pair sumT, sumS, vna_ontop, vna_atom (12
// doubles), per atom f3naa, f3nab, f3nac, kinetic, vna, pulay (18 doubles).
// In host code the name g_noalloc_scratch is only a host-side stand-in, so
// the kernels get the device address from cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double
    g_noalloc_scratch[12 * FB_NOALLOC_MAX_PAIRS + 18 * FB_NOALLOC_MAX_ATOMS];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[128];  // device address per device ordinal

// once per device, with that device current (fb_create calls it)
static int noalloc_scratch(fb_ctx *ctx, double **out) {
  if (ctx->device < 0 || ctx->device >= 128) return fail(ctx, FB_ERR_ARG, "device ordinal %d", ctx->device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[ctx->device]) {
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(ctx, FB_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_noalloc_ptr[ctx->device] = p;
  }
  *out = g_noalloc_ptr[ctx->device];
  return FB_OK;
}

extern "C" int fb_dassemble_noalloc(fb_ctx *ctx, const double *rho_dev, const double *cape_dev, double *ftot_dev) {
  if (!ctx || !rho_dev || !ftot_dev) return FB_ERR_ARG;
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if (ctx->theory == FB_THEORY_DOGS)
    return fail(ctx, FB_ERR_UNSUPPORTED, "fb_dassemble_noalloc computes the Harris force pass only; use fb_dassemble for DOGS");
  int N = ctx->N, P = ctx->P;
  if (P > FB_NOALLOC_MAX_PAIRS || N > FB_NOALLOC_MAX_ATOMS)
    return fail(ctx, FB_ERR_CAPACITY,
                "fb_dassemble_noalloc handles at most %d pairs and %d atoms; this system has %d pairs, %d atoms",
                FB_NOALLOC_MAX_PAIRS, FB_NOALLOC_MAX_ATOMS, P, N);
  CU(cudaSetDevice(ctx->device));
  double *scr = nullptr;
  CHK(noalloc_scratch(ctx, &scr));
  AsmArgs a = asm_args(ctx);
  a.rho = rho_dev;
  a.cape = cape_dev;
  a.keep_dblocks = false;
  a.dS = a.dT = nullptr;
  double *pp = scr, *pa = scr + 12 * FB_NOALLOC_MAX_PAIRS;
  a.sumT = pp;
  a.sumS = pp + 3 * (size_t)P;
  a.ontop = pp + 6 * (size_t)P;
  a.atomf = pp + 9 * (size_t)P;
  a.f3naa = pa;
  a.f3nab = pa + 3 * (size_t)N;
  a.f3nac = pa + 6 * (size_t)N;
  a.kin = pa + 9 * (size_t)N;
  a.vna = pa + 12 * (size_t)N;
  a.pul = pa + 15 * (size_t)N;
  a.ftot = ftot_dev;
  // the three-center terms are accumulated with atomics: clear them (the
  // array keeps the previous call's values); every other term is overwritten
  CU(cudaMemsetAsync(a.f3naa, 0, 9 * (size_t)N * sizeof(double), ctx->stream));
  CU(cudaMemsetAsync(ctx->d_status.p, 0, sizeof(unsigned), ctx->stream));
  unsigned what = cape_dev ? FB_ALL : (FB_ALL & ~FB_S);
  int e;
  if ((e = launch_dassemble_2c(a, what & (FB_S | FB_T | FB_VNA2C), ctx->stream)))
    return fail(ctx, FB_ERR_CUDA, "launch dassemble_2c: %s", cudaGetErrorString((cudaError_t)e));
  if ((e = launch_dassemble_3c(a, ctx->stream)))
    return fail(ctx, FB_ERR_CUDA, "launch dassemble_3c: %s", cudaGetErrorString((cudaError_t)e));
  if ((e = launch_build_forces(a, what, ctx->stream)))
    return fail(ctx, FB_ERR_CUDA, "launch build_forces: %s", cudaGetErrorString((cudaError_t)e));
  ctx->launches += 3;
  unsigned st = 0;
  CU(cudaMemcpyAsync(&st, ctx->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (st) return status_error(ctx, st);
  return FB_OK;
}

// ---------------------------------------------------------------------------
// MLP-3c surrogate (fb_mlp_*)
// ---------------------------------------------------------------------------
static MlpTables mlp_tables(fb_ctx *ctx) {
  MlpTables t;
  t.fd = ctx->d_fd.as<FdataDev>();
  t.table3c = ctx->d_tab3.as<double>();
  t.gxy = ctx->d_gxy.as<double>();
  t.lin = ctx->d_lin.as<unsigned char>();
  return t;
}

extern "C" {

int fb_mlp_init(fb_ctx *ctx, unsigned long long seed) {
  if (!ctx) return FB_ERR_ARG;
  if (!ctx->have_fdata) return fail(ctx, FB_ERR_STATE, "fb_load_fdata first");
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = mlp_init(ctx->mlp, ctx->fdh, seed, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  return FB_OK;
}

long long fb_mlp_nparams(const fb_ctx *ctx) { return ctx && ctx->mlp.ready ? ctx->mlp.nparams : 0; }

int fb_mlp_layout(const fb_ctx *ctx, long long *offsets) {
  if (!ctx || !offsets) return FB_ERR_ARG;
  if (!ctx->mlp.ready) return FB_ERR_STATE;
  const MlpState &m = ctx->mlp;
  long long o[10] = {m.o_emb, m.o_w1, m.o_b1, m.o_w2, m.o_b2, m.o_w3, m.o_b3, m.o_w4, m.o_b4, m.nparams};
  std::memcpy(offsets, o, sizeof o);
  return FB_OK;
}

int fb_mlp_get_params(fb_ctx *ctx, float *out) {
  if (!ctx || !out) return FB_ERR_ARG;
  if (!ctx->mlp.ready) return fail(ctx, FB_ERR_STATE, "fb_mlp_init first");
  CU(cudaSetDevice(ctx->device));
  CU(cudaMemcpyAsync(out, ctx->mlp.params.p, ctx->mlp.nparams * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FB_OK;
}

int fb_mlp_scales(fb_ctx *ctx, float *out) {
  if (!ctx || !out) return FB_ERR_ARG;
  if (!ctx->mlp.ready) return fail(ctx, FB_ERR_STATE, "fb_mlp_init first");
  std::memcpy(out, ctx->mlp.h_scale.data(), ctx->mlp.h_scale.size() * sizeof(float));
  return FB_OK;
}

int fb_mlp_train(fb_ctx *ctx, long long nsamples, int epochs, int batch, double lr, unsigned long long seed,
                 double *loss_per_epoch) {
  if (!ctx) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = mlp_train(ctx->mlp, mlp_tables(ctx), nsamples, epochs, batch, lr, seed, loss_per_epoch, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  ctx->launches += (long long)epochs * (nsamples / std::max(batch, 1)) * 26;
  return FB_OK;
}

int fb_mlp_samples(fb_ctx *ctx, int n, unsigned long long seed, float *feat3, int *triple, float *target) {
  if (!ctx || n < 1 || !feat3 || !triple || !target) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = mlp_samples(ctx->mlp, mlp_tables(ctx), n, seed, feat3, triple, target, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  return FB_OK;
}

int fb_mlp_grad(fb_ctx *ctx, int n, const float *feat3, const int *triple, const float *target, float *grad,
                double *loss) {
  if (!ctx || !feat3 || !triple || !target || !grad || !loss) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = mlp_grad(ctx->mlp, n, feat3, triple, target, grad, loss, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  return FB_OK;
}

int fb_mlp_validate(fb_ctx *ctx, int samples_per_bin, unsigned long long seed, double *max_err) {
  if (!ctx || samples_per_bin < 1) return FB_ERR_ARG;
  if (!ctx->have_fdata) return fail(ctx, FB_ERR_STATE, "fb_load_fdata first");
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int cells = trip_cells(ctx);
  int st = mlp_validate(ctx->mlp, mlp_tables(ctx), samples_per_bin, cells, seed, ctx->h_bin_err, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  ctx->mlp_cells = cells;
  if (max_err) {
    double m = 0.0;
    for (float v : ctx->h_bin_err) m = std::max(m, (double)v);
    *max_err = m;
  }
  return FB_OK;
}

int fb_mlp_bin_errors(fb_ctx *ctx, float *out, long long *nbins) {
  if (!ctx) return FB_ERR_ARG;
  if (nbins) *nbins = (long long)ctx->h_bin_err.size();
  if (out) std::memcpy(out, ctx->h_bin_err.data(), ctx->h_bin_err.size() * sizeof(float));
  return FB_OK;
}

int fb_mlp_gate(fb_ctx *ctx, double tol_ha, double *tau, double *coverage) {
  if (!ctx || !(tol_ha > 0.0)) return FB_ERR_ARG;
  if (!ctx->mlp.ready) return fail(ctx, FB_ERR_STATE, "fb_mlp_init first");
  if (ctx->h_bin_err.empty()) return fail(ctx, FB_ERR_STATE, "fb_mlp_validate first");
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  CU(cudaSetDevice(ctx->device));
  // the most triplets that add into one block: count them per destination pair
  int T = ctx->T, nmax = 1;
  if (T > 0) {
    std::vector<int> tdst(T), cnt(ctx->P, 0);
    CU(cudaMemcpy(tdst.data(), ctx->d_tdst.p, T * sizeof(int), cudaMemcpyDeviceToHost));
    for (int t = 0; t < T; t++) nmax = std::max(nmax, ++cnt[tdst[t]]);
  }
  // |error of a block element| <= P_eq2 * 3 * nmax * (largest per-triplet
  // error of a molecular-frame element): rows and columns of a p-shell
  // rotation have 1-norms of at most sqrt(3) each
  double t_eV = tol_ha * P_Hartree;
  ctx->mlp_tau = t_eV / (P_eq2 * 3.0 * (double)nmax);
  size_t nb = ctx->h_bin_err.size();
  std::vector<unsigned char> ok(nb);
  for (size_t b = 0; b < nb; b++) ok[b] = ctx->h_bin_err[b] <= ctx->mlp_tau ? 1 : 0;
  CHK(ctx->d_binok.ensure(nb));
  CU(cudaMemcpy(ctx->d_binok.p, ok.data(), nb, cudaMemcpyHostToDevice));
  ctx->mlp_mode = FB_MLP_GATED;
  CHK(bin_triplets(ctx));
  CU(cudaStreamSynchronize(ctx->stream));
  if (tau) *tau = ctx->mlp_tau;
  if (coverage) *coverage = T > 0 ? (double)ctx->mlp_n / (double)T : 0.0;
  return FB_OK;
}

int fb_mlp_set_mode(fb_ctx *ctx, int mode) {
  if (!ctx || (mode != FB_MLP_OFF && mode != FB_MLP_GATED && mode != FB_MLP_ALL)) return FB_ERR_ARG;
  if (mode != FB_MLP_OFF && !ctx->mlp.ready) return fail(ctx, FB_ERR_STATE, "fb_mlp_init first");
  if (mode == FB_MLP_GATED && !ctx->d_binok.p) return fail(ctx, FB_ERR_STATE, "fb_mlp_gate first");
  if (mode != FB_MLP_OFF && ctx->fdh.have_d)
    return fail(ctx, FB_ERR_UNSUPPORTED, "MLP-3c covers s and sp bases");
  CU(cudaSetDevice(ctx->device));
  ctx->mlp_mode = mode;
  if (ctx->have_neigh) {
    CHK(bin_triplets(ctx));
    CU(cudaStreamSynchronize(ctx->stream));
  }
  return FB_OK;
}

int fb_mlp_eval_points(fb_ctx *ctx, int n, const float *pts, const int *triple, int derivs, float *out) {
  if (!ctx || n < 1 || !pts || !triple || !out) return FB_ERR_ARG;
  if (!ctx->mlp.ready) return fail(ctx, FB_ERR_STATE, "fb_mlp_init first");
  for (int i = 0; i < n; i++)
    if (triple[i] < 0 || triple[i] >= ctx->mlp.ntrip || ctx->mlp.h_nme[triple[i]] == 0)
      return fail(ctx, FB_ERR_ARG, "point %d: species triple %d has no table", i, triple[i]);
  CU(cudaSetDevice(ctx->device));
  int rows = derivs ? 4 : 1;
  DevBuf p, t, o;
  CHK(p.ensure((size_t)n * 3 * sizeof(float)));
  CHK(t.ensure((size_t)n * sizeof(int)));
  CHK(o.ensure((size_t)n * rows * MLP_ME_STRIDE * sizeof(float)));
  CU(cudaMemcpyAsync(p.p, pts, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(t.p, triple, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  int saved = ctx->mlp_n;
  ctx->mlp_n = n;
  MlpEvalArgs m = mlp_eval_args(ctx);
  ctx->mlp_n = saved;
  m.pts = p.as<float>();
  m.ptrip = t.as<int>();
  m.out = o.as<float>();
  AsmArgs a = asm_args(ctx);
  KL(KT_MLP_EVAL, mlp_launch(ctx, m, a, derivs != 0));
  CU(cudaMemcpyAsync(out, o.p, (size_t)n * rows * MLP_ME_STRIDE * sizeof(float), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  p.release();
  t.release();
  o.release();
  return FB_OK;
}

int fb_mlp_set_engine(fb_ctx *ctx, int engine) {
  if (!ctx || (engine != FB_MLP_ENGINE_MMA && engine != FB_MLP_ENGINE_TC)) return FB_ERR_ARG;
  ctx->mlp_engine = engine;
  return FB_OK;
}

int fb_mlp_routed(const fb_ctx *ctx, int *n_mlp, int *n_total) {
  if (!ctx) return FB_ERR_ARG;
  if (n_mlp) *n_mlp = mlp_routes(ctx) ? ctx->mlp_n : 0;
  if (n_total) *n_total = ctx->T;
  return FB_OK;
}

int fb_mlp_forward(fb_ctx *ctx, int n, const float *feat3, const int *triple, float *out) {
  if (!ctx || !feat3 || !triple || !out) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string e;
  int st = mlp_forward(ctx->mlp, n, feat3, triple, out, ctx->stream, e);
  if (st) return fail(ctx, st, "%s", e.c_str());
  return FB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Bloch sums into dense H(k), S(k) (fb_bloch, fb_bloch_device)
// ---------------------------------------------------------------------------
static int bloch_run(fb_ctx *ctx, int nk, const double *kpts, const double *extra_dev, double *Hk, double *Sk) {
  if (!ctx->have_neigh) return fail(ctx, FB_ERR_STATE, "fb_neighbors first");
  if (ctx->nstruct != 1) return fail(ctx, FB_ERR_UNSUPPORTED, "Bloch sums are per structure (a batch of one)");
  unsigned need = (Hk ? (FB_T | FB_VNA2C) : 0u) | (Sk ? FB_S : 0u);
  if ((ctx->assembled & need) != need) return fail(ctx, FB_ERR_STATE, "fb_assemble the S / T / vna blocks first");
  int N = ctx->N;
  std::vector<int> slot(N);
  long long n = 0;
  for (int i = 0; i < N; i++) {
    slot[i] = (int)n;
    n += ctx->fdh.sp[ctx->h_isp[i]].norb;
  }
  CHK(ctx->d_orb_slot.ensure(N * sizeof(int)));
  CU(cudaMemcpyAsync(ctx->d_orb_slot.p, slot.data(), N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  DevBuf dk;
  CHK(dk.ensure((size_t)nk * 3 * sizeof(double)));
  CU(cudaMemcpyAsync(dk.p, kpts, (size_t)nk * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  size_t bytes = (size_t)nk * 2 * n * n * sizeof(double);
  AsmArgs a = asm_args(ctx);
  if (Hk) {
    CU(cudaMemsetAsync(Hk, 0, bytes, ctx->stream));
    KL(KT_BLOCH, launch_bloch(a, ctx->P, nk, dk.as<double>(), ctx->d_pair_owner.as<int>(), ctx->d_r3v.as<double>(),
                              ctx->d_orb_slot.as<int>(), n, ctx->d_T.as<double>(), ctx->d_vb.as<double>(),
                              ctx->d_vbo.as<double>(), Hk, ctx->stream));
    if (extra_dev)
      KL(KT_BLOCH, launch_bloch(a, ctx->P, nk, dk.as<double>(), ctx->d_pair_owner.as<int>(), ctx->d_r3v.as<double>(),
                                ctx->d_orb_slot.as<int>(), n, extra_dev, nullptr, nullptr, Hk, ctx->stream));
  }
  if (Sk) {
    CU(cudaMemsetAsync(Sk, 0, bytes, ctx->stream));
    KL(KT_BLOCH, launch_bloch(a, ctx->P, nk, dk.as<double>(), ctx->d_pair_owner.as<int>(), ctx->d_r3v.as<double>(),
                              ctx->d_orb_slot.as<int>(), n, ctx->d_S.as<double>(), nullptr, nullptr, Sk, ctx->stream));
  }
  CU(cudaStreamSynchronize(ctx->stream));
  dk.release();
  return FB_OK;
}

extern "C" {

long long fb_norbitals(const fb_ctx *ctx) {
  if (!ctx || ctx->N < 1) return 0;
  long long n = 0;
  for (int i = 0; i < ctx->N; i++) n += ctx->fdh.sp[ctx->h_isp[i]].norb;
  return n;
}

int fb_bloch_device(fb_ctx *ctx, int nk, const double *kpts, const void *extra_dev, void *Hk_dev, void *Sk_dev) {
  if (!ctx || nk < 1 || !kpts || (!Hk_dev && !Sk_dev)) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  return bloch_run(ctx, nk, kpts, static_cast<const double *>(extra_dev), static_cast<double *>(Hk_dev),
                   static_cast<double *>(Sk_dev));
}

int fb_solve_k(fb_ctx *ctx, int nk, const double *kpts, const void *extra_dev, double *eigen, void *c_dev,
               int *dropped) {
  if (!ctx || nk < 1 || !kpts || !eigen) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  std::string why;
  if (!solver_available(why)) return fail(ctx, FB_ERR_UNSUPPORTED, "fb_solve_k: %s", why.c_str());
  long long n = fb_norbitals(ctx);
  if (n < 1) return fail(ctx, FB_ERR_STATE, "fb_set_structure first");
  if (n > 46340) return fail(ctx, FB_ERR_CAPACITY, "fb_solve_k handles at most 46340 orbitals (n^2 < 2^31)");
  size_t mb = (size_t)n * n * 2 * sizeof(double);
  CHK(ctx->d_sol_S.ensure(mb));
  CHK(ctx->d_sol_H.ensure(mb));
  CHK(ctx->d_sol_W.ensure(mb));
  CHK(ctx->d_sol_T.ensure(mb));
  CHK(ctx->d_sol_lam.ensure((size_t)n * sizeof(double)));
  CHK(ctx->d_sol_eps.ensure((size_t)n * sizeof(double)));
  CHK(ctx->d_sol_info.ensure(sizeof(int)));
  int lwork = 0;
  if (lowdin_work_size(ctx->solver, ctx->stream, (int)n, ctx->d_sol_S.as<double>(), ctx->d_sol_lam.as<double>(),
                       &lwork, why))
    return fail(ctx, FB_ERR_CUDA, "fb_solve_k: %s", why.c_str());
  CHK(ctx->d_sol_work.ensure((size_t)std::max(lwork, 1) * 2 * sizeof(double)));
  LowdinBufs b;
  b.Sk = ctx->d_sol_S.as<double>();
  b.Hk = ctx->d_sol_H.as<double>();
  b.W = ctx->d_sol_W.as<double>();
  b.T = ctx->d_sol_T.as<double>();
  b.lam = ctx->d_sol_lam.as<double>();
  b.eps = ctx->d_sol_eps.as<double>();
  b.work = ctx->d_sol_work.as<double>();
  b.lwork = lwork;
  b.info = ctx->d_sol_info.as<int>();
  for (int k = 0; k < nk; k++) {
    CHK(bloch_run(ctx, 1, kpts + 3 * k, static_cast<const double *>(extra_dev), b.Hk, b.Sk));
    double *c = c_dev ? static_cast<double *>(c_dev) + (size_t)k * 2 * n * n : nullptr;
    int rc = lowdin_solve(ctx->solver, ctx->stream, (int)n, b, eigen + (size_t)k * n, c,
                          dropped ? dropped + k : nullptr, why);
    ctx->launches += c ? 4 : 3;  // scaling kernel + library kernels not counted
    if (rc == -3) return fail(ctx, FB_ERR_SOLVER, "fb_solve_k, k-point %d: %s", k, why.c_str());
    if (rc) return fail(ctx, FB_ERR_CUDA, "fb_solve_k, k-point %d: %s", k, why.c_str());
  }
  return FB_OK;
}

int fb_bloch(fb_ctx *ctx, int nk, const double *kpts, double *Hk, double *Sk) {
  if (!ctx || nk < 1 || !kpts || (!Hk && !Sk)) return FB_ERR_ARG;
  CU(cudaSetDevice(ctx->device));
  long long n = fb_norbitals(ctx);
  size_t bytes = (size_t)nk * 2 * n * n * sizeof(double);
  DevBuf h, sb;
  if (Hk) CHK(h.ensure(bytes));
  if (Sk) CHK(sb.ensure(bytes));
  int st = bloch_run(ctx, nk, kpts, nullptr, Hk ? h.as<double>() : nullptr, Sk ? sb.as<double>() : nullptr);
  if (st) return st;
  if (Hk) CU(cudaMemcpy(Hk, h.p, bytes, cudaMemcpyDeviceToHost));
  if (Sk) CU(cudaMemcpy(Sk, sb.p, bytes, cudaMemcpyDeviceToHost));
  h.release();
  sb.release();
  return FB_OK;
}

}  // extern "C"
