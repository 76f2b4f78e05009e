// fb_mlp.h -- MLP-3c surrogate of the three-center table interpolation
// (host side).  No reference counterpart: the reference evaluates every
// three-center matrix element by interpolating its Fdata tables
// (getMEs_Fdata_3c, e.FDATA/M_Fdata_3c.f90:293-517).
//
// Network: inputs (2 x / xmax - 1, 2 y / ymax - 1, cos theta) of a triplet
// (each as a BF16 pair, high and low part) plus a 16-float embedding of its
// species triple (in1, in2, indna), three
// hidden layers of 128 with SiLU, 64 outputs of which 50 are used: the
// Legendre coefficient itheta = 1..5 of each of the (at most) 10 bcna matrix
// elements, output = (itheta - 1) * 10 + ime, divided by a per-output scale
// (the largest |table value| of that coefficient over the grid).  Weights
// and the activations fed to the tensor cores are BF16, accumulation FP32.
// Training data come from the FP64 table interpolator itself.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fb_devbuf.h"
#include "fb_fdata.h"

namespace fb {

constexpr int MLP_IN = 32;    // 3 coordinates + 16 embedding + zero padding
constexpr int MLP_EMB = 16;
constexpr int MLP_H = 128;
constexpr int MLP_OUT = 64;   // 5 theta x 10 ME used, padded
constexpr int MLP_ME = 10;    // matrix elements per Legendre term (sp x sp)
// the 3 coordinates enter twice: their BF16 roundings in columns 0..2 and the
// BF16 roundings of the remainders in columns MLP_LO..MLP_LO+2, both through
// the same (tied) weights, so the products see ~16-bit coordinates
constexpr int MLP_LO = 3 + MLP_EMB;

struct MlpState {
  bool ready = false;
  int nsp = 0, ntrip = 0;
  long long nparams = 0;
  // offsets (in floats) of the blocks of the parameter vector
  long long o_emb = 0, o_w1 = 0, o_b1 = 0, o_w2 = 0, o_b2 = 0, o_w3 = 0, o_b3 = 0, o_w4 = 0, o_b4 = 0;
  DevBuf params, grad, adam_m, adam_v;  // FP32 master parameters and Adam moments
  DevBuf wbf;                           // BF16 weights, plain and transposed
  DevBuf scale;                         // [ntrip][MLP_OUT] output scales
  DevBuf tmeta;                         // [ntrip] int: nME of the triple's bcna cell (0: no table)
  long long adam_t = 0;
  std::vector<float> h_scale;
  std::vector<int> h_nme;
  // training work space
  DevBuf dX, dXt, dY, dTrip;  // data set
  DevBuf Z, H, Ht, O, dO, dOt, dZ, dZt, dXg, part;
  int batch_cap = 0;
  long long data_cap = 0;
};

// MLP-3c evaluation for the assembly (fb_mlp_eval.cu): the first n
// triplets of the binned order through the network
struct MlpEvalArgs {
  int n;                     // triplets in the list
  const int *list;           // triplet indices (the binned order)
  const __nv_bfloat16 *wbf;  // BF16 weights: W1 [128][32], W2, W3 [128][128], W4 [64][128]
  const float *params;       // FP32 parameters (biases, embedding)
  long long o_emb, o_b1, o_b2, o_b3, o_b4;
  const float *scale;        // [ntrip][64]
  int nsp;
  float *out;                // [n][10] values, or [n][4][10]: F, dF/dcos, dF/dx, dF/dy
  // points instead of triplets (tests): pts [n][3] = (x, y, cos), ptrip [n]
  const float *pts;
  const int *ptrip;
};

// Device tables the sample generator interpolates (FP64, as assembled).
struct MlpTables {
  const FdataDev *fd;
  const double *table3c, *gxy;
  const unsigned char *lin;
};

// random parameters (seeded) and the output scales of the loaded Fdata
int mlp_init(MlpState &m, const FdataHost &f, unsigned long long seed, cudaStream_t s, std::string &err);
// Adam training on nsamples table samples; loss per epoch into hist
int mlp_train(MlpState &m, const MlpTables &t, long long nsamples, int epochs, int batch, double lr,
              unsigned long long seed, double *hist, cudaStream_t s, std::string &err);
// loss and gradient of one batch given on the host (n rows)
int mlp_grad(MlpState &m, int n, const float *feat3, const int *trip, const float *target, float *grad,
             double *loss, cudaStream_t s, std::string &err);
// forward pass of n rows given on the host (normalized outputs, n x MLP_OUT)
int mlp_forward(MlpState &m, int n, const float *feat3, const int *trip, float *out, cudaStream_t s,
                std::string &err);
// per-bin maximum error of the network (table units, Legendre-combined
// values) over per_bin samples of each interpolation bin (triple x cells)
int mlp_validate(MlpState &m, const MlpTables &t, int per_bin, int cells, unsigned long long seed,
                 std::vector<float> &bin_err, cudaStream_t s, std::string &err);
// table samples as the trainer draws them (for tests): features, triple, normalized targets
int mlp_samples(MlpState &m, const MlpTables &t, int n, unsigned long long seed, float *feat3, int *trip,
                float *target, cudaStream_t s, std::string &err);

}  // namespace fb
