// fb_solve.h -- the k-point Lowdin solver (fb_solve.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace fb {

// overlap eigenvalues below this count as a linear dependence
// (h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:71)
constexpr double LOWDIN_OVERTOL = 1.0e-4;

struct SolverHandles {
  void *dn = nullptr;    // cusolverDnHandle_t
  void *blas = nullptr;  // cublasHandle_t
};

// device buffers of one solve: four n x n complex matrices (interleaved re,
// im), two n-vectors, the zheevd workspace (lwork complex) and its info flag
struct LowdinBufs {
  double *Sk, *Hk, *W, *T;
  double *lam, *eps;
  double *work;
  int lwork;
  int *info;
};

bool solver_available(std::string &why);
// zheevd workspace (complex elements) for n x n
int lowdin_work_size(SolverHandles &h, cudaStream_t s, int n, double *A, double *lam, int *lwork, std::string &err);
// Sk and Hk hold S(k) and H(k) on entry (both are overwritten); band
// energies to eps_host (n, ascending), eigenvectors c to c_dev (n x n
// complex, may be null), the number of dropped overlap eigenvalues to
// dropped (may be null).  Returns 0, -1 (libraries absent), -2 (a call
// failed) or -3 (no convergence, or more than half of the overlap
// eigenvalues below overtol), with err set.
int lowdin_solve(SolverHandles &h, cudaStream_t s, int n, const LowdinBufs &b, double *eps_host, double *c_dev,
                 int *dropped, std::string &err);
void solver_destroy(SolverHandles &h);

}  // namespace fb
