// fb_solve.cu -- the k-point Lowdin solver that follows the Bloch sums:
// kspace_Lowdin (h.SOLVESH/M_kspace_Lowdin.f90:740-880) with diagonalize_S
// and diagonalize_H_Lowdin (h.SOLVESH/M_diagonalization_Lowdin_kpoints.f90:
// 145-403).  Per k-point, with S(k) and H(k) dense on the device:
//   1. eigenpairs of S (zheev on the upper triangle, :190-193);
//   2. the eigenvalues below overtol = 1e-4 are a linear dependence: with m
//      of them (ascending order), columns m+1..n move to 1..n-m and the
//      trailing m columns keep what they held (:222-233);
//   3. every column j of that matrix is scaled by lambda_j^(-1/4) and
//      S12 = W W^H (:336-343; norbitals_new = size(eigen) = n there, so the
//      trailing columns enter too);
//   4. Z = S12 (H S12) (:352-357), eigenpairs of Z: the band energies and
//      c_Lowdin (:372-379); c = S12 c_Lowdin (:386-388).
// The eigen-decompositions are cuSOLVER's zheevd and the products cuBLAS's
// zgemm (plain library calls, FP64 complex); the column shift and scaling
// is this file's kernel.  Both libraries are opened at the first solve, so
// the rest of libfbgpu loads and runs where they are absent.
#include <dlfcn.h>

#include <cublas_v2.h>
#include <cusolverDn.h>

#include <mutex>
#include <string>
#include <vector>

#include "fb_solve.h"

namespace fb {

namespace {

struct SolverLib {
  bool ok = false;
  std::string why;
  cusolverStatus_t (*dn_create)(cusolverDnHandle_t *) = nullptr;
  cusolverStatus_t (*dn_destroy)(cusolverDnHandle_t) = nullptr;
  cusolverStatus_t (*dn_set_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
  cusolverStatus_t (*zheevd_size)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int,
                                  const cuDoubleComplex *, int, const double *, int *) = nullptr;
  cusolverStatus_t (*zheevd)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, cuDoubleComplex *, int,
                             double *, cuDoubleComplex *, int, int *) = nullptr;
  cublasStatus_t (*blas_create)(cublasHandle_t *) = nullptr;
  cublasStatus_t (*blas_destroy)(cublasHandle_t) = nullptr;
  cublasStatus_t (*blas_set_stream)(cublasHandle_t, cudaStream_t) = nullptr;
  cublasStatus_t (*zgemm)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int,
                          const cuDoubleComplex *, const cuDoubleComplex *, int, const cuDoubleComplex *, int,
                          const cuDoubleComplex *, cuDoubleComplex *, int) = nullptr;
};

template <class F>
bool sym(void *h, const char *name, F &f) {
  f = reinterpret_cast<F>(dlsym(h, name));
  return f != nullptr;
}

SolverLib open_solver_lib() {
  SolverLib L;
  void *blas = dlopen("libcublas.so.13", RTLD_NOW | RTLD_GLOBAL);
  if (!blas) blas = dlopen("libcublas.so", RTLD_NOW | RTLD_GLOBAL);
  void *dn = dlopen("libcusolver.so.12", RTLD_NOW | RTLD_GLOBAL);
  if (!dn) dn = dlopen("libcusolver.so", RTLD_NOW | RTLD_GLOBAL);
  if (!blas || !dn) {
    L.why = std::string("cannot open ") + (!blas ? "libcublas" : "libcusolver");
    return L;
  }
  bool ok = sym(dn, "cusolverDnCreate", L.dn_create) && sym(dn, "cusolverDnDestroy", L.dn_destroy) &&
            sym(dn, "cusolverDnSetStream", L.dn_set_stream) &&
            sym(dn, "cusolverDnZheevd_bufferSize", L.zheevd_size) && sym(dn, "cusolverDnZheevd", L.zheevd) &&
            sym(blas, "cublasCreate_v2", L.blas_create) && sym(blas, "cublasDestroy_v2", L.blas_destroy) &&
            sym(blas, "cublasSetStream_v2", L.blas_set_stream) && sym(blas, "cublasZgemm_v2", L.zgemm);
  if (!ok) {
    L.why = "a cuSOLVER / cuBLAS entry point is missing";
    return L;
  }
  L.ok = true;
  return L;
}

SolverLib &solver_lib() {
  static std::once_flag once;
  static SolverLib L;
  std::call_once(once, [] { L = open_solver_lib(); });
  return L;
}

// W[:, j] = U[:, src] * lam[src]^(-1/4), src = j + m for j < n - m, else j
// (the column shift of diagonalize_S and the scaling of diagonalize_H_Lowdin)
__global__ void k_lowdin_scale(long long n, int m, const double2 *__restrict__ U, const double *__restrict__ lam,
                               double2 *__restrict__ W) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  long long j = idx / n, r = idx - j * n;
  long long src = j < n - m ? j + m : j;
  double sc = pow(lam[src], -0.25);
  double2 u = U[src * n + r];
  W[idx] = make_double2(u.x * sc, u.y * sc);
}

}  // namespace

bool solver_available(std::string &why) {
  SolverLib &L = solver_lib();
  why = L.why;
  return L.ok;
}

void solver_destroy(SolverHandles &h) {
  SolverLib &L = solver_lib();
  if (!L.ok) return;
  if (h.dn) L.dn_destroy(static_cast<cusolverDnHandle_t>(h.dn));
  if (h.blas) L.blas_destroy(static_cast<cublasHandle_t>(h.blas));
  h.dn = h.blas = nullptr;
}

int lowdin_solve(SolverHandles &h, cudaStream_t s, int n, const LowdinBufs &b, double *eps_host, double *c_dev,
                 int *dropped, std::string &err) {
  SolverLib &L = solver_lib();
  if (!L.ok) {
    err = "the eigensolver needs cuSOLVER and cuBLAS: " + L.why;
    return -1;
  }
  if (!h.dn) {
    cusolverDnHandle_t d;
    if (L.dn_create(&d) != CUSOLVER_STATUS_SUCCESS) {
      err = "cusolverDnCreate failed";
      return -2;
    }
    h.dn = d;
  }
  if (!h.blas) {
    cublasHandle_t c;
    if (L.blas_create(&c) != CUBLAS_STATUS_SUCCESS) {
      err = "cublasCreate failed";
      return -2;
    }
    h.blas = c;
  }
  auto dn = static_cast<cusolverDnHandle_t>(h.dn);
  auto bl = static_cast<cublasHandle_t>(h.blas);
  L.dn_set_stream(dn, s);
  L.blas_set_stream(bl, s);
  auto Z = [](double *p) { return reinterpret_cast<cuDoubleComplex *>(p); };
  const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
  // 1. eigenpairs of S (vectors overwrite Sk)
  if (L.zheevd(dn, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, Z(b.Sk), n, b.lam, Z(b.work), b.lwork,
               b.info) != CUSOLVER_STATUS_SUCCESS) {
    err = "zheevd (S) failed to launch";
    return -2;
  }
  std::vector<double> lam(n);
  int info = 0;
  if (cudaMemcpyAsync(lam.data(), b.lam, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&info, b.info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    err = "copy of the overlap eigenvalues failed";
    return -2;
  }
  if (info != 0) {
    err = "zheevd of S(k) did not converge (info " + std::to_string(info) + ")";
    return -3;
  }
  // 2. mineig: the last ascending eigenvalue below overtol (1-based), + 1
  int m = 0;
  for (int k = 0; k < n; k++)
    if (lam[k] < LOWDIN_OVERTOL) m = k + 1;
  if (dropped) *dropped = m;
  // with more than half of the eigenvalues dropped, the trailing columns
  // that keep their place include eigenvalues below overtol: the reference
  // raises them to the power -1/4 (a NaN for the negative ones) and goes on
  // with a meaningless S^-1/2; report it instead
  if (2 * m > n) {
    err = std::to_string(m) + " of " + std::to_string(n) +
          " overlap eigenvalues are below 1e-4: the Lowdin S^-1/2 is undefined (S(k) is far from positive definite)";
    return -3;
  }
  // 3. W = shifted, scaled eigenvectors; S12 = W W^H (into Tmp)
  long long nn = (long long)n * n;
  int threads = 256;
  k_lowdin_scale<<<(unsigned)((nn + threads - 1) / threads), threads, 0, s>>>(
      n, m, reinterpret_cast<const double2 *>(b.Sk), b.lam, reinterpret_cast<double2 *>(b.W));
  if (cudaGetLastError() != cudaSuccess) {
    err = "Lowdin scaling kernel failed to launch";
    return -2;
  }
  bool okg = L.zgemm(bl, CUBLAS_OP_N, CUBLAS_OP_C, n, n, n, &one, Z(b.W), n, Z(b.W), n, &zero, Z(b.T), n) ==
             CUBLAS_STATUS_SUCCESS;
  // 4. W = H S12, Hk = S12 W = Z; eigenpairs of Z (vectors overwrite Hk)
  okg = okg && L.zgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, Z(b.Hk), n, Z(b.T), n, &zero, Z(b.W), n) ==
                   CUBLAS_STATUS_SUCCESS;
  okg = okg && L.zgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, Z(b.T), n, Z(b.W), n, &zero, Z(b.Hk), n) ==
                   CUBLAS_STATUS_SUCCESS;
  if (!okg) {
    err = "zgemm failed";
    return -2;
  }
  if (L.zheevd(dn, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, Z(b.Hk), n, b.eps, Z(b.work), b.lwork,
               b.info) != CUSOLVER_STATUS_SUCCESS) {
    err = "zheevd (H) failed to launch";
    return -2;
  }
  // c = S12 c_Lowdin
  if (c_dev && L.zgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, Z(b.T), n, Z(b.Hk), n, &zero, Z(c_dev), n) !=
                   CUBLAS_STATUS_SUCCESS) {
    err = "zgemm (c) failed";
    return -2;
  }
  if (cudaMemcpyAsync(eps_host, b.eps, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&info, b.info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    err = "copy of the band energies failed";
    return -2;
  }
  if (info != 0) {
    err = "zheevd of the Lowdin-transformed H(k) did not converge (info " + std::to_string(info) + ")";
    return -3;
  }
  return 0;
}

int lowdin_work_size(SolverHandles &h, cudaStream_t s, int n, double *A, double *lam, int *lwork, std::string &err) {
  SolverLib &L = solver_lib();
  if (!L.ok) {
    err = "the eigensolver needs cuSOLVER and cuBLAS: " + L.why;
    return -1;
  }
  if (!h.dn) {
    cusolverDnHandle_t d;
    if (L.dn_create(&d) != CUSOLVER_STATUS_SUCCESS) {
      err = "cusolverDnCreate failed";
      return -2;
    }
    h.dn = d;
  }
  auto dn = static_cast<cusolverDnHandle_t>(h.dn);
  L.dn_set_stream(dn, s);
  if (L.zheevd_size(dn, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                    reinterpret_cast<const cuDoubleComplex *>(A), n, lam, lwork) != CUSOLVER_STATUS_SUCCESS) {
    err = "zheevd workspace query failed";
    return -2;
  }
  return 0;
}

}  // namespace fb
