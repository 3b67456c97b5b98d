// Eigenvalue gradients with respect to the stored entries of a sparse
// symmetric matrix (the adjoint / "backward" entry point).
//
// For a simple eigenpair of A x = lambda B x with x^T B x = 1 and B fixed,
// the Hellmann-Feynman theorem gives d lambda / d a_ij = x_i x_j.  A stored
// off-diagonal entry of the one-triangle CSR stands for both a_ij and a_ji,
// so its derivative is 2 x_i x_j.  For f = sum_k w_k lambda_k the gradient is
// the weighted sum over the eigenpairs; for a cluster of equal eigenvalues it
// is basis-independent when the whole cluster is included with one weight.
//
// Device work: per-column normalisation s_k = x_k^T B x_k (B diagonal or I)
// by a deterministic two-pass reduction, then one pass over the nonzeros
// (thread per row, rows read their entries and the eigenvector rows once).
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "../../include/jadamilu_gb300.h"

namespace jdg {
namespace {

constexpr int GR_TPB = 256;
constexpr int GR_MAXK = 64;

// partial[b * k + c] = sum over this block's rows of bdiag_i * x_c(i)^2
__global__ void colnorm_partial_kernel(int n, int k, const double* __restrict__ X, long ldx,
                                       const double* __restrict__ bdiag, double* __restrict__ partial) {
  __shared__ double red[GR_TPB];
  for (int c = 0; c < k; ++c) {
    double s = 0;
    for (int i = blockIdx.x * GR_TPB + threadIdx.x; i < n; i += gridDim.x * GR_TPB) {
      const double v = X[(long)c * ldx + i];
      s += (bdiag ? bdiag[i] : 1.0) * v * v;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = GR_TPB / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(long)blockIdx.x * k + c] = red[0];
    __syncthreads();
  }
}

// coef[c] = w_c / sum_b partial[b * k + c]  (fixed order)
__global__ void colnorm_final_kernel(int nb, int k, const double* __restrict__ partial, const double* __restrict__ w,
                                     double* __restrict__ coef) {
  const int c = threadIdx.x;
  if (c >= k) return;
  double s = 0;
  for (int b = 0; b < nb; ++b) s += partial[(long)b * k + c];
  coef[c] = w[c] / s;
}

// grad[q] = c_q * sum_c coef_c x_c(i) x_c(j), i the row of stored entry q
__global__ void eig_grad_kernel(int n, int k, const int* __restrict__ ia, const int* __restrict__ ja,
                                const double* __restrict__ X, long ldx, const double* __restrict__ coef,
                                double* __restrict__ grad) {
  const int i = blockIdx.x * GR_TPB + threadIdx.x;
  if (i >= n) return;
  double xi[GR_MAXK];
  for (int c = 0; c < k; ++c) xi[c] = coef[c] * X[(long)c * ldx + i];
  const int b = ia[i] - 1, e = ia[i + 1] - 1;
  for (int q = b; q < e; ++q) {
    const int j = ja[q] - 1;
    double g = 0;
    for (int c = 0; c < k; ++c) g += xi[c] * X[(long)c * ldx + j];
    grad[q] = (j == i) ? g : 2.0 * g;
  }
}

}  // namespace
}  // namespace jdg

using namespace jdg;

// Gradient of sum_k w[k] lambda_k with respect to every stored entry of the
// one-triangle CSR (ia, ja) used for A; see include/jadamilu_gb300.h.
JDG_API int jdgpu_deig_grad(int n, const int* ia, const int* ja, int neig, const double* X, int ldx,
                            const double* w, const double* bdiag, double* grad) {
  if (n <= 0 || neig <= 0 || neig > GR_MAXK || ldx < n) return -1;
  const int nnz = ia[n] - 1;
  int *dia = nullptr, *dja = nullptr;
  double *dX = nullptr, *dw = nullptr, *db = nullptr, *dpart = nullptr, *dcoef = nullptr, *dg = nullptr;
  int rc = 0;
  try {
    const int nb = std::min(std::max(1, (n + GR_TPB - 1) / GR_TPB), 152 * 4);
    CK(cudaMalloc(&dia, sizeof(int) * (n + 1)));
    CK(cudaMalloc(&dja, sizeof(int) * std::max(1, nnz)));
    CK(cudaMalloc(&dX, sizeof(double) * (size_t)ldx * neig));
    CK(cudaMalloc(&dw, sizeof(double) * neig));
    CK(cudaMalloc(&dpart, sizeof(double) * (size_t)nb * neig));
    CK(cudaMalloc(&dcoef, sizeof(double) * neig));
    CK(cudaMalloc(&dg, sizeof(double) * std::max(1, nnz)));
    if (bdiag) CK(cudaMalloc(&db, sizeof(double) * n));
    CK(cudaMemcpy(dia, ia, sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dja, ja, sizeof(int) * nnz, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dX, X, sizeof(double) * (size_t)ldx * neig, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dw, w, sizeof(double) * neig, cudaMemcpyHostToDevice));
    if (bdiag) CK(cudaMemcpy(db, bdiag, sizeof(double) * n, cudaMemcpyHostToDevice));
    colnorm_partial_kernel<<<nb, GR_TPB>>>(n, neig, dX, ldx, db, dpart);
    colnorm_final_kernel<<<1, GR_MAXK>>>(nb, neig, dpart, dw, dcoef);
    eig_grad_kernel<<<(n + GR_TPB - 1) / GR_TPB, GR_TPB>>>(n, neig, dia, dja, dX, ldx, dcoef, dg);
    CK(cudaGetLastError());
    k::add_launches(3);
    CK(cudaMemcpy(grad, dg, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_deig_grad: %s\n", e.what());
    rc = -99;
  }
  cudaFree(dia);
  cudaFree(dja);
  cudaFree(dX);
  cudaFree(dw);
  cudaFree(db);
  cudaFree(dpart);
  cudaFree(dcoef);
  cudaFree(dg);
  return rc;
}
