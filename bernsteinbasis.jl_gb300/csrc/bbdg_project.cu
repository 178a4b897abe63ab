// FP64 L2 degree reduction between Bernstein degrees (N -> M < N), per element and field:
//     c_M = M_MM^{-1} E_{M->N}^T M_NN c_N
// with M_nn the Bernstein mass matrix of the reference tetrahedron (closed form
// M_ab = |T| C_n(a) C_n(b) / (C_2n(a+b) C(2n+3,3))) and E_{M->N} the 3D degree elevation
// (B^M_a = sum_g E[g,a] B^N_g, E[g,a] = C_M(a) C_{N-M}(g-a) / C_N(g)). The dense
// Np(M) x Np(N) operator is formed once per (N, M) on the host in FP64 and applied by an
// FP64 kernel. No counterpart in the reference (used to reduce degree-10 solutions to
// degree 5 for the learned closure).
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "bbdg_internal.cuh"

namespace {

struct ProjOp {
  int N = 0, M = 0, NpN = 0, NpM = 0;
  double* d_P = nullptr;  // [NpM][NpN]
};

std::mutex g_proj_mu;
std::map<std::pair<bb_ctx*, int>, ProjOp> g_proj;

double lgamma1(int n) { return std::lgamma(double(n) + 1.0); }
double multinom(const int* a, int m) {
  int n = 0;
  double l = 0.0;
  for (int q = 0; q < m; ++q) {
    n += a[q];
    l -= lgamma1(a[q]);
  }
  return std::round(std::exp(l + lgamma1(n)));
}

std::vector<std::array<int, 4>> multi_indices(int n) {
  std::vector<std::array<int, 4>> r;
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n - k; ++j)
      for (int i = 0; i <= n - j - k; ++i) r.push_back({i, j, k, n - i - j - k});
  return r;
}

std::vector<double> mass(int n) {
  const auto L = multi_indices(n);
  const size_t np = L.size();
  const double c = (4.0 / 3.0) / ((2.0 * n + 3) * (2.0 * n + 2) * (2.0 * n + 1) / 6.0);
  std::vector<double> Mm(np * np);
  for (size_t a = 0; a < np; ++a)
    for (size_t b = 0; b < np; ++b) {
      int ab[4];
      for (int q = 0; q < 4; ++q) ab[q] = L[a][q] + L[b][q];
      Mm[a * np + b] = c * multinom(L[a].data(), 4) * multinom(L[b].data(), 4) / multinom(ab, 4);
    }
  return Mm;
}

// Solves A X = B (A n x n, B n x m, row-major) by Gaussian elimination with partial pivoting.
bool solve(std::vector<double> A, std::vector<double>& B, int n, int m) {
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
    if (A[p * n + c] == 0.0) return false;
    if (p != c) {
      for (int q = 0; q < n; ++q) std::swap(A[c * n + q], A[p * n + q]);
      for (int q = 0; q < m; ++q) std::swap(B[c * m + q], B[p * m + q]);
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A[r * n + c] / A[c * n + c];
      if (f == 0.0) continue;
      for (int q = c; q < n; ++q) A[r * n + q] -= f * A[c * n + q];
      for (int q = 0; q < m; ++q) B[r * m + q] -= f * B[c * m + q];
    }
  }
  for (int r = 0; r < n; ++r)
    for (int q = 0; q < m; ++q) B[r * m + q] /= A[r * n + r];
  return true;
}

const ProjOp* proj_op(bb_ctx* ctx, int N, int M) {
  std::lock_guard<std::mutex> lock(g_proj_mu);
  auto key = std::make_pair(ctx, N * 64 + M);
  auto it = g_proj.find(key);
  if (it != g_proj.end()) return &it->second;
  const auto LN = multi_indices(N), LM = multi_indices(M);
  const int npN = (int)LN.size(), npM = (int)LM.size();
  // E^T M_NN: (E^T)[a][g] = E[g][a]
  std::vector<double> MN = mass(N), rhs((size_t)npM * npN, 0.0);
  std::vector<double> ET((size_t)npM * npN, 0.0);
  for (int a = 0; a < npM; ++a)
    for (int g = 0; g < npN; ++g) {
      int d[4];
      bool ok = true;
      for (int q = 0; q < 4; ++q) {
        d[q] = LN[g][q] - LM[a][q];
        ok = ok && d[q] >= 0;
      }
      if (!ok) continue;
      ET[(size_t)a * npN + g] =
          multinom(LM[a].data(), 4) * multinom(d, 4) / multinom(LN[g].data(), 4);
    }
  for (int a = 0; a < npM; ++a)
    for (int g = 0; g < npN; ++g) {
      double sacc = 0.0;
      for (int h = 0; h < npN; ++h) sacc += ET[(size_t)a * npN + h] * MN[(size_t)h * npN + g];
      rhs[(size_t)a * npN + g] = sacc;
    }
  if (!solve(mass(M), rhs, npM, npN)) return nullptr;
  ProjOp op;
  op.N = N;
  op.M = M;
  op.NpN = npN;
  op.NpM = npM;
  if (cudaMalloc(&op.d_P, sizeof(double) * rhs.size()) != cudaSuccess) return nullptr;
  if (cudaMemcpy(op.d_P, rhs.data(), sizeof(double) * rhs.size(), cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    cudaFree(op.d_P);
    return nullptr;
  }
  return &(g_proj[key] = op);
}

constexpr int kCols = 16;  // element-field columns per block

// out[col][a] = sum_b P[a][b] in[col][b] for 16 columns per block, FP64 accumulation.
template <class TI, class TO>
__global__ void __launch_bounds__(256) project_kernel(const double* __restrict__ P, int npM,
                                                      int npN, int64_t ncols,
                                                      const TI* __restrict__ in,
                                                      TO* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* X = reinterpret_cast<double*>(smem);  // [kCols][npN]
  const int64_t nblk = (ncols + kCols - 1) / kCols;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t c0 = blk * kCols;
    const int nc = (int)min64(kCols, ncols - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < nc * npN; t += blockDim.x) X[t] = (double)in[c0 * npN + t];
    __syncthreads();
    for (int t = threadIdx.x; t < npM * kCols; t += blockDim.x) {
      const int a = t / kCols, c = t - a * kCols;
      if (c >= nc) continue;
      const double* Pa = P + (size_t)a * npN;
      const double* x = X + (size_t)c * npN;
      double acc = 0.0;
      for (int b = 0; b < npN; ++b) acc = fma(__ldg(Pa + b), x[b], acc);
      out[(c0 + c) * npM + a] = (TO)acc;
    }
  }
}

}  // namespace

extern "C" int bb_project(bb_ctx* ctx, int N, int M, int64_t K, int nf, int dtype_in,
                          const void* in, int dtype_out, void* out, void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N) || M < 1 || M >= N || K < 0 || nf < 1 || !valid_dtype(dtype_in) ||
      !valid_dtype(dtype_out) || !in || !out)
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_project (need 1 <= M < N <= %d)",
                   BB_MAX_DEGREE);
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  const ProjOp* op = proj_op(ctx, N, M);
  if (!op) return bb_fail(ctx, BB_ERR_NOMEM, "projection operator set-up failed");
  if (K == 0) return BB_OK;
  const int64_t ncols = K * nf;
  const size_t smem = sizeof(double) * kCols * op->NpN;
  if (smem > ctx->smem_optin) return bb_fail(ctx, BB_ERR_ARG, "degree too large for bb_project");
  cudaStream_t st = (cudaStream_t)stream;
  int grid = (int)std::min<int64_t>((ncols + kCols - 1) / kCols, (int64_t)ctx->num_sms * 8);
#define BB_PROJ(TI, TO)                                                                    \
  do {                                                                                     \
    BB_CUDA(ctx, cudaFuncSetAttribute(project_kernel<TI, TO>,                              \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    project_kernel<TI, TO><<<grid, 256, smem, st>>>(op->d_P, op->NpM, op->NpN, ncols,       \
                                                    (const TI*)in, (TO*)out);              \
  } while (0)
  if (dtype_in == BB_F64 && dtype_out == BB_F64) BB_PROJ(double, double);
  else if (dtype_in == BB_F64) BB_PROJ(double, float);
  else if (dtype_out == BB_F64) BB_PROJ(float, double);
  else BB_PROJ(float, float);
#undef BB_PROJ
  return bb_check_launch(ctx, "project_kernel");
}
