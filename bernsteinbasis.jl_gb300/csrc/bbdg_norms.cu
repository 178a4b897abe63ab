// FP64 reductions for energy and error norms (warp-shuffle trees, deterministic two-pass).
//
// bb_norms:      per field sum a^2, sum (a-b)^2, sum b^2 over the coefficient arrays.
// bb_mass_norms: per field sum_e J_e a_e^T M a_e with M the Bernstein mass matrix of the
//                reference tetrahedron, in closed form:
//                M_ab = |T| / C(2N+3,3) * C_N(a) C_N(b) / C_2N(a+b),  |T| = 4/3,
//                C_n(a) the multinomial n! / (a0! a1! a2! a3!).
#include <cmath>
#include <vector>

#include "bbdg_internal.cuh"

namespace {

constexpr int kRedThreads = 256;
constexpr int kMaxFields = 8;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of `n` values per thread; result valid in thread 0.
template <int NV>
__device__ void block_sum(double (&v)[NV], double* sred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int m = 0; m < NV; ++m) v[m] = warp_sum(v[m]);
  if (lane == 0)
    for (int m = 0; m < NV; ++m) sred[warp * NV + m] = v[m];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int m = 0; m < NV; ++m) {
      double x = lane < nw ? sred[lane * NV + m] : 0.0;
      v[m] = warp_sum(x);
    }
  }
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(kRedThreads) norms_partial(int64_t n, int nf, const T* __restrict__ a,
                                                             const T* __restrict__ b,
                                                             double* __restrict__ part) {
  __shared__ double sred[32 * 3];
  for (int f = 0; f < nf; ++f) {
    const T* af = a + (size_t)f * n;
    const T* bf = b ? b + (size_t)f * n : nullptr;
    double v[3] = {0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
      const double x = (double)af[i];
      v[0] += x * x;
      if (bf) {
        const double y = (double)bf[i];
        v[1] += (x - y) * (x - y);
        v[2] += y * y;
      }
    }
    block_sum<3>(v, sred);
    if (threadIdx.x == 0)
      for (int m = 0; m < 3; ++m) part[((size_t)blockIdx.x * nf + f) * 3 + m] = v[m];
  }
}

// Sums `nblocks` rows of `width` partials in a fixed order: out[c] = sum_r part[r*width + c].
__global__ void __launch_bounds__(kRedThreads) sum_rows(int nrows, int width, const double* __restrict__ part,
                                                        double* __restrict__ out) {
  __shared__ double sred[32];
  for (int c = 0; c < width; ++c) {
    double v[1] = {0.0};
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) v[0] += part[(size_t)r * width + c];
    block_sum<1>(v, sred);
    if (threadIdx.x == 0) out[c] = v[0];
  }
}

// Mass-matrix quadratic form, EB elements per block iteration.
constexpr int kEB = 8;
template <class T>
__global__ void __launch_bounds__(kRedThreads) mass_partial(int N, int64_t K, int nf, const T* __restrict__ a,
                                                            const T* __restrict__ b,
                                                            const T* __restrict__ geo,
                                                            const uint32_t* __restrict__ node3,
                                                            const double* __restrict__ wN,
                                                            const double* __restrict__ invC2N,
                                                            double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int Np = np3(N), N2 = 2 * N;
  const int n2 = np3(N2);
  double* sInv = reinterpret_cast<double*>(smem);
  double* sC = sInv + n2;                   // [kEB][Np]
  uint32_t* sNode = reinterpret_cast<uint32_t*>(sC + kEB * Np);
  __shared__ double sred[32 * kMaxFields];
  for (int t = threadIdx.x; t < n2; t += blockDim.x) sInv[t] = invC2N[t];
  for (int t = threadIdx.x; t < Np; t += blockDim.x) sNode[t] = node3[t];
  double acc[kMaxFields];
  for (int f = 0; f < kMaxFields; ++f) acc[f] = 0.0;
  const int64_t nblk = (K + kEB - 1) / kEB;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * kEB;
    const int ne = (int)min64(kEB, K - e0);
    for (int f = 0; f < nf; ++f) {
      __syncthreads();
      for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
        const int le = t / Np, n = t - le * Np;
        const size_t gi = ((size_t)f * K + e0) * Np + t;
        double x = (double)a[gi];
        if (b) x -= (double)b[gi];
        sC[le * Np + n] = x * wN[n];
      }
      __syncthreads();
      for (int al = threadIdx.x; al < Np; al += blockDim.x) {
        const uint32_t c1 = sNode[al];
        const int i1 = c1 & 0xff, j1 = (c1 >> 8) & 0xff, k1 = c1 >> 16;
        double s[kEB];
#pragma unroll
        for (int le = 0; le < kEB; ++le) s[le] = 0.0;
        for (int be = 0; be < Np; ++be) {
          const uint32_t c2 = sNode[be];
          const double w = sInv[ijk3(N2, i1 + (c2 & 0xff), j1 + ((c2 >> 8) & 0xff), k1 + (c2 >> 16))];
#pragma unroll
          for (int le = 0; le < kEB; ++le) s[le] += w * sC[le * Np + be];
        }
        for (int le = 0; le < ne; ++le)
          acc[f] += s[le] * sC[le * Np + al] * (double)geo[(e0 + le) * BB_GEO_STRIDE + 10];
      }
    }
  }
  __syncthreads();
  block_sum<kMaxFields>(acc, sred);
  if (threadIdx.x == 0)
    for (int f = 0; f < nf; ++f) part[(size_t)blockIdx.x * nf + f] = acc[f];
}

double multinom(int n, const int* a, int m) {
  double r = std::tgamma(n + 1.0);
  for (int q = 0; q < m; ++q) r /= std::tgamma(a[q] + 1.0);
  return std::round(r);
}

int ensure_red(bb_ctx* ctx, size_t entries) {
  if (ctx->red_cap >= entries) return BB_OK;
  cudaFree(ctx->d_red);
  cudaFreeHost(ctx->h_red);
  ctx->d_red = nullptr;
  ctx->h_red = nullptr;
  ctx->red_cap = 0;
  if (cudaMalloc(&ctx->d_red, entries * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_red, 64 * sizeof(double)) != cudaSuccess)
    return bb_fail(ctx, BB_ERR_NOMEM, "reduction scratch allocation failed");
  ctx->red_cap = entries;
  return BB_OK;
}

}  // namespace

extern "C" int bb_norms(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, const void* a,
                        const void* b, double* out_host, void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N) || K < 0 || nf < 1 || nf > kMaxFields || !valid_dtype(dtype) || !a ||
      !out_host)
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_norms");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = K * np3(N);
  int grid = ctx->num_sms * 2;
  rc = ensure_red(ctx, (size_t)grid * nf * 3 + 3 * nf);
  if (rc) return rc;
  double* part = ctx->d_red;
  double* fin = ctx->d_red + (size_t)grid * nf * 3;
  if (dtype == BB_F64)
    norms_partial<double><<<grid, kRedThreads, 0, st>>>(n, nf, (const double*)a, (const double*)b, part);
  else
    norms_partial<float><<<grid, kRedThreads, 0, st>>>(n, nf, (const float*)a, (const float*)b, part);
  rc = bb_check_launch(ctx, "norms_partial");
  if (rc) return rc;
  sum_rows<<<1, kRedThreads, 0, st>>>(grid, nf * 3, part, fin);
  rc = bb_check_launch(ctx, "sum_rows");
  if (rc) return rc;
  BB_CUDA(ctx, cudaMemcpyAsync(ctx->h_red, fin, sizeof(double) * 3 * nf, cudaMemcpyDeviceToHost, st));
  BB_CUDA(ctx, cudaStreamSynchronize(st));
  bool finite = true;
  for (int m = 0; m < 3 * nf; ++m) {
    out_host[m] = ctx->h_red[m];
    finite = finite && std::isfinite(out_host[m]);
  }
  return finite ? BB_OK : bb_fail(ctx, BB_ERR_NONFINITE, "non-finite norm");
}

extern "C" int bb_mass_norms(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, const void* a,
                             const void* b, const void* geo, double* out_host, void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N) || K < 0 || nf < 1 || nf > kMaxFields || !valid_dtype(dtype) || !a ||
      !geo || !out_host)
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_mass_norms");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  const int Np = np3(N), n2 = np3(2 * N);
  // host-side closed-form weights: wN[a] = C_N(a), invC2N[g] = |T| / (C(2N+3,3) C_2N(g))
  std::vector<double> wN(Np), inv(n2);
  {
    int m = 0;
    for (int k = 0; k <= N; ++k)
      for (int j = 0; j <= N - k; ++j)
        for (int i = 0; i <= N - j - k; ++i) {
          int al[4] = {i, j, k, N - i - j - k};
          wN[m++] = multinom(N, al, 4);
        }
    const double c = (4.0 / 3.0) / ((2.0 * N + 3) * (2.0 * N + 2) * (2.0 * N + 1) / 6.0);
    m = 0;
    for (int k = 0; k <= 2 * N; ++k)
      for (int j = 0; j <= 2 * N - k; ++j)
        for (int i = 0; i <= 2 * N - j - k; ++i) {
          int g[4] = {i, j, k, 2 * N - i - j - k};
          inv[m++] = c / multinom(2 * N, g, 4);
        }
  }
  const size_t smem = sizeof(double) * ((size_t)n2 + (size_t)kEB * Np) + 4 * (size_t)Np;
  if (smem > ctx->smem_optin) return bb_fail(ctx, BB_ERR_ARG, "degree too large for mass norms");
  int grid = ctx->num_sms * 2;
  const size_t extra = (size_t)Np + n2;
  rc = ensure_red(ctx, (size_t)grid * nf + nf + extra);
  if (rc) return rc;
  double* part = ctx->d_red;
  double* fin = part + (size_t)grid * nf;
  double* dW = fin + nf;
  double* dInv = dW + Np;
  BB_CUDA(ctx, cudaMemcpyAsync(dW, wN.data(), sizeof(double) * Np, cudaMemcpyHostToDevice, st));
  BB_CUDA(ctx, cudaMemcpyAsync(dInv, inv.data(), sizeof(double) * n2, cudaMemcpyHostToDevice, st));
  const uint32_t* node3 = t->d_words + t->o_node3;
  if (dtype == BB_F64) {
    BB_CUDA(ctx, cudaFuncSetAttribute(mass_partial<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mass_partial<double><<<grid, kRedThreads, smem, st>>>(N, K, nf, (const double*)a, (const double*)b,
                                                          (const double*)geo, node3, dW, dInv, part);
  } else {
    BB_CUDA(ctx, cudaFuncSetAttribute(mass_partial<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mass_partial<float><<<grid, kRedThreads, smem, st>>>(N, K, nf, (const float*)a, (const float*)b,
                                                         (const float*)geo, node3, dW, dInv, part);
  }
  rc = bb_check_launch(ctx, "mass_partial");
  if (rc) return rc;
  sum_rows<<<1, kRedThreads, 0, st>>>(grid, nf, part, fin);
  rc = bb_check_launch(ctx, "sum_rows");
  if (rc) return rc;
  BB_CUDA(ctx, cudaMemcpyAsync(ctx->h_red, fin, sizeof(double) * nf, cudaMemcpyDeviceToHost, st));
  BB_CUDA(ctx, cudaStreamSynchronize(st));
  bool finite = true;
  for (int m = 0; m < nf; ++m) {
    out_host[m] = ctx->h_red[m];
    finite = finite && std::isfinite(out_host[m]);
  }
  return finite ? BB_OK : bb_fail(ctx, BB_ERR_NONFINITE, "non-finite norm");
}

// -------------------------------------------------------------------------------------
// bb_norms_noalloc: the same per-field sums without any allocation, for callers that must
// not allocate device memory (code running while a CUDA graph is being captured on its
// stream, runtimes whose device memory is owned by their own pool allocator, latency-bound
// loops). Its partial sums live in a file-scope device array of fixed size that every GPU
// loading this library holds until exit.
// -------------------------------------------------------------------------------------
namespace {

constexpr int kNoAllocBlocks = 512;  // fixed grid of the partial-sum kernel
static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks * kMaxFields * 3];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
void* g_noalloc_ctx[kNoAllocMaxDevices] = {};  // driver context the address belongs to

using CtxGetCurrentFn = int (*)(void**);  // cuCtxGetCurrent(CUcontext*)

// The calling thread's current driver context, or nullptr if it cannot be read. A device's
// primary context is replaced by cudaDeviceReset; the module, and with it the array, is then
// loaded again, possibly at another address.
void* current_driver_context() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  void* c = nullptr;
  if (!fn || fn(&c) != 0) return nullptr;
  return c;
}

// Device address of g_noalloc_partials on the current device, looked up once per device (and
// again if the device's context was replaced). In host code the array's name is only a
// host-side stand-in, not a device address.
int noalloc_scratch(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return BB_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  void* c = current_driver_context();
  if (!g_noalloc_ptr[dev] || c != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) return BB_ERR_CUDA;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
    g_noalloc_ctx[dev] = c;
  }
  *out = g_noalloc_ptr[dev];
  return BB_OK;
}

// Launches through cudaLaunchKernel, whose return value belongs to this launch alone: an error
// left pending by some earlier, unrelated runtime call is neither reported nor cleared here.
// A launch error of our own is cleared so that it does not surface in a later caller's check.
int noalloc_launch(const void* fn, int grid, void** args, cudaStream_t st) {
  cudaError_t e = cudaLaunchKernel(fn, dim3(grid), dim3(kRedThreads), args, 0, st);
  if (e == cudaSuccess) return BB_OK;
  (void)cudaGetLastError();
  return BB_ERR_CUDA;
}

}  // namespace

extern "C" int bb_norms_noalloc(int N, int64_t K, int nf, int dtype, const void* a,
                                const void* b, double* out_dev, void* stream) {
  if (!valid_degree(N) || K < 0 || !valid_dtype(dtype) || !a || !out_dev) return BB_ERR_ARG;
  if (nf < 1 || nf > kMaxFields) return BB_ERR_ARG;  // the scratch holds kMaxFields fields
  double* part = nullptr;
  int rc = noalloc_scratch(&part);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t n = K * np3(N);
  // every block writes all of its partials before sum_rows reads them: nothing to clear
  void* pargs[] = {&n, &nf, const_cast<void**>(&a), const_cast<void**>(&b), &part};
  const void* partial = dtype == BB_F64 ? (const void*)norms_partial<double>
                                        : (const void*)norms_partial<float>;
  rc = noalloc_launch(partial, kNoAllocBlocks, pargs, st);
  if (rc) return rc;
  int nrows = kNoAllocBlocks, width = nf * 3;
  void* sargs[] = {&nrows, &width, &part, &out_dev};
  return noalloc_launch((const void*)sum_rows, 1, sargs, st);
}
