// Learned per-element closure: a 3-layer MLP (nin -> h1 -> h2 -> nout, GELU after the two
// hidden layers) trained and evaluated on the GPU with the tcgen05 BF16 GEMM (FP32
// accumulation), plus the element feature gather and the correction apply. No counterpart in
// the reference.
//
// Parameters live in one flat FP32 buffer, layer by layer: W1 [h1][nin], b1 [h1],
// W2 [h2][h1], b2 [h2], W3 [nout][h2], b3 [nout] (row-major, out x in); gradients and the two
// Adam moments use the same layout. BF16 copies of W1..W3 (and of W2^T, W3^T for the
// backward pass) are refreshed after every parameter change.
//
// Forward (B rows):   pre1 = X W1^T + b1, H1 = GELU(pre1)      (X BF16, H1 BF16)
//                     pre2 = H1 W2^T + b2, H2 = GELU(pre2)
//                     Y = H2 W3^T + b3                          (FP32)
// Loss:               L = 1/(B nout) sum (Y - T)^2
// Backward:           dY = 2 (Y - T) / (B nout)                 (BF16 for the GEMMs)
//                     dW3 = dY^T H2, db3 = colsum(dY)
//                     dP2 = (dY W3) * GELU'(pre2), dW2 = dP2^T H1, db2 = colsum(dP2)
//                     dP1 = (dP2 W2) * GELU'(pre1), dW1 = dP1^T X, db1 = colsum(dP1)
// The weight gradients contract over the batch, so the forward pass also writes the
// transposed BF16 activations (X^T comes from the caller) and those GEMMs split K over CTAs.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bbdg_gemm.cuh"
#include "bbdg_internal.cuh"

struct bb_mlp {
  bb_ctx* ctx = nullptr;
  int dim[4] = {0, 0, 0, 0};  // nin, h1, h2, nout
  int64_t max_batch = 0;
  int64_t nparams = 0;
  int64_t oW[3] = {0, 0, 0}, ob[3] = {0, 0, 0};
  float* p = nullptr;  // FP32 master parameters
  float* g = nullptr;  // gradients
  float* m = nullptr;  // Adam first moment
  float* v = nullptr;  // Adam second moment
  __nv_bfloat16* Wb[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16* WT[3] = {nullptr, nullptr, nullptr};  // [1], [2] used
  float* pre[2] = {nullptr, nullptr};
  __nv_bfloat16* H[2] = {nullptr, nullptr};
  __nv_bfloat16* HT[2] = {nullptr, nullptr};
  __nv_bfloat16 *dY = nullptr, *dYT = nullptr, *dP2 = nullptr, *dP2T = nullptr, *dP1T = nullptr;
  const void* XT = nullptr;  // caller's X^T of the last training forward
  int64_t fwd_B = -1;        // batch of the last training forward (-1: none)
  int64_t steps = 0;
  std::vector<void*> allocs;
};

namespace {

template <class P>
bool dev_alloc(bb_mlp* n, P** ptr, size_t count) {
  void* q = nullptr;
  if (cudaMalloc(&q, count * sizeof(P)) != cudaSuccess) return false;
  n->allocs.push_back(q);
  *ptr = (P*)q;
  return true;
}

// splitmix64: seeded, platform-independent initial weights
uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void cast_weights_kernel(const float* __restrict__ W, int out, int in,
                                    __nv_bfloat16* __restrict__ Wb,
                                    __nv_bfloat16* __restrict__ WT) {
  const int64_t n = (int64_t)out * in;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int o = (int)(t / in), i = (int)(t - (int64_t)o * in);
    const __nv_bfloat16 b = __float2bfloat16_rn(W[t]);
    Wb[t] = b;
    if (WT) WT[(int64_t)i * out + o] = b;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt * c1) / (sqrtf(vt * c2) + eps);
  }
}

// dY = scale (Y - T) as BF16 in both layouts, db += column sums of the FP32 dY,
// loss += sum (Y - T)^2 * lscale. 32 x 32 tiles, 32 x 8 threads.
__global__ void mse_grad_kernel(const float* __restrict__ Y, const float* __restrict__ T,
                                int64_t B, int n, float scale, float lscale,
                                __nv_bfloat16* __restrict__ dY, __nv_bfloat16* __restrict__ dYT,
                                float* __restrict__ db, double* __restrict__ loss) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  const int c0 = blockIdx.x * 32;
  float l = 0.0f;
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i;
    const int c = c0 + tx;
    float gv = 0.0f;
    if (r < B && c < n) {
      const float d = Y[r * n + c] - T[r * n + c];
      l = fmaf(d, d, l);
      gv = scale * d;
      dY[r * n + c] = __float2bfloat16_rn(gv);
    }
    tile[i][tx] = gv;
  }
  __syncthreads();
  if (ty == 0 && c0 + tx < n) {
    float sacc = 0.0f;
    for (int i = 0; i < 32; ++i) sacc += tile[i][tx];
    atomicAdd(db + c0 + tx, sacc);
  }
  for (int i = ty; i < 32; i += 8) {
    const int c = c0 + i;
    const int64_t r = r0 + tx;
    if (c < n && r < B) dYT[(int64_t)c * B + r] = __float2bfloat16_rn(tile[tx][i]);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if (tx == 0) atomicAdd(loss, (double)l * (double)lscale);
}

// out[c][r] = in[r][c] for a [rows x cols] BF16 matrix, 32 x 32 tiles.
__global__ void transpose_bf16_kernel(const __nv_bfloat16* __restrict__ in, int64_t rows,
                                      int cols, __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 tile[32][34];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r0 = (int64_t)blockIdx.y * 32;
  const int c0 = blockIdx.x * 32;
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i;
    if (r < rows && c0 + tx < cols) tile[i][tx] = in[r * cols + c0 + tx];
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int c = c0 + i;
    const int64_t r = r0 + tx;
    if (c < cols && r < rows) out[(int64_t)c * rows + r] = tile[tx][i];
  }
}

// Closure features of element e (nf fields, degree N), scaled and rounded to BF16:
//   [fld][p]        own coefficients, p < Np
//   [f][fld][a]     the neighbour's coefficients on the shared face f, face node a < Nfp, in
//                   this element's face ordering (the exterior trace the flux sees)
template <class T>
__global__ void closure_features_kernel(const uint32_t* __restrict__ gtab, int o_fvol,
                                        int o_fperm, int N, int64_t K, int nf,
                                        const int32_t* __restrict__ conn,
                                        const T* __restrict__ q, float scale,
                                        __nv_bfloat16* __restrict__ X, int* status) {
  const int Np = np3(N), Nfp = np2(N);
  const int nown = nf * Np, nin = nown + 4 * nf * Nfp;
  const uint16_t* fvol = reinterpret_cast<const uint16_t*>(gtab + o_fvol);
  const uint16_t* fperm = reinterpret_cast<const uint16_t*>(gtab + o_fperm);
  for (int64_t e = blockIdx.x; e < K; e += gridDim.x) {
    for (int t = threadIdx.x; t < nin; t += blockDim.x) {
      float val;
      if (t < nown) {
        const int fld = t / Np, p = t - fld * Np;
        val = (float)q[((int64_t)fld * K + e) * Np + p];
      } else {
        const int u = t - nown;
        const int f = u / (nf * Nfp), rest = u - f * nf * Nfp;
        const int fld = rest / Nfp, a = rest - fld * Nfp;
        const int32_t c = __ldg(conn + e * 4 + f);
        const int64_t nbr = (int64_t)((uint32_t)c >> 5);
        const int nface = (c >> 3) & 3, o = c & 7;
        if (nbr >= K || o > 5) {
          atomicOr(status, 1);
          val = 0.0f;
        } else {
          const int vP = fvol[nface * Nfp + fperm[o * Nfp + a]];
          val = (float)q[((int64_t)fld * K + nbr) * Np + vP];
        }
      }
      X[e * nin + t] = __float2bfloat16_rn(val * scale);
    }
  }
}

// q[fld][e][p] += alpha * Y[e][fld * Np + p]
template <class T>
__global__ void closure_apply_kernel(int Np, int64_t K, int nf, float alpha,
                                     const float* __restrict__ Y, T* __restrict__ q) {
  const int64_t n = K * nf * Np;
  const int nw = nf * Np;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / nw;
    const int j = (int)(t - e * nw);
    const int fld = j / Np, p = j - fld * Np;
    const int64_t off = ((int64_t)fld * K + e) * Np + p;
    q[off] = (T)((float)q[off] + alpha * Y[t]);
  }
}

int grid_for(bb_ctx* ctx, int64_t n, int threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads,
                                                     (int64_t)ctx->num_sms * 16));
}

int refresh_bf16(bb_mlp* n, cudaStream_t st) {
  for (int l = 0; l < 3; ++l) {
    const int out = n->dim[l + 1], in = n->dim[l];
    cast_weights_kernel<<<grid_for(n->ctx, (int64_t)out * in, 256), 256, 0, st>>>(
        n->p + n->oW[l], out, in, n->Wb[l], n->WT[l]);
    int rc = bb_check_launch(n->ctx, "cast_weights_kernel");
    if (rc) return rc;
  }
  return BB_OK;
}

// Split-K GEMM for the batch contractions: about two waves of CTAs over the SMs.
int kt_split(bb_ctx* ctx, int64_t M, int N, int K) {
  const int64_t tiles = ((M + 127) / 128) * ((N + 127) / 128);
  const int nkt = (K + 63) / 64;
  int64_t splits = std::max<int64_t>(1, (2 * (int64_t)ctx->num_sms + tiles - 1) / tiles);
  splits = std::min<int64_t>(splits, std::max(1, nkt / 4));
  return (int)((nkt + splits - 1) / splits);
}

GemmEpilogue epi(bb_mlp* n) {
  GemmEpilogue e{};
  e.alpha = 1.0f;
  e.status = bb_ctx_status_word(n->ctx);
  return e;
}

}  // namespace

extern "C" int bb_mlp_create(bb_ctx* ctx, int nin, int h1, int h2, int nout, int64_t max_batch,
                             uint64_t seed, bb_mlp** out) {
  if (!ctx || !out) return BB_ERR_ARG;
  *out = nullptr;
  const int d[4] = {nin, h1, h2, nout};
  for (int i = 0; i < 4; ++i)
    if (d[i] < 8 || d[i] % 8 != 0 || d[i] > 65536)
      return bb_fail(ctx, BB_ERR_ARG, "MLP widths must be multiples of 8 in [8, 65536]");
  if (max_batch < 8 || max_batch % 8 != 0 || max_batch > ((int64_t)1 << 31) / 1024)
    return bb_fail(ctx, BB_ERR_ARG, "max_batch must be a positive multiple of 8");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  if (!bb_ctx_status_word(ctx)) return bb_fail(ctx, BB_ERR_NOMEM, "status word allocation failed");
  bb_mlp* n = new bb_mlp();
  n->ctx = ctx;
  for (int i = 0; i < 4; ++i) n->dim[i] = d[i];
  n->max_batch = max_batch;
  int64_t off = 0;
  for (int l = 0; l < 3; ++l) {
    n->oW[l] = off;
    off += (int64_t)d[l + 1] * d[l];
    n->ob[l] = off;
    off += d[l + 1];
  }
  n->nparams = off;
  const int64_t B = max_batch;
  bool ok = dev_alloc(n, &n->p, off) && dev_alloc(n, &n->g, off) && dev_alloc(n, &n->m, off) &&
            dev_alloc(n, &n->v, off);
  for (int l = 0; l < 3 && ok; ++l) {
    ok = dev_alloc(n, &n->Wb[l], (size_t)d[l + 1] * d[l]);
    if (ok && l > 0) ok = dev_alloc(n, &n->WT[l], (size_t)d[l + 1] * d[l]);
  }
  for (int l = 0; l < 2 && ok; ++l)
    ok = dev_alloc(n, &n->pre[l], (size_t)B * d[l + 1]) &&
         dev_alloc(n, &n->H[l], (size_t)B * d[l + 1]) &&
         dev_alloc(n, &n->HT[l], (size_t)B * d[l + 1]);
  ok = ok && dev_alloc(n, &n->dY, (size_t)B * nout) && dev_alloc(n, &n->dYT, (size_t)B * nout) &&
       dev_alloc(n, &n->dP2, (size_t)B * h2) && dev_alloc(n, &n->dP2T, (size_t)B * h2) &&
       dev_alloc(n, &n->dP1T, (size_t)B * h1);
  if (!ok) {
    bb_fail(ctx, BB_ERR_NOMEM, "MLP allocation failed");
    for (void* a : n->allocs) cudaFree(a);
    delete n;
    return BB_ERR_NOMEM;
  }
  // uniform(-1/sqrt(in), 1/sqrt(in)) weights, zero biases
  std::vector<float> h(off, 0.0f);
  uint64_t s = seed;
  for (int l = 0; l < 3; ++l) {
    const double a = 1.0 / std::sqrt((double)d[l]);
    for (int64_t i = 0; i < (int64_t)d[l + 1] * d[l]; ++i) {
      const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      h[n->oW[l] + i] = (float)((2.0 * u - 1.0) * a);
    }
  }
  if (cudaMemcpy(n->p, h.data(), off * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(n->m, 0, off * sizeof(float)) != cudaSuccess ||
      cudaMemset(n->v, 0, off * sizeof(float)) != cudaSuccess ||
      cudaMemset(n->g, 0, off * sizeof(float)) != cudaSuccess || refresh_bf16(n, nullptr) ||
      cudaDeviceSynchronize() != cudaSuccess) {
    bb_fail(ctx, BB_ERR_CUDA, "MLP initialisation failed");
    for (void* a : n->allocs) cudaFree(a);
    delete n;
    return BB_ERR_CUDA;
  }
  *out = n;
  return BB_OK;
}

extern "C" int bb_mlp_destroy(bb_mlp* n) {
  if (!n) return BB_ERR_ARG;
  cudaSetDevice(n->ctx->device);
  for (void* a : n->allocs) cudaFree(a);
  delete n;
  return BB_OK;
}

extern "C" int64_t bb_mlp_num_params(const bb_mlp* n) { return n ? n->nparams : -1; }

extern "C" int bb_mlp_set_params(bb_mlp* n, const float* host, void* stream) {
  if (!n || !host) return BB_ERR_ARG;
  int rc = bb_set_device(n->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  BB_CUDA(n->ctx, cudaMemcpyAsync(n->p, host, n->nparams * sizeof(float), cudaMemcpyHostToDevice, st));
  BB_CUDA(n->ctx, cudaMemsetAsync(n->m, 0, n->nparams * sizeof(float), st));
  BB_CUDA(n->ctx, cudaMemsetAsync(n->v, 0, n->nparams * sizeof(float), st));
  n->steps = 0;
  rc = refresh_bf16(n, st);
  if (rc) return rc;
  BB_CUDA(n->ctx, cudaStreamSynchronize(st));
  return BB_OK;
}

extern "C" int bb_mlp_get_params(bb_mlp* n, float* host, void* stream) {
  if (!n || !host) return BB_ERR_ARG;
  int rc = bb_set_device(n->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  BB_CUDA(n->ctx, cudaMemcpyAsync(host, n->p, n->nparams * sizeof(float), cudaMemcpyDeviceToHost, st));
  BB_CUDA(n->ctx, cudaStreamSynchronize(st));
  return BB_OK;
}

extern "C" int bb_mlp_get_grads(bb_mlp* n, float* host, void* stream) {
  if (!n || !host) return BB_ERR_ARG;
  int rc = bb_set_device(n->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  BB_CUDA(n->ctx, cudaMemcpyAsync(host, n->g, n->nparams * sizeof(float), cudaMemcpyDeviceToHost, st));
  BB_CUDA(n->ctx, cudaStreamSynchronize(st));
  return BB_OK;
}

extern "C" int bb_mlp_fwd(bb_mlp* n, int64_t B, const void* X, const void* XT, float* Y,
                          int train, void* stream) {
  if (!n) return BB_ERR_ARG;
  bb_ctx* ctx = n->ctx;
  if (!X || !Y || (train && !XT)) return bb_fail(ctx, BB_ERR_ARG, "bb_mlp_fwd: null pointer");
  if (B < 1 || B > n->max_batch) return bb_fail(ctx, BB_ERR_ARG, "batch outside [1, max_batch]");
  if (train && B % 8 != 0) return bb_fail(ctx, BB_ERR_ARG, "training batch must be a multiple of 8");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int* d = n->dim;
  const void* in = X;
  for (int l = 0; l < 2; ++l) {
    GemmEpilogue e = epi(n);
    e.bias = n->p + n->ob[l];
    e.act = 1;
    e.Pre = train ? n->pre[l] : nullptr;
    e.Cb = n->H[l];
    e.CbT = train ? n->HT[l] : nullptr;
    e.ldc = d[l + 1];
    e.ldt = (int)B;
    rc = bb_gemm_launch(ctx, B, d[l + 1], d[l], in, n->Wb[l], e, st);
    if (rc) return rc;
    in = n->H[l];
  }
  GemmEpilogue e = epi(n);
  e.bias = n->p + n->ob[2];
  e.Cf = Y;
  e.ldc = d[3];
  rc = bb_gemm_launch(ctx, B, d[3], d[2], in, n->Wb[2], e, st);
  if (rc) return rc;
  n->fwd_B = train ? B : -1;
  n->XT = train ? XT : nullptr;
  return BB_OK;
}

extern "C" int bb_mlp_bwd(bb_mlp* n, int64_t B, const float* Y, const float* T, double* loss_dev,
                          void* stream) {
  if (!n) return BB_ERR_ARG;
  bb_ctx* ctx = n->ctx;
  if (!Y || !T || !loss_dev) return bb_fail(ctx, BB_ERR_ARG, "bb_mlp_bwd: null pointer");
  if (B != n->fwd_B || !n->XT)
    return bb_fail(ctx, BB_ERR_ARG, "bb_mlp_bwd needs a training bb_mlp_fwd of the same batch");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int* d = n->dim;
  const int nin = d[0], h1 = d[1], h2 = d[2], nout = d[3];
  BB_CUDA(ctx, cudaMemsetAsync(n->g, 0, n->nparams * sizeof(float), st));
  BB_CUDA(ctx, cudaMemsetAsync(loss_dev, 0, sizeof(double), st));
  {
    dim3 grid((nout + 31) / 32, (unsigned)((B + 31) / 32));
    const double inv = 1.0 / ((double)B * nout);
    mse_grad_kernel<<<grid, dim3(32, 8), 0, st>>>(Y, T, B, nout, (float)(2.0 * inv), (float)inv,
                                                  n->dY, n->dYT, n->g + n->ob[2], loss_dev);
    rc = bb_check_launch(ctx, "mse_grad_kernel");
    if (rc) return rc;
  }
  // dW3 = dY^T H2
  GemmEpilogue e = epi(n);
  e.Cf = n->g + n->oW[2];
  e.ldc = h2;
  e.kt_per = kt_split(ctx, nout, h2, (int)B);
  if ((rc = bb_gemm_launch(ctx, nout, h2, (int)B, n->dYT, n->HT[1], e, st))) return rc;
  // dP2 = (dY W3) * GELU'(pre2), db2
  e = epi(n);
  e.act = 2;
  e.Pre = n->pre[1];
  e.Cb = n->dP2;
  e.CbT = n->dP2T;
  e.bias_grad = n->g + n->ob[1];
  e.ldc = h2;
  e.ldt = (int)B;
  if ((rc = bb_gemm_launch(ctx, B, h2, nout, n->dY, n->WT[2], e, st))) return rc;
  // dW2 = dP2^T H1
  e = epi(n);
  e.Cf = n->g + n->oW[1];
  e.ldc = h1;
  e.kt_per = kt_split(ctx, h2, h1, (int)B);
  if ((rc = bb_gemm_launch(ctx, h2, h1, (int)B, n->dP2T, n->HT[0], e, st))) return rc;
  // dP1 = (dP2 W2) * GELU'(pre1), db1
  e = epi(n);
  e.act = 2;
  e.Pre = n->pre[0];
  e.CbT = n->dP1T;
  e.bias_grad = n->g + n->ob[0];
  e.ldc = h1;
  e.ldt = (int)B;
  if ((rc = bb_gemm_launch(ctx, B, h1, h2, n->dP2, n->WT[1], e, st))) return rc;
  // dW1 = dP1^T X
  e = epi(n);
  e.Cf = n->g + n->oW[0];
  e.ldc = nin;
  e.kt_per = kt_split(ctx, h1, nin, (int)B);
  if ((rc = bb_gemm_launch(ctx, h1, nin, (int)B, n->dP1T, n->XT, e, st))) return rc;
  return BB_OK;
}

extern "C" int bb_mlp_step(bb_mlp* n, float lr, float beta1, float beta2, float eps,
                           void* stream) {
  if (!n) return BB_ERR_ARG;
  if (!(lr > 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) ||
      !(eps > 0.0f))
    return bb_fail(n->ctx, BB_ERR_ARG, "bad Adam hyper-parameters");
  int rc = bb_set_device(n->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  n->steps += 1;
  const double c1 = 1.0 / (1.0 - std::pow((double)beta1, (double)n->steps));
  const double c2 = 1.0 / (1.0 - std::pow((double)beta2, (double)n->steps));
  adam_kernel<<<grid_for(n->ctx, n->nparams, 256), 256, 0, st>>>(
      n->p, n->g, n->m, n->v, n->nparams, lr, beta1, beta2, eps, (float)c1, (float)c2);
  rc = bb_check_launch(n->ctx, "adam_kernel");
  if (rc) return rc;
  return refresh_bf16(n, st);
}

extern "C" int bb_transpose_bf16(bb_ctx* ctx, int64_t rows, int cols, const void* in, void* out,
                                 void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!in || !out || rows < 0 || cols < 0 || (rows + 31) / 32 > 65535)
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_transpose_bf16");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  if (rows == 0 || cols == 0) return BB_OK;
  dim3 grid((cols + 31) / 32, (unsigned)((rows + 31) / 32));
  transpose_bf16_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)in, rows, cols, (__nv_bfloat16*)out);
  return bb_check_launch(ctx, "transpose_bf16_kernel");
}

extern "C" int bb_closure_features(bb_ctx* ctx, int N, int64_t K, int nf, const int32_t* conn,
                                   int dtype, const void* q, float scale, void* X, void* XT,
                                   void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N) || K < 1 || (nf != 4 && nf != 6) || !valid_dtype(dtype) || !conn || !q ||
      !X || K > ((int64_t)1 << 27))
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_closure_features");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "degree tables unavailable");
  int* status = bb_ctx_status_word(ctx);
  if (!status) return bb_fail(ctx, BB_ERR_NOMEM, "status word allocation failed");
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = (int)std::min<int64_t>(K, (int64_t)ctx->num_sms * 32);
  if (dtype == BB_F64)
    closure_features_kernel<double><<<grid, 256, 0, st>>>(t->d_words, t->o_fvol, t->o_fperm, N, K,
                                                          nf, conn, (const double*)q, scale,
                                                          (__nv_bfloat16*)X, status);
  else
    closure_features_kernel<float><<<grid, 256, 0, st>>>(t->d_words, t->o_fvol, t->o_fperm, N, K,
                                                         nf, conn, (const float*)q, scale,
                                                         (__nv_bfloat16*)X, status);
  rc = bb_check_launch(ctx, "closure_features_kernel");
  if (rc || !XT) return rc;
  const int nin = nf * np3(N) + 4 * nf * np2(N);
  return bb_transpose_bf16(ctx, K, nin, X, XT, stream);
}

extern "C" int bb_closure_apply(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, float alpha,
                                const float* Y, void* q, void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N) || K < 0 || nf < 1 || !valid_dtype(dtype) || !Y || !q)
    return bb_fail(ctx, BB_ERR_ARG, "bad argument to bb_closure_apply");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  if (K == 0) return BB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = K * nf * np3(N);
  const int grid = grid_for(ctx, n, 256);
  if (dtype == BB_F64)
    closure_apply_kernel<double><<<grid, 256, 0, st>>>(np3(N), K, nf, alpha, Y, (double*)q);
  else
    closure_apply_kernel<float><<<grid, 256, 0, st>>>(np3(N), K, nf, alpha, Y, (float*)q);
  return bb_check_launch(ctx, "closure_apply_kernel");
}
