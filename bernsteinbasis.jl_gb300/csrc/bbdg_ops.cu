// Context, per-degree tables and the reference-element operator kernels (sm_103a).
//
// Operators keep the reference's matrix layout (one column per element) and semantics:
//   derivative  src/BernsteinDerivativeMatrix_3D.jl:96-231
//   lift        src/BernsteinLift.jl:66-164 (elevation, reduction, face lift), :191-269
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "bbdg_internal.cuh"
#include "bbdg_stack_slots.cuh"

// -------------------------------------------------------------------------------------
// context
// -------------------------------------------------------------------------------------
int bb_fail(bb_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return code;
}

int bb_set_device(bb_ctx* ctx) {
  BB_CUDA(ctx, cudaSetDevice(ctx->device));
  return BB_OK;
}

int bb_check_launch(bb_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bb_fail(ctx, BB_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  ctx->launches++;
  return BB_OK;
}

int bb_device_status_error(bb_ctx* ctx, int word) {
  if (word & 2)
    return bb_fail(ctx, BB_ERR_TIMEOUT, "a device-side bounded wait ran out (status 0x%x)", word);
  if (word & 4)
    return bb_fail(ctx, BB_ERR_DEVICE, "debug index check failed (status 0x%x)", word);
  return bb_fail(ctx, BB_ERR_DEVICE, "device check failed: corrupt connectivity (status 0x%x)",
                 word);
}

extern "C" int bb_ctx_set_wait_limit(bb_ctx* ctx, uint32_t polls) {
  if (!ctx) return BB_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->wait_iters = polls;
  ++ctx->config_epoch;
  return BB_OK;
}

extern "C" int bb_ctx_set_test_fault(bb_ctx* ctx, int mode) {
  if (!ctx || mode < 0 || mode > 1) return BB_ERR_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->test_fault = mode;
  ++ctx->config_epoch;
  return BB_OK;
}

extern "C" int bb_version(void) { return 10000; }

extern "C" int bb_ctx_create(int device, bb_ctx** out) {
  if (!out) return BB_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return BB_ERR_ARG;
  bb_ctx* c = new (std::nothrow) bb_ctx();
  if (!c) return BB_ERR_NOMEM;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) !=
          cudaSuccess) {
    delete c;
    return BB_ERR_CUDA;
  }
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  c->smem_optin = (size_t)optin;
  *out = c;
  return BB_OK;
}

static void free_tables(DegTables* t) {
  if (!t) return;
  cudaFree(t->d_words);
  delete t;
}

extern "C" int bb_ctx_destroy(bb_ctx* ctx) {
  if (!ctx) return BB_ERR_ARG;
  cudaSetDevice(ctx->device);
  for (auto& t : ctx->tabs) free_tables(t);
  cudaFree(ctx->d_red);
  cudaFreeHost(ctx->h_red);
  cudaFree(ctx->d_status);
  delete ctx;
  return BB_OK;
}

extern "C" const char* bb_ctx_last_error(const bb_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int64_t bb_ctx_launch_count(const bb_ctx* ctx) { return ctx ? ctx->launches : -1; }

// l_j(N) = (-1)^j C(N, j) / (1 + j)  (src/constants.jl:10-12)
// Stage-kernel lift-stack slot of entry q (the generated tables of bbdg_stack_slots.cuh).
static int stack_slot_of(int N, int q) {
  switch (N) {
    case 9: return stack_slot<9>(q);
    case 10: return stack_slot<10>(q);
    default: return q;
  }
}

const DegTables* bb_tables(bb_ctx* ctx, int N) {
  if (!valid_degree(N)) return nullptr;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (ctx->tabs[N]) return ctx->tabs[N];
  DegTables* t = new DegTables();
  t->N = N;
  t->Np = np3(N);
  t->NpM1 = np3(N - 1);
  t->Nfp = np2(N);
  const int n2 = np3(N + 1);
  int off = 0;
  t->o_node3 = off; off += t->Np;
  t->o_node3m1 = off; off += t->NpM1;
  t->o_node2 = off; off += (n2 + 1) / 2;
  t->o_fvol = off; off += (4 * t->Nfp + 1) / 2;
  t->o_fperm = off; off += (6 * t->Nfp + 1) / 2;
  t->o_fstack = off; off += (4 * t->Np + 1) / 2;
  t->o_sslot = off; off += (t->Np + 1) / 2;
  t->nwords = off;
  if (off != deg_table_words(N)) {  // the tile-size estimates rely on the same count
    delete t;
    return nullptr;
  }
  std::vector<uint32_t> w(off, 0u);
  auto put16 = [&](int word_off, int idx, int v) {
    uint16_t* p = reinterpret_cast<uint16_t*>(w.data() + word_off);
    p[idx] = (uint16_t)v;
  };
  int m = 0;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N - k; ++j)
      for (int i = 0; i <= N - j - k; ++i) w[t->o_node3 + m++] = i | (j << 8) | (k << 16);
  m = 0;
  for (int k = 0; k <= N - 1; ++k)
    for (int j = 0; j <= N - 1 - k; ++j)
      for (int i = 0; i <= N - 1 - j - k; ++i) w[t->o_node3m1 + m++] = i | (j << 8) | (k << 16);
  for (int n = 0; n <= N + 1; ++n) {
    int base = np3(n - 1), q = 0;
    for (int b = 0; b <= n; ++b)
      for (int a = 0; a <= n - b; ++a) put16(t->o_node2, base + q++, a | (b << 8));
  }
  for (int f = 0; f < 4; ++f) {
    int q = 0;
    for (int b = 0; b <= N; ++b)
      for (int a = 0; a <= N - b; ++a) put16(t->o_fvol, f * t->Nfp + q++, face_vol(N, f, a, b, 0));
  }
  for (int o = 0; o < 6; ++o) {
    int q = 0;
    for (int b = 0; b <= N; ++b)
      for (int a = 0; a <= N - b; ++a) {
        const int wgt[3] = {a, b, N - a - b};
        int wn[3];
        for (int v = 0; v < 3; ++v) wn[perm_of(o, v)] = wgt[v];
        put16(t->o_fperm, o * t->Nfp + q++, ij2(N, wn[0], wn[1]));
      }
  }
  // face f's lift stack in stack order (layer d outer, then j, then i, i + j <= N - d) ->
  // volume index of the coefficient it lands on
  for (int f = 0; f < 4; ++f) {
    int q = 0;
    for (int d = 0; d <= N; ++d)
      for (int b = 0; b <= N - d; ++b)
        for (int a = 0; a <= N - d - b; ++a) put16(t->o_fstack, f * t->Np + q++, face_vol(N, f, a, b, d));
  }
  for (int q = 0; q < t->Np; ++q) put16(t->o_sslot, q, stack_slot_of(N, q));
  // (the lift weights l_j(N), constants.jl:10-12, are carried by the chain recursion:
  // no table of them is needed)
  bool ok = cudaMalloc(&t->d_words, sizeof(uint32_t) * off) == cudaSuccess &&
            cudaMemcpy(t->d_words, w.data(), sizeof(uint32_t) * off, cudaMemcpyHostToDevice) ==
                cudaSuccess;
  if (!ok) {
    free_tables(t);
    return nullptr;
  }
  ctx->tabs[N] = t;
  return t;
}

// -------------------------------------------------------------------------------------
// derivative kernels
// -------------------------------------------------------------------------------------
// (D x)_row for one axis, written as the reference does (fast_D{r,s,t}_multiply!):
// val = sum of (multi-index entry) * (difference of two neighbours), out = val / 2 (in
// double the halving rides in the weights, halved_weight / finish_half).
template <class T>
__device__ __forceinline__ T deriv_row(int axis, int N, const T* x, int i, int j, int k, int row) {
  const int l = N - i - j - k;
  const T xr = x[row];
  T val;
  if (axis == 0) {  // BernsteinDerivativeMatrix_3D.jl:96-132
    T x4 = (i > 0) ? x[ijk3(N, i - 1, j, k)] : T(0);
    val = halved_weight<T>(i) * (xr - x4);
    if (j > 0) val += halved_weight<T>(j) * (x[ijk3(N, i + 1, j - 1, k)] - x[ijk3(N, i, j - 1, k)]);
    if (k > 0) val += halved_weight<T>(k) * (x[ijk3(N, i + 1, j, k - 1)] - x[ijk3(N, i, j, k - 1)]);
    T x1 = (l > 0) ? x[ijk3(N, i + 1, j, k)] : T(0);
    val += halved_weight<T>(l) * (x1 - xr);
  } else if (axis == 1) {  // :138-174
    val = T(0);
    if (i > 0) val = halved_weight<T>(i) * (x[ijk3(N, i - 1, j + 1, k)] - x[ijk3(N, i - 1, j, k)]);
    T x4 = (j > 0) ? x[ijk3(N, i, j - 1, k)] : T(0);
    val += halved_weight<T>(j) * (xr - x4);
    if (k > 0) val += halved_weight<T>(k) * (x[ijk3(N, i, j + 1, k - 1)] - x[ijk3(N, i, j, k - 1)]);
    T x2 = (l > 0) ? x[ijk3(N, i, j + 1, k)] : T(0);
    val += halved_weight<T>(l) * (x2 - xr);
  } else {  // :180-216
    val = T(0);
    if (i > 0) val = halved_weight<T>(i) * (x[ijk3(N, i - 1, j, k + 1)] - x[ijk3(N, i - 1, j, k)]);
    if (j > 0) val += halved_weight<T>(j) * (x[ijk3(N, i, j - 1, k + 1)] - x[ijk3(N, i, j - 1, k)]);
    T x4 = (k > 0) ? x[ijk3(N, i, j, k - 1)] : T(0);
    val += halved_weight<T>(k) * (xr - x4);
    T x3 = (l > 0) ? x[ijk3(N, i, j, k + 1)] : T(0);
    val += halved_weight<T>(l) * (x3 - xr);
  }
  return finish_half(val);
}

// Applies up to three derivative operators (mask bits r,s,t) to EPB element columns per
// block iteration: stage the columns in shared memory, one thread per output coefficient.
template <class T>
__global__ void __launch_bounds__(256) deriv_kernel(DegTables tab, const uint32_t* __restrict__ gtab,
                                                    int64_t K, int epb, int mask,
                                                    const T* __restrict__ x, T* __restrict__ o0,
                                                    T* __restrict__ o1, T* __restrict__ o2) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = tab.N, Np = tab.Np;
  T* sx = reinterpret_cast<T*>(smem);
  uint32_t* stab = reinterpret_cast<uint32_t*>(smem + align16(sizeof(T) * (size_t)epb * Np));
  const SmemTables st = load_tables(tab, gtab, stab);
  const int64_t nblk = (K + epb - 1) / epb;
  T* outs[3] = {o0, o1, o2};
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    copy_g2s(sx, x + e0 * Np, ne * Np);
    __syncthreads();
    for (int it = threadIdx.x; it < ne * Np; it += blockDim.x) {
      const int le = it / Np, row = it - le * Np;
      const uint32_t c = st.node3[row];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
#pragma unroll
      for (int a = 0; a < 3; ++a)
        if (mask & (1 << a)) outs[a][e0 * Np + it] = deriv_row<T>(a, N, sx + le * Np, i, j, k, row);
    }
  }
}

// Factored form of the same operators, D_a x(alpha) = 1/2 sum_b alpha_b w_a(alpha - e_b) with
// w_a(beta) = x(beta + e_a) - x(beta + e_3) at degree N-1 (b over the four barycentric
// indices; the reference's four terms per row, BernsteinDerivativeMatrix_3D.jl:96-216, are
// exactly these). Per block: packed index tables in shared memory built once, then per tile
// of EPB elements one pass forms w for every requested axis and one pass forms the outputs.
template <class T>
__global__ void __launch_bounds__(256) deriv_fact_kernel(DegTables tab,
                                                         const uint32_t* __restrict__ gtab,
                                                         int64_t K, int epb, int mask,
                                                         const T* __restrict__ x,
                                                         T* __restrict__ o0, T* __restrict__ o1,
                                                         T* __restrict__ o2) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = tab.N, Np = tab.Np, NPM1 = tab.NpM1, NW = NPM1 + 1;
  T* sx = reinterpret_cast<T*>(smem);                  // [epb][Np]
  T* sW = sx + (size_t)epb * Np;                       // [3][epb][NW], entry NPM1 = 0
  uint2* sVN = reinterpret_cast<uint2*>(smem + align16(sizeof(T) * ((size_t)epb * Np + 3 * (size_t)epb * NW)));
  uint2* sGA = sVN + NPM1;                             // [Np] degree N-1 indices of alpha - e_b
  uint32_t* sGW = reinterpret_cast<uint32_t*>(sGA + Np);  // [Np] alpha_b as 4 bytes
  const uint32_t Z = (uint32_t)NPM1;
  for (int t = threadIdx.x; t < NPM1; t += blockDim.x) {
    const uint32_t c = gtab[tab.o_node3m1 + t];
    const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
    sVN[t] = make_uint2(ijk3(N, i + 1, j, k) | (ijk3(N, i, j + 1, k) << 16),
                        ijk3(N, i, j, k + 1) | (ijk3(N, i, j, k) << 16));
  }
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {
    const uint32_t c = gtab[tab.o_node3 + t];
    const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
    const uint32_t m0 = i > 0 ? ijk3(N - 1, i - 1, j, k) : Z;
    const uint32_t m1 = j > 0 ? ijk3(N - 1, i, j - 1, k) : Z;
    const uint32_t m2 = k > 0 ? ijk3(N - 1, i, j, k - 1) : Z;
    const uint32_t m3 = l > 0 ? ijk3(N - 1, i, j, k) : Z;
    sGA[t] = make_uint2(m0 | (m1 << 16), m2 | (m3 << 16));
    sGW[t] = (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16) | ((uint32_t)l << 24);
  }
  for (int t = threadIdx.x; t < 3 * epb; t += blockDim.x) sW[(size_t)t * NW + NPM1] = T(0);
  T* outs[3] = {o0, o1, o2};
  // it / d as (it * ceil(2^32 / d)) >> 32 (exact for it < 2^32 / d; d = 1 gives 2^32)
  const uint64_t inv_m1 = 0xFFFFFFFFull / (uint64_t)NPM1 + 1ull;
  const uint64_t inv_np = 0xFFFFFFFFull / (uint64_t)Np + 1ull;
  const int64_t nblk = (K + epb - 1) / epb;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    copy_g2s(sx, x + e0 * Np, ne * Np);
    __syncthreads();
    for (int it = threadIdx.x; it < ne * NPM1; it += blockDim.x) {
      const int le = (int)(((uint64_t)it * inv_m1) >> 32), b = it - le * NPM1;
      const uint2 vn = sVN[b];
      const T* xe = sx + (size_t)le * Np;
      const T x3 = xe[vn.y >> 16];
      if (mask & 1) sW[((size_t)0 * epb + le) * NW + b] = xe[vn.x & 0xffff] - x3;
      if (mask & 2) sW[((size_t)1 * epb + le) * NW + b] = xe[vn.x >> 16] - x3;
      if (mask & 4) sW[((size_t)2 * epb + le) * NW + b] = xe[vn.y & 0xffff] - x3;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < ne * Np; it += blockDim.x) {
      const int le = (int)(((uint64_t)it * inv_np) >> 32), n = it - le * Np;
      const uint2 ga = sGA[n];
      const uint32_t gw = sGW[n];
      const int m0 = ga.x & 0xffff, m1 = ga.x >> 16, m2 = ga.y & 0xffff, m3 = ga.y >> 16;
      const T a0 = halved_weight<T>(gw & 0xff), a1 = halved_weight<T>((gw >> 8) & 0xff),
              a2 = halved_weight<T>((gw >> 16) & 0xff), a3 = halved_weight<T>(gw >> 24);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (!(mask & (1 << a))) continue;
        const T* w = sW + ((size_t)a * epb + le) * NW;
        outs[a][e0 * Np + it] = finish_half(a0 * w[m0] + a1 * w[m1] + a2 * w[m2] + a3 * w[m3]);
      }
    }
  }
}

// -------------------------------------------------------------------------------------
// lift kernels
// -------------------------------------------------------------------------------------
// Full lift (nfaces = 4) or single-face lift (nfaces = 1, face index 3 = the face written
// directly, src/BernsteinLift.jl:139-164) of EPB element columns per block iteration.
template <class T>
__global__ void __launch_bounds__(256) lift_kernel(DegTables tab, const uint32_t* __restrict__ gtab,
                                                   int64_t K, int epb,
                                                   int nfaces, const T* __restrict__ x,
                                                   T* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = tab.N, Np = tab.Np, Nfp = tab.Nfp;
  const int S = np2(N + 1);
  const int in_cols = nfaces * Nfp;
  T* sin = reinterpret_cast<T*>(smem);
  T* sout = sin + epb * in_cols;
  T* bufA = sout + epb * Np;
  T* bufB = bufA + epb * S;
  uint32_t* stab = reinterpret_cast<uint32_t*>(
      smem + align16(sizeof(T) * ((size_t)epb * (in_cols + Np + 2 * S))));
  const SmemTables st = load_tables(tab, gtab, stab);
  const int64_t nblk = (K + epb - 1) / epb;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    copy_g2s(sin, x + e0 * in_cols, ne * in_cols);
    for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) sout[t] = T(0);
    __syncthreads();
    if (nfaces == 4) {
      // face 4 (t = -1) first, then f1, f2, f3, as src/BernsteinLift.jl:202-218
      for (int q = 0; q < 4; ++q) {
        const int f = (q + 3) & 3;  // faces 3, 0, 1, 2
        lift_face_accumulate<T>(N, f, ne, 1, st.node2, sin + f * Nfp, in_cols, 0, sout, Np, 0,
                                bufA, bufB);
      }
    } else {
      lift_face_accumulate<T>(N, 3, ne, 1, st.node2, sin, Nfp, 0, sout, Np, 0, bufA, bufB);
    }
    copy_s2g(out + e0 * Np, sout, ne * Np);
  }
}

// Fused operator pass: Dr, Ds, Dt of the volume columns and the lift of the face columns
// of the same EPB elements, one launch, each input read once.
template <class T>
__global__ void __launch_bounds__(256) fused_kernel(DegTables tab, const uint32_t* __restrict__ gtab,
                                                    int64_t K, int epb,
                                                    const T* __restrict__ x, const T* __restrict__ faces,
                                                    T* __restrict__ dr, T* __restrict__ ds,
                                                    T* __restrict__ dt, T* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = tab.N, Np = tab.Np, Nfp = tab.Nfp;
  const int S = np2(N + 1);
  const int in_cols = 4 * Nfp;
  T* sx = reinterpret_cast<T*>(smem);
  T* sin = sx + epb * Np;
  T* sout = sin + epb * in_cols;
  T* bufA = sout + epb * Np;
  T* bufB = bufA + epb * S;
  uint32_t* stab = reinterpret_cast<uint32_t*>(
      smem + align16(sizeof(T) * ((size_t)epb * (Np + in_cols + Np + 2 * S))));
  const SmemTables st = load_tables(tab, gtab, stab);
  T* outs[3] = {dr, ds, dt};
  const int64_t nblk = (K + epb - 1) / epb;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    copy_g2s(sx, x + e0 * Np, ne * Np);
    copy_g2s(sin, faces + e0 * in_cols, ne * in_cols);
    for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) sout[t] = T(0);
    __syncthreads();
    for (int it = threadIdx.x; it < ne * Np; it += blockDim.x) {
      const int le = it / Np, row = it - le * Np;
      const uint32_t c = st.node3[row];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
#pragma unroll
      for (int a = 0; a < 3; ++a) outs[a][e0 * Np + it] = deriv_row<T>(a, N, sx + le * Np, i, j, k, row);
    }
    for (int q = 0; q < 4; ++q) {
      const int f = (q + 3) & 3;  // faces 3, 0, 1, 2
      lift_face_accumulate<T>(N, f, ne, 1, st.node2, sin + f * Nfp, in_cols, 0, sout, Np, 0,
                              bufA, bufB);
    }
    copy_s2g(out + e0 * Np, sout, ne * Np);
  }
}

// 2D elevation (degree N -> N+1) or reduction (degree N -> N-1), one thread per output.
template <class T>
__global__ void tri_op_kernel(int N, int64_t K, int elevate, const T* __restrict__ x,
                              T* __restrict__ out) {
  const int nin = np2(N), nout = elevate ? np2(N + 1) : np2(N - 1);
  const int64_t total = K * nout;
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < total;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = it / nout;
    int m = (int)(it - e * nout);
    const T* xe = x + e * nin;
    const int n = elevate ? N + 1 : N - 1;
    int b = 0;
    while (m >= tri_off(n, b + 1)) ++b;
    const int a = m - tri_off(n, b);
    T val;
    if (elevate) {  // src/BernsteinLift.jl:100-125
      const int c = n - a - b;
      val = T(0);
      if (a > 0) val = T(a) * xe[ij2(N, a - 1, b)];
      if (b > 0) val = fma(T(b), xe[ij2(N, a, b - 1)], val);
      if (c > 0) val = fma(T(c), xe[ij2(N, a, b)], val);
      val = val / T(N + 1);
    } else {  // src/BernsteinLift.jl:66-90
      val = fma(T(a + 1), xe[ij2(N, a + 1, b)],
                fma(T(b + 1), xe[ij2(N, a, b + 1)], T(N - a - b) * xe[ij2(N, a, b)]));
      val = val / T(N);
    }
    out[it] = val;
  }
}

// -------------------------------------------------------------------------------------
// launch helpers
// -------------------------------------------------------------------------------------
static int grid_for(bb_ctx* ctx, int64_t nblk, int per_sm) {
  int64_t g = (int64_t)ctx->num_sms * per_sm;
  if (nblk < g) g = nblk;
  return (int)(g < 1 ? 1 : g);
}

template <class T>
static int launch_deriv(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x,
                        void* o0, void* o1, void* o2, cudaStream_t st) {
  if (sizeof(T) == 4) {
    const int rc = bb_deriv_fast(ctx, t, K, mask, x, o0, o1, o2, st);
    if (rc >= 0) return rc;  // otherwise no specialised kernel for this degree or mask
  }
  {
    // factored kernel: tile of epb elements plus the w rows and the index tables
    int epb = 16;
    size_t smem = 0;
    for (; epb >= 1; epb /= 2) {
      smem = align16(sizeof(T) * ((size_t)epb * t->Np + 3 * (size_t)epb * (t->NpM1 + 1))) +
             8 * (size_t)t->NpM1 + 8 * (size_t)t->Np + 4 * (size_t)t->Np;
      if (smem <= 48 * 1024) break;
    }
    if (epb >= 1 && t->Np <= 65535) {
      BB_CUDA(ctx, cudaFuncSetAttribute(deriv_fact_kernel<T>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      const int64_t nblk = (K + epb - 1) / epb;
      deriv_fact_kernel<T><<<grid_for(ctx, nblk, 8), 256, smem, st>>>(
          *t, t->d_words, K, epb, mask, (const T*)x, (T*)o0, (T*)o1, (T*)o2);
      return bb_check_launch(ctx, "deriv_fact_kernel");
    }
  }
  const int epb = 8;
  const size_t smem = align16(sizeof(T) * (size_t)epb * t->Np) + 4 * (size_t)t->nwords;
  if (smem > ctx->smem_optin) return bb_fail(ctx, BB_ERR_ARG, "degree too large for deriv tile");
  BB_CUDA(ctx, cudaFuncSetAttribute(deriv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const int64_t nblk = (K + epb - 1) / epb;
  deriv_kernel<T><<<grid_for(ctx, nblk, 8), 256, smem, st>>>(
      *t, t->d_words, K, epb, mask, (const T*)x, (T*)o0, (T*)o1, (T*)o2);
  return bb_check_launch(ctx, "deriv_kernel");
}

template <class T>
static int launch_lift(bb_ctx* ctx, const DegTables* t, int64_t K, int nfaces, const void* x,
                       void* out, cudaStream_t st) {
  if (sizeof(T) == 4) {
    const int rc = bb_lift_fast(ctx, t, K, nfaces, x, out, st);
    if (rc >= 0) return rc;  // otherwise no specialised kernel for this degree
  }
  const int S = np2(t->N + 1);
  int epb = 8;
  size_t smem = 0;
  for (; epb >= 1; epb /= 2) {
    smem = align16(sizeof(T) * ((size_t)epb * (nfaces * t->Nfp + t->Np + 2 * S))) +
           4 * (size_t)t->nwords;
    if (smem <= 64 * 1024) break;
  }
  if (epb < 1) return bb_fail(ctx, BB_ERR_ARG, "degree too large for lift tile");
  BB_CUDA(ctx, cudaFuncSetAttribute(lift_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const int64_t nblk = (K + epb - 1) / epb;
  lift_kernel<T><<<grid_for(ctx, nblk, 4), 256, smem, st>>>(*t, t->d_words, K, epb, nfaces,
                                                             (const T*)x, (T*)out);
  return bb_check_launch(ctx, "lift_kernel");
}

template <class T>
static int launch_fused(bb_ctx* ctx, const DegTables* t, int64_t K, const void* x, const void* faces,
                        void* dr, void* ds, void* dt, void* out, cudaStream_t st) {
  const int S = np2(t->N + 1);
  int epb = 8;
  size_t smem = 0;
  for (; epb >= 1; epb /= 2) {
    smem = align16(sizeof(T) * ((size_t)epb * (2 * t->Np + 4 * t->Nfp + 2 * S))) +
           4 * (size_t)t->nwords;
    if (smem <= 64 * 1024) break;
  }
  if (epb < 1) return bb_fail(ctx, BB_ERR_ARG, "degree too large for fused tile");
  BB_CUDA(ctx, cudaFuncSetAttribute(fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const int64_t nblk = (K + epb - 1) / epb;
  fused_kernel<T><<<grid_for(ctx, nblk, 4), 256, smem, st>>>(*t, t->d_words, K, epb, (const T*)x,
                                                              (const T*)faces, (T*)dr, (T*)ds,
                                                              (T*)dt, (T*)out);
  return bb_check_launch(ctx, "fused_kernel");
}

static int check_common(bb_ctx* ctx, int N, int64_t K, int dtype) {
  if (!ctx) return BB_ERR_ARG;
  if (!valid_degree(N)) return bb_fail(ctx, BB_ERR_ARG, "degree N=%d outside 1..%d", N, BB_MAX_DEGREE);
  if (K < 0) return bb_fail(ctx, BB_ERR_ARG, "negative element count");
  if (!valid_dtype(dtype)) return bb_fail(ctx, BB_ERR_ARG, "dtype must be BB_F32 or BB_F64");
  return bb_set_device(ctx);
}

// -------------------------------------------------------------------------------------
// C ABI
// -------------------------------------------------------------------------------------
extern "C" int bb_deriv_apply(bb_ctx* ctx, int axis, int N, int64_t K, int dtype, const void* x,
                              void* out, void* stream) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (axis < 0 || axis > 2) return bb_fail(ctx, BB_ERR_ARG, "axis must be 0, 1 or 2");
  if (K == 0) return BB_OK;
  if (!x || !out) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  if (x == out) return bb_fail(ctx, BB_ERR_ARG, "out must not alias x");
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  void* o[3] = {nullptr, nullptr, nullptr};
  o[axis] = out;
  return dtype == BB_F64
             ? launch_deriv<double>(ctx, t, K, 1 << axis, x, o[0], o[1], o[2], (cudaStream_t)stream)
             : launch_deriv<float>(ctx, t, K, 1 << axis, x, o[0], o[1], o[2], (cudaStream_t)stream);
}

extern "C" int bb_grad_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* dr,
                             void* ds, void* dt, void* stream) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (K == 0) return BB_OK;
  if (!x || !dr || !ds || !dt) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  return dtype == BB_F64 ? launch_deriv<double>(ctx, t, K, 7, x, dr, ds, dt, (cudaStream_t)stream)
                         : launch_deriv<float>(ctx, t, K, 7, x, dr, ds, dt, (cudaStream_t)stream);
}

extern "C" int bb_lift_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* faces,
                             void* out, void* stream) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (K == 0) return BB_OK;
  if (!faces || !out) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  return dtype == BB_F64 ? launch_lift<double>(ctx, t, K, 4, faces, out, (cudaStream_t)stream)
                         : launch_lift<float>(ctx, t, K, 4, faces, out, (cudaStream_t)stream);
}

extern "C" int bb_face_lift_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x,
                                  void* out, void* stream) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (K == 0) return BB_OK;
  if (!x || !out) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  return dtype == BB_F64 ? launch_lift<double>(ctx, t, K, 1, x, out, (cudaStream_t)stream)
                         : launch_lift<float>(ctx, t, K, 1, x, out, (cudaStream_t)stream);
}

static int tri_op(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* out,
                  void* stream, int elevate) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (!elevate && N < 1) return bb_fail(ctx, BB_ERR_ARG, "reduction needs N >= 1");
  if (K == 0) return BB_OK;
  if (!x || !out) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  const int nout = elevate ? np2(N + 1) : np2(N - 1);
  const int64_t total = K * nout;
  const int grid = grid_for(ctx, (total + 255) / 256, 16);
  if (dtype == BB_F64)
    tri_op_kernel<double><<<grid, 256, 0, (cudaStream_t)stream>>>(N, K, elevate, (const double*)x,
                                                                  (double*)out);
  else
    tri_op_kernel<float><<<grid, 256, 0, (cudaStream_t)stream>>>(N, K, elevate, (const float*)x,
                                                                 (float*)out);
  return bb_check_launch(ctx, "tri_op_kernel");
}

extern "C" int bb_elevation_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x,
                                  void* out, void* stream) {
  return tri_op(ctx, N, K, dtype, x, out, stream, 1);
}

extern "C" int bb_reduction_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x,
                                  void* out, void* stream) {
  return tri_op(ctx, N, K, dtype, x, out, stream, 0);
}

extern "C" int bb_fused_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x,
                              const void* faces, void* dr, void* ds, void* dt, void* lift,
                              void* stream) {
  int rc = check_common(ctx, N, K, dtype);
  if (rc) return rc;
  if (K == 0) return BB_OK;
  if (!x || !faces || !dr || !ds || !dt || !lift) return bb_fail(ctx, BB_ERR_ARG, "null pointer");
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == BB_F32 && N <= 15) {
    // the gradient and lift calls back to back (degree-specialised kernels where they exist)
    // move the same bytes faster than the one-launch table-driven pass
    rc = launch_deriv<float>(ctx, t, K, 7, x, dr, ds, dt, st);
    return rc ? rc : launch_lift<float>(ctx, t, K, 4, faces, lift, st);
  }
  return dtype == BB_F64 ? launch_fused<double>(ctx, t, K, x, faces, dr, ds, dt, lift, st)
                         : launch_fused<float>(ctx, t, K, x, faces, dr, ds, dt, lift, st);
}
