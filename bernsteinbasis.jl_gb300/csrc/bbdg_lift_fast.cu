// Degree-specialised FP32 lift operators (BernsteinLift mul! and face_lift_multiply!).
//
// One thread runs one face's whole lift chain (src/BernsteinLift.jl:139-164) in registers, with
// the degree a compile-time constant so that every multi-index is an immediate:
//   E_0 = L0 x, the 7-point stencil of (N+1)^2/2 R_{N+1} E_{N->N+1} on the face's Nfp inputs
//   E_d = R_{N-d+1} E_{d-1}, in place in registers (ascending order, as the reference)
//   layer d of the face's volume stack = l_d E_d (l_0 = 1)
//
// 4-face lift (BernsteinLift mul!): one warp per block and 8 elements per warp, one lane per
// (element, face) chain. Each chain writes its l_d-scaled stack to shared memory in stack order
// (odd lane stride: conflict-free); the warp then forms every output coefficient as the sum of
// its four stack entries in the reference's face order (t=-1 face first, then faces 1, 2, 3 through
// the permutations of src/BernsteinLift.jl:207-218) and stores it coalesced. No atomics, so the
// result does not depend on scheduling. The next tile's inputs arrive while this tile is worked on:
// in registers (degrees up to 9), by a bulk copy into their own buffer (degrees 10 and 11), or
// from 12 on pulled into L2 a tile ahead and read with coalesced loads into the stack area at the
// start of the tile (no input buffer, so more elements per warp fit: 4 up to N = 13).
//
// Single-face lift (face_lift_multiply!): the t = -1 face's stack is already in volume order, so
// the chain writes the output tile directly.
#include <algorithm>

#include "bbdg_internal.cuh"

namespace {

__host__ __device__ constexpr int lf_tri(int n, int j) { return j * (2 * n + 3 - j) / 2; }
__host__ __device__ constexpr int lf_tet(int n, int k) {
  return ((n + 1) * (n + 2) * (n + 3) - (n + 1 - k) * (n + 2 - k) * (n + 3 - k)) / 6;
}
__host__ __device__ constexpr int lf_ij(int n, int i, int j) { return i + lf_tri(n, j); }
__host__ __device__ constexpr int lf_ijk(int n, int i, int j, int k) {
  return i + lf_tri(n, j) + lf_tet(n, k) - j * k;
}

// One face chain from the Nfp inputs X (registers) to the l_d-scaled stack g (shared memory,
// g[lf_ijk(N, i, j, d)] = F_d(i, j) = l_d E_d(i, j); for the t = -1 face this is the volume
// order). The chain carries F_d itself: l_d / l_{d-1} = -(N-d+1)/(d+1) and R_{N-d+1} divides by
// N-d+1, so F_d = -1/(d+1) [(i+1) F_{d-1}(i+1,j) + (j+1) F_{d-1}(i,j+1) + (N-d+1-i-j) F_{d-1}(i,j)]
// with F_0 = E_0 = L0 x.
template <int N>
__device__ __forceinline__ void lift_chain_stack(const float (&X)[(N + 1) * (N + 2) / 2],
                                                 float* g) {
  constexpr int NFP = (N + 1) * (N + 2) / 2;
  float E[NFP];
#pragma unroll
  for (int j = 0; j <= N; ++j) {
#pragma unroll
    for (int i = 0; i + j <= N; ++i) {
      const int k = N - i - j;
      float v = float((i + 1) * (i + 1) + (j + 1) * (j + 1) + (k + 1) * (k + 1)) * X[lf_ij(N, i, j)];
      if (j > 0) v = fmaf(float((i + 1) * j), X[lf_ij(N, i + 1, j - 1)], v);
      if (k > 0) v = fmaf(float((i + 1) * k), X[lf_ij(N, i + 1, j)], v);
      if (i > 0) v = fmaf(float((j + 1) * i), X[lf_ij(N, i - 1, j + 1)], v);
      if (k > 0) v = fmaf(float((j + 1) * k), X[lf_ij(N, i, j + 1)], v);
      if (i > 0) v = fmaf(float((k + 1) * i), X[lf_ij(N, i - 1, j)], v);
      if (j > 0) v = fmaf(float((k + 1) * j), X[lf_ij(N, i, j - 1)], v);
      E[lf_ij(N, i, j)] = 0.5f * v;
      g[lf_ij(N, i, j)] = E[lf_ij(N, i, j)];
    }
  }
#pragma unroll
  for (int d = 1; d <= N; ++d) {
    const int n = N - d + 1;  // input degree of this reduction
    const float inv = -1.0f / float(d + 1);
#pragma unroll
    for (int j = 0; j < n; ++j) {
#pragma unroll
      for (int i = 0; i + j < n; ++i) {
        // reduction_multiply! (src/BernsteinLift.jl:81-85) times l_d / l_{d-1}, in place,
        // ascending
        const float v = float(i + 1) * inv * E[lf_ij(N, i + 1, j)] +
                        (float(j + 1) * inv * E[lf_ij(N, i, j + 1)] +
                         float(n - i - j) * inv * E[lf_ij(N, i, j)]);
        E[lf_ij(N, i, j)] = v;
        g[lf_ijk(N, i, j, d)] = v;
      }
    }
  }
}

__device__ __forceinline__ uint32_t lf_saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

template <int N>
struct Lift4 {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NFP = (N + 1) * (N + 2) / 2;
  static constexpr int NPS = NP | 1;    // stack stride: odd, conflict-free stack stores
  static constexpr int NFPP = NFP | 1;  // input row stride when staged from registers
  // elements per warp: 8 (32 chains) while the stacks leave room for several warps per SM;
  // 4 (16 chains, half the lanes idle in the chain phase) from N = 11 on and 2 from N = 14
  // on, which keeps several warps per SM for the loads and the gather (measured at N = 11
  // and 12: +16 %, +17 %; at N = 10 -15 %; at N = 13 with the staged inputs 4 beats 2 by 14 %,
  // at N = 14 and 15 2 beats 4 and 8)
  static constexpr int EPW = N >= 14 ? 2 : N >= 11 ? 4 : 8;
  // from N = 12: the next tile's inputs go to L2 (bulk prefetch), this tile's are read with
  // coalesced 16-byte loads and staged through the stack area (N = 12: 0.29 -> 0.31 of the
  // HBM copy rate, N = 13: 0.20 -> 0.235; slower at N = 10, 11 than the bulk-copy buffer)
  static constexpr bool STAGED = N >= 12;
  static constexpr int INW = EPW * 4 * NFP;  // input floats per tile
  // next tile in registers when they fit beside the chain, else a bulk copy
  static constexpr bool REG_PREFETCH = N <= 9;
  static constexpr int NV4 = (INW / 4 + 31) / 32;  // float4 inputs per lane
  // shared memory, bytes: [bulk input buffer][stacks (also the register-staged input)][perm]
  static constexpr int IN_B = (REG_PREFETCH || STAGED) ? 0 : INW * 4;
  static constexpr int G_B = IN_B;
  static constexpr int P_B = G_B + (EPW * 4 * NPS * 4 + 15) / 16 * 16;
  static constexpr int BAR_B = P_B + (NP * 4 + 15) / 16 * 16;
  static constexpr int SMEM = BAR_B + 16;
  static_assert(NFPP <= NPS, "staged inputs fit in the stack area");
  static_assert(REG_PREFETCH ? EPW == 8 : true, "the register path stages 32 chains");
  static_assert(EPW * 4 <= 32, "one chain per lane");
  static_assert(NP < 1024, "stack positions are packed in 10 bits");
  static_assert(INW % 4 == 0 && (INW * 4) % 16 == 0, "tiles are whole 16-byte chunks");
};

template <int N>
__global__ void __launch_bounds__(32) lift4_kernel(int64_t K, const float* __restrict__ x,
                                                   float* __restrict__ out, int* status,
                                                   uint32_t wait_iters) {
  using L = Lift4<N>;
  constexpr int NP = L::NP, NFP = L::NFP, NPS = L::NPS, NFPP = L::NFPP, EPW = L::EPW;
  constexpr int INW = L::INW, NV4 = L::NV4;
  extern __shared__ __align__(16) unsigned char smem[];
  float* sIn = reinterpret_cast<float*>(smem);  // bulk-copy input buffer (degrees > 9)
  float* sG = reinterpret_cast<float*>(smem + L::G_B);
  uint32_t* sP = reinterpret_cast<uint32_t*>(smem + L::P_B);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::BAR_B);
  const int t = threadIdx.x;
  // stack positions of coefficient n on faces f0 (i,k,j), f1 (j,k,l), f2 (j,k,i)
  for (int n = t; n < NP; n += 32) {
    int m = n, k = 0, j = 0;
    while (m >= (N - k + 1) * (N - k + 2) / 2) m -= (N - k + 1) * (N - k + 2) / 2, ++k;
    while (m >= N - k - j + 1) m -= N - k - j + 1, ++j;
    const int i = m, l = N - i - j - k;
    sP[n] = (uint32_t)lf_ijk(N, i, k, j) | ((uint32_t)lf_ijk(N, j, k, l) << 10) |
            ((uint32_t)lf_ijk(N, j, k, i) << 20);
  }
  const int64_t ntile = (K + EPW - 1) / EPW;
  auto tile_ne = [&](int64_t tile) { return (int)(K - tile * EPW < EPW ? K - tile * EPW : EPW); };
  float4 pf[L::REG_PREFETCH ? NV4 : 1];
  auto fetch = [&](int64_t tile) {  // registers path
    const float4* xs = reinterpret_cast<const float4*>(x + tile * EPW * 4 * NFP);
    const int nv = tile_ne(tile) * 4 * NFP / 4;
#pragma unroll
    for (int r = 0; r < NV4; ++r)
      if (t + 32 * r < nv) pf[r] = __ldg(xs + t + 32 * r);
  };
  auto issue = [&](int64_t tile) {  // bulk-copy path, lane 0
    const uint32_t bytes = (uint32_t)(tile_ne(tile) * 4 * NFP * 4);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lf_saddr(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            lf_saddr(sIn)),
        "l"(x + tile * EPW * 4 * NFP), "r"(bytes), "r"(lf_saddr(bar))
        : "memory");
  };
  // bounded wait for the bulk copy with the given phase parity (2^24 polls, about a second,
  // unless the context sets another limit)
  const uint32_t wlim = wait_iters ? wait_iters : (1u << 24);
  auto wait_in = [&](uint32_t parity) {
    for (uint32_t it = 0; it < wlim; ++it) {
      uint32_t ok;
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          " selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(ok)
          : "r"(lf_saddr(bar)), "r"(parity)
          : "memory");
      if (ok) return true;
      if (it > 64) __nanosleep(64);
    }
    return false;
  };
  if constexpr (L::REG_PREFETCH) {
    if (blockIdx.x < ntile) fetch(blockIdx.x);
  } else if constexpr (!L::STAGED) {
    if (t == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(lf_saddr(bar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      if (blockIdx.x < ntile) issue(blockIdx.x);
    }
  }
  __syncwarp();
  uint32_t ph = 0;
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int ne = tile_ne(tile);
    const int64_t next = tile + gridDim.x;
    float X[NFP];
    if constexpr (L::REG_PREFETCH) {
      // stage this tile's inputs (chain c = element * 4 + face in rows of NFPP) and take each
      // lane's row into registers; then the next tile's loads go out
      const int nv = ne * 4 * NFP / 4;
#pragma unroll
      for (int r = 0; r < NV4; ++r) {
        const int v = t + 32 * r;
        if (v < nv) {
          const float qq[4] = {pf[r].x, pf[r].y, pf[r].z, pf[r].w};
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            const int g = 4 * v + w, ch = g / NFP, m = g - ch * NFP;
            sG[ch * NFPP + m] = qq[w];
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < NFP; ++m) X[m] = sG[t * NFPP + m];
      __syncwarp();  // every staged input is in registers before the stacks overwrite them
      if (next < ntile) fetch(next);
    } else if constexpr (L::STAGED) {
      // the tile's inputs, pulled into L2 a tile ago: coalesced 16-byte loads, staged in the
      // stack area (free until the chains write it) in rows of NFPP, then one row per lane
      const float4* xs = reinterpret_cast<const float4*>(x + tile * EPW * 4 * NFP);
      const int nv = ne * NFP;  // float4s of the tile (4 NFP floats per element)
      constexpr int UNR = 8;
      for (int v0 = 0; v0 < nv; v0 += 32 * UNR) {
        float4 buf[UNR];
#pragma unroll
        for (int r = 0; r < UNR; ++r) {
          const int v = v0 + t + 32 * r;
          if (v < nv) buf[r] = __ldg(xs + v);
        }
#pragma unroll
        for (int r = 0; r < UNR; ++r) {
          const int v = v0 + t + 32 * r;
          if (v < nv) {
            const float qq[4] = {buf[r].x, buf[r].y, buf[r].z, buf[r].w};
#pragma unroll
            for (int w = 0; w < 4; ++w) {
              const int g = 4 * v + w, ch = g / NFP, m = g - ch * NFP;
              sG[ch * NFPP + m] = qq[w];
            }
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < NFP; ++m) X[m] = sG[(t < ne * 4 ? t : 0) * NFPP + m];
      __syncwarp();  // every staged input is in registers before the stacks overwrite them
      if (t == 0 && next < ntile) {
        // 16-byte aligned start and size: x is (checked by the caller) and a tile is
        // EPW * 4 * NFP floats, a multiple of 4
        const uint32_t bytes = (uint32_t)(tile_ne(next) * 4 * NFP * 4);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(x + next * EPW * 4 * NFP),
                     "r"(bytes)
                     : "memory");
      }
    } else {
      if (!wait_in(ph)) {
        if (t == 0) {
          atomicOr(status, 2);
          wait_in(ph);  // let the copy in flight land before the block exits (bounded)
        }
        return;
      }
      ph ^= 1u;
#pragma unroll
      for (int m = 0; m < NFP; ++m) X[m] = sIn[(t < EPW * 4 ? t : 0) * NFP + m];
      __syncwarp();
      if (t == 0 && next < ntile) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(next);
      }
    }
    if (t / 4 < ne) lift_chain_stack<N>(X, sG + t * NPS);
    __syncwarp();
    // out(n) = f3 stack(n) + f0 stack(p0) + f1 stack(p1) + f2 stack(p2), coalesced stores
    float* os = out + tile * EPW * NP;
    for (int v = t; v < ne * NP; v += 32) {
      const int e = v / NP, n = v - e * NP;
      const uint32_t p = sP[n];
      const float* G = sG + e * 4 * NPS;
      os[v] = ((G[3 * NPS + n] + G[p & 1023u]) + G[NPS + ((p >> 10) & 1023u)]) +
              G[2 * NPS + (p >> 20)];
    }
    __syncwarp();
  }
  (void)INW;
}

template <int N>
int launch_lift4(bb_ctx* ctx, int64_t K, const void* x, void* out, cudaStream_t st) {
  using L = Lift4<N>;
  auto kern = lift4_kernel<N>;
  int* status = bb_ctx_status_word(ctx);
  if (!status) return bb_fail(ctx, BB_ERR_NOMEM, "status word allocation failed");
  BB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, L::SMEM));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "lift tile does not fit");
  const int64_t ntile = (K + L::EPW - 1) / L::EPW;
  const int grid = (int)std::min<int64_t>(ntile, (int64_t)per_sm * ctx->num_sms);
  kern<<<grid, 32, L::SMEM, st>>>(K, (const float*)x, (float*)out, status, ctx->wait_iters);
  return bb_check_launch(ctx, "lift4_kernel");
}

// Single face (the t = -1 face, k = 0): its stack is the output in volume order.
template <int N>
struct Lift1 {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NFP = (N + 1) * (N + 2) / 2;
  static constexpr int NFPP = NFP | 1;
  static constexpr int NPS = NP | 1;
  static constexpr int EPB = 32;
  static constexpr int SMEM = EPB * (NFPP + NPS) * 4;
};

template <int N>
__global__ void __launch_bounds__(32) lift1_kernel(int64_t K, const float* __restrict__ x,
                                                   float* __restrict__ out) {
  using L = Lift1<N>;
  constexpr int NP = L::NP, NFP = L::NFP, NFPP = L::NFPP, NPS = L::NPS, EPB = L::EPB;
  extern __shared__ __align__(16) float sm1[];
  float* sx = sm1;              // [EPB][NFPP]
  float* so = sm1 + EPB * NFPP;  // [EPB][NPS]
  const int t = threadIdx.x;
  const int64_t ntile = (K + EPB - 1) / EPB;
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int64_t e0 = tile * EPB;
    const int ne = (int)min64(EPB, K - e0);
    __syncwarp();
    for (int g = t; g < ne * NFP; g += 32) {
      const int ch = g / NFP, m = g - ch * NFP;
      sx[ch * NFPP + m] = __ldg(x + e0 * NFP + g);
    }
    __syncwarp();
    if (t < ne) {
      float X[NFP];
#pragma unroll
      for (int m = 0; m < NFP; ++m) X[m] = sx[t * NFPP + m];
      lift_chain_stack<N>(X, so + t * NPS);
    }
    __syncwarp();
    for (int v = t; v < ne * NP; v += 32) {
      const int e = v / NP, n = v - e * NP;
      out[e0 * NP + v] = so[e * NPS + n];
    }
  }
}

template <int N>
int launch_lift1(bb_ctx* ctx, int64_t K, const void* x, void* out, cudaStream_t st) {
  using L = Lift1<N>;
  auto kern = lift1_kernel<N>;
  BB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, L::SMEM));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "lift tile does not fit");
  const int64_t ntile = (K + L::EPB - 1) / L::EPB;
  const int grid = (int)std::min<int64_t>(ntile, (int64_t)per_sm * ctx->num_sms);
  kern<<<grid, 32, L::SMEM, st>>>(K, (const float*)x, (float*)out);
  return bb_check_launch(ctx, "lift1_kernel");
}

}  // namespace

// FP32 lift of K columns with the degree-specialised kernels; nfaces 4 (BernsteinLift, N <= 15)
// or 1 (face_lift_multiply!, N <= 12). Returns -1 when no specialised kernel applies (degree
// above those, or a 4-face input or output that is not 16-byte aligned), and the caller runs
// the generic kernel.
int bb_lift_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int nfaces, const void* x,
                 void* out, cudaStream_t st) {
  if (nfaces == 4 && ((((uintptr_t)x) | ((uintptr_t)out)) & 15) != 0) return -1;
#define BB_LF(n_)                                                                  \
  case n_:                                                                         \
    return nfaces == 4 ? launch_lift4<n_>(ctx, K, x, out, st)                      \
                       : launch_lift1<n_>(ctx, K, x, out, st);
  switch (t->N) {
    // the single-face kernel stops at N = 12 (its 32-element tiles leave too few warps per SM
    // above); the level-parallel kernel runs it there
    BB_LF(1) BB_LF(2) BB_LF(3) BB_LF(4) BB_LF(5) BB_LF(6) BB_LF(7) BB_LF(8) BB_LF(9)
    BB_LF(10) BB_LF(11) BB_LF(12)
    case 13:
      return nfaces == 4 ? launch_lift4<13>(ctx, K, x, out, st) : -1;
    case 14:
      return nfaces == 4 ? launch_lift4<14>(ctx, K, x, out, st) : -1;
    case 15:
      return nfaces == 4 ? launch_lift4<15>(ctx, K, x, out, st) : -1;
    default:
      return -1;
  }
#undef BB_LF
}
