// BF16 tensor-core GEMM for sm_103a (tcgen05 + TMEM + TMA), FP32 accumulation:
//     C[M x N] = alpha * A[M x K] * B[N x K]^T, then a fused epilogue (bbdg_gemm.cuh).
// A and B are row-major BF16 with K contiguous ("K-major" operands).
//
// Persistent, warp-specialised kernel, one CTA per SM (192 threads):
//   warp 0      TMA producer: 128 x 64 boxes of A and BN x 64 boxes of B, 128-byte swizzle,
//               into a STAGES-deep shared-memory ring (mbarrier full / empty pairs);
//   warp 1      MMA issuer: one thread issues tcgen05.mma (kind::f16, M=128, N=BN, K=16)
//               into one of two TMEM accumulators and releases ring stages and finished
//               accumulators with tcgen05.commit;
//   warps 2-5   epilogue: tcgen05.ld of 32-column chunks (warp w reads TMEM lanes
//               32(w%4)..+31 = tile rows), staged through a per-warp shared tile so that
//               every global store of a warp covers one contiguous row segment (row-major
//               outputs) or one contiguous column segment (the transposed output).
// The two accumulators let the epilogue of tile i overlap the main loop of tile i+1.
// Tiles are visited n-fastest so that CTAs running together share A rows in L2; split-K
// partial tiles (gridless: part of the tile index) add into the FP32 output atomically.
// Every mbarrier wait is bounded (about a second): on time-out the kernel sets the status
// word, stops issuing work, lets its copies and MMAs in flight finish (bounded) and frees
// its TMEM. Used by the learned per-element closure (an MLP trained and run in BF16).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cmath>
#include <mutex>

#include "bbdg_internal.cuh"
#include "bbdg_gemm.cuh"

namespace {

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of a K-major operand tile in the 128-byte swizzle layout:
// start address >> 4 (bits 0-13), leading byte offset 16 B >> 4 (unused for this layout),
// stride byte offset 1024 B >> 4 (8 rows x 128 B), descriptor version 1 (bits 46-47), layout
// SWIZZLE_128B = 2 (bits 61-63). The tile base must be 1024-byte aligned.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t smem_addr) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: `limit` polls (2^24, about a second, by default), false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    if (mbar_test(b, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(saddr(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   saddr(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 32 lanes x 32 bit, 32 consecutive columns per thread (warp w % 4 reads lanes 32(w%4)..+31).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
// d/dx [x Phi(x)] = Phi(x) + x phi(x)
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Epilogue variants fixed at compile time (F != 0); F == 0 reads every option at run time.
enum : int {
  kBias = 1,      // v += bias[c]
  kAct1 = 2,      // Pre = v (if kPreW), v = GELU(v)
  kAct2 = 4,      // v *= GELU'(Pre)
  kPreW = 8,      // store the pre-activation
  kCf = 16,       // Cf = v
  kCfAdd = 32,    // Cf += v atomically (split-K)
  kCb = 64,       // Cb = bf16(v)
  kBgrad = 128,   // bias_grad[c] += sum over rows of v
};
constexpr int kEpiMlpHiddenTrain = kBias | kAct1 | kPreW | kCb;
constexpr int kEpiMlpHidden = kBias | kAct1 | kCb;
constexpr int kEpiBiasF32 = kBias | kCf;
constexpr int kEpiGeluGradBf16 = kAct2 | kCb | kBgrad;
constexpr int kEpiGeluGrad = kAct2 | kBgrad;
constexpr int kEpiSplitK = kCfAdd;
constexpr int kEpiF32 = kCf;
constexpr int kEpiBf16 = kCb;

__device__ __forceinline__ void st_bf16x4(__nv_bfloat16* p, float4 v) {
  __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
  uint2 u;
  u.x = *reinterpret_cast<uint32_t*>(&lo);
  u.y = *reinterpret_cast<uint32_t*>(&hi);
  *reinterpret_cast<uint2*>(p) = u;
}

// One element of the epilogue with compile-time options.
template <int F>
__device__ __forceinline__ float epi_value(float x, float b, const GemmEpilogue& ep, size_t off) {
  if (F & kBias) x += b;
  if (F & kAct1) {
    if (F & kPreW) ep.Pre[off] = x;
    x = gelu(x);
  }
  if (F & kAct2) x *= gelu_grad(ep.Pre[off]);
  return x;
}

// Row pass of a staged 32 x 32 chunk (T, pitch 36 floats) with compile-time options: lane l
// handles columns c0 + 4 (l % 8) .. + 3 of rows 4 i + l / 8, so one warp store writes four
// contiguous 128-byte (FP32) or 64-byte (BF16) row segments. vec: every output row start is
// 16-byte aligned (ldc % 4 == 0 and aligned bases), else the lane falls back to scalars.
template <int F>
__device__ __forceinline__ void epi_rows(const GemmEpilogue& ep, float* T, int r0, int c0,
                                         int rows, int lane, bool vec) {
  const int q = lane >> 3, cg = (lane & 7) * 4;
  const int c = c0 + cg;
  const int ncol = min(4, ep.N - c);  // columns of this lane inside the matrix (may be <= 0)
  float b[4] = {0.f, 0.f, 0.f, 0.f};
  if (F & kBias) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < ncol) b[j] = ep.bias[c + j];
  }
  float g[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int rr = 4 * i + q;
    float4 x4 = *reinterpret_cast<const float4*>(T + rr * 36 + cg);
    if (rr < rows && ncol > 0) {
      const size_t off = (size_t)(r0 + rr) * ep.ldc + c;
      float x[4] = {ep.alpha * x4.x, ep.alpha * x4.y, ep.alpha * x4.z, ep.alpha * x4.w};
      if (vec && ncol == 4) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (F & kBias) x[j] += b[j];
        }
        if (F & kAct2) {
          const float4 p4 = *reinterpret_cast<const float4*>(ep.Pre + off);
          const float pr[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) x[j] *= gelu_grad(pr[j]);
        }
        if (F & kAct1) {
          if (F & kPreW) *reinterpret_cast<float4*>(ep.Pre + off) = make_float4(x[0], x[1], x[2], x[3]);
#pragma unroll
          for (int j = 0; j < 4; ++j) x[j] = gelu(x[j]);
        }
        x4 = make_float4(x[0], x[1], x[2], x[3]);
        if (F & kCf) *reinterpret_cast<float4*>(ep.Cf + off) = x4;
        if (F & kCfAdd) {
#pragma unroll
          for (int j = 0; j < 4; ++j) atomicAdd(ep.Cf + off + j, x[j]);
        }
        if (F & kCb) st_bf16x4(ep.Cb + off, x4);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (j < ncol) {
            x[j] = epi_value<F>(x[j], b[j], ep, off + j);
            if (F & kCf) ep.Cf[off + j] = x[j];
            if (F & kCfAdd) atomicAdd(ep.Cf + off + j, x[j]);
            if (F & kCb) ep.Cb[off + j] = __float2bfloat16_rn(x[j]);
          }
        }
        x4 = make_float4(x[0], x[1], x[2], x[3]);
      }
      if (F & kBgrad) {
        g[0] += x4.x;
        g[1] += x4.y;
        g[2] += x4.z;
        g[3] += x4.w;
      }
      *reinterpret_cast<float4*>(T + rr * 36 + cg) = x4;
    }
  }
  if (F & kBgrad) {
    // lanes l, l+8, l+16, l+24 hold the same columns
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      g[j] += __shfl_xor_sync(0xffffffffu, g[j], 8);
      g[j] += __shfl_xor_sync(0xffffffffu, g[j], 16);
    }
    if (q == 0) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < ncol) atomicAdd(ep.bias_grad + c + j, g[j]);
    }
  }
}

// Row pass with every option read at run time (any alignment, any combination).
__device__ __forceinline__ void epi_rows_generic(const GemmEpilogue& ep, float* T, int r0,
                                                 int c0, int rows, int lane, bool split) {
  const int c = c0 + lane;
  const bool cin = c < ep.N;
  const float b = (cin && ep.bias) ? ep.bias[c] : 0.0f;
  float gsum = 0.0f;
  for (int rr = 0; rr < rows; ++rr) {
    float x = ep.alpha * T[rr * 36 + lane] + b;
    if (cin) {
      const size_t off = (size_t)(r0 + rr) * ep.ldc + c;
      if (ep.act == 1) {
        if (ep.Pre) ep.Pre[off] = x;
        x = gelu(x);
      } else if (ep.act == 2) {
        x *= gelu_grad(ep.Pre[off]);
      }
      if (ep.Cf) {
        if (split) atomicAdd(ep.Cf + off, x);
        else ep.Cf[off] = ep.accumulate ? ep.Cf[off] + x : x;
      }
      if (ep.Cb) ep.Cb[off] = __float2bfloat16_rn(x);
      gsum += x;
    }
    T[rr * 36 + lane] = x;
  }
  if (ep.bias_grad && cin) atomicAdd(ep.bias_grad + c, gsum);
}

template <int BN_>
struct GemmCfg {
  static constexpr int BM = 128, BN = BN_, BK = 64, UMMA_K = 16;
  static constexpr int A_BYTES = BM * BK * 2;            // 16 KiB
  static constexpr int B_BYTES = BN * BK * 2;            // 32 or 16 KiB
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int STAGES = (192 * 1024) / STAGE_BYTES;  // 4 or 6
  static constexpr int TMEM_COLS = 2 * BN;               // two FP32 accumulators
  static constexpr int EPI_WARPS = 4;
  static constexpr int THREADS = 64 + 32 * EPI_WARPS;
  static constexpr int EPI_PITCH = 36;                   // floats; 16-byte rows
  static constexpr int EPI_BYTES = EPI_WARPS * 32 * EPI_PITCH * 4;
  static constexpr int NBAR = 2 * STAGES + 5;
  static constexpr int SMEM = STAGES * STAGE_BYTES + EPI_BYTES + 8 * NBAR + 16 + 1024;
  // instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9 and
  // 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
                                    ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
  static_assert(TMEM_COLS <= 512, "TMEM budget");
};

struct TileSched {
  int m_tiles, n_tiles, splits, kt_per, nkt_all;
  __device__ __forceinline__ void decode(int tile, int& mt, int& nt, int& kt0, int& nkt) const {
    nt = tile % n_tiles;
    const int rest = tile / n_tiles;
    mt = rest % m_tiles;
    const int z = rest / m_tiles;
    kt0 = z * kt_per;
    nkt = min(kt_per, nkt_all - kt0);
  }
  __host__ __device__ __forceinline__ int total() const { return m_tiles * n_tiles * splits; }
};

__device__ __forceinline__ bool flag_set(const volatile int* f) { return *f != 0; }

template <int BN, int F>
__global__ void __launch_bounds__(GemmCfg<BN>::THREADS, 1)
    gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                        const __grid_constant__ CUtensorMap tmB, GemmEpilogue ep, TileSched ts) {
  using C = GemmCfg<BN>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t base = saddr(smem_raw);
  unsigned char* smem = smem_raw + ((1024 - (base & 1023)) & 1023);  // 1024-aligned ring
  float* epi = reinterpret_cast<float*>(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::STAGES * C::STAGE_BYTES + C::EPI_BYTES);
  uint64_t* full = bars;                    // [STAGES] TMA -> MMA
  uint64_t* empty = bars + C::STAGES;       // [STAGES] MMA -> TMA
  uint64_t* tfull = bars + 2 * C::STAGES;   // [2] MMA -> epilogue
  uint64_t* tempty = tfull + 2;             // [2] epilogue -> MMA
  uint64_t* mdone = tempty + 2;             // every MMA of this CTA complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + C::NBAR);
  __shared__ int s_abort, s_issued, s_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    s_abort = 0;
    s_issued = 0;
    s_consumed = 0;
    for (int s = 0; s < C::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], C::EPI_WARPS);
    }
    mbar_init(mdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  volatile int* abort_flag = &s_abort;
  const uint32_t wlim = ep.wait_iters ? ep.wait_iters : (1u << 24);
  const int total = ts.total();

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      int it = 0;
      for (int tile = blockIdx.x; tile < total && !flag_set(abort_flag); tile += gridDim.x) {
        int mt, nt, kt0, nkt;
        ts.decode(tile, mt, nt, kt0, nkt);
        for (int kt = 0; kt < nkt; ++kt, ++it) {
          const int s = it % C::STAGES;
          if (!mbar_wait(&empty[s], ((it / C::STAGES) & 1) ^ 1, wlim)) {
            atomicOr(ep.status, 2);
            *abort_flag = 1;
            break;
          }
          unsigned char* st = smem + s * C::STAGE_BYTES;
          mbar_expect_tx(&full[s], C::STAGE_BYTES);
          // test-only fault mode: the stage's barrier is armed but its copies are left out,
          // so the MMA issuer's bounded wait on it runs out
          if (ep.fault == 1 && it == 1) continue;
          tma_load_2d(st, &tmA, (kt0 + kt) * C::BK, mt * C::BM, &full[s]);
          tma_load_2d(st + C::A_BYTES, &tmB, (kt0 + kt) * C::BK, nt * BN, &full[s]);
        }
      }
      s_issued = it;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      int it = 0, local = 0;
      for (int tile = blockIdx.x; tile < total && !flag_set(abort_flag);
           tile += gridDim.x, ++local) {
        int mt, nt, kt0, nkt;
        ts.decode(tile, mt, nt, kt0, nkt);
        const int a = local & 1;
        if (!mbar_wait(&tempty[a], ((local >> 1) & 1) ^ 1, wlim)) {
          atomicOr(ep.status, 2);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(a * BN);
        bool ok = true;
        for (int kt = 0; kt < nkt; ++kt, ++it) {
          const int s = it % C::STAGES;
          if (!mbar_wait(&full[s], (it / C::STAGES) & 1, wlim)) {
            atomicOr(ep.status, 2);
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = saddr(smem + s * C::STAGE_BYTES);
          const uint32_t b0 = a0 + C::A_BYTES;
#pragma unroll
          for (int k = 0; k < C::BK / C::UMMA_K; ++k)  // 16 BF16 = 32 bytes along K per MMA
            umma_bf16(d, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), C::IDESC,
                      (kt | k) != 0);
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[a]);
      }
      s_consumed = it;
      umma_commit(mdone);
    }
  } else {
    // ---- epilogue warps ----
    const int g = warp & 3;  // TMEM lane quarter this warp may access
    // 16-byte vector stores need 16-byte aligned row starts for every row-major output
    const bool vec = (ep.ldc % 4 == 0) && ((((uintptr_t)ep.Cf | (uintptr_t)ep.Pre) & 15) == 0) &&
                     ((((uintptr_t)ep.Cb) & 7) == 0);
    float* T = epi + (warp - 2) * 32 * C::EPI_PITCH;
    int local = 0;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x, ++local) {
      int mt, nt, kt0, nkt;
      ts.decode(tile, mt, nt, kt0, nkt);
      const int a = local & 1;
      int ok = 0;
      if (lane == 0) {
        ok = !flag_set(abort_flag) && mbar_wait(&tfull[a], (local >> 1) & 1, wlim);
        if (!ok && !flag_set(abort_flag)) {
          atomicOr(ep.status, 2);
          *abort_flag = 1;
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      tc_fence_after();
      const int r0 = mt * C::BM + g * 32;
      const int n0 = nt * BN;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(a * BN + c0), v);
        if (c0 + 32 == BN) {
          // accumulator fully read: hand it back to the MMA warp
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[a]);
        }
        if (n0 + c0 >= ep.N) continue;
        // stage the chunk: lane = row, 8 x 16-byte stores (conflict-free with pitch 36)
#pragma unroll
        for (int j = 0; j < 32; j += 4)
          *reinterpret_cast<float4*>(T + lane * C::EPI_PITCH + j) =
              make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        __syncwarp();
        const int rows = min(32, ep.M - r0);
        if (F == 0) epi_rows_generic(ep, T, r0, n0 + c0, rows, lane, ep.kt_per < ts.nkt_all);
        else epi_rows<F>(ep, T, r0, n0 + c0, rows, lane, vec);
        if (ep.CbT) {
          // column pass: lane owns row r0 + lane; each store covers one column segment
          __syncwarp();
          if (lane < rows) {
            const int cols = min(32, ep.N - (n0 + c0));
            __nv_bfloat16* o = ep.CbT + (size_t)(n0 + c0) * ep.ldt + r0 + lane;
#pragma unroll 8
            for (int j = 0; j < cols; ++j)
              o[(size_t)j * ep.ldt] = __float2bfloat16_rn(T[lane * C::EPI_PITCH + j]);
          }
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // MMAs still in flight (normal exit: none) must finish before TMEM is freed
    if (!mbar_wait(mdone, 0, wlim)) atomicOr(ep.status, 2);
    if (flag_set(abort_flag)) {
      // copies issued but never consumed land before the CTA exits
      for (int it = s_consumed; it < s_issued; ++it)
        mbar_wait(&full[it % C::STAGES], (it / C::STAGES) & 1, wlim);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(C::TMEM_COLS)
                 : "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder(bb_ctx* ctx) {
  if (g_encode) return BB_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return bb_fail(ctx, BB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return BB_OK;
}

// Tensor map of a row-major [rows x K] BF16 matrix, boxes of `box_rows` x 64, 128-byte swizzle.
int make_map(bb_ctx* ctx, CUtensorMap* tm, const void* ptr, int64_t rows, int K, int box_rows) {
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return bb_fail(ctx, BB_ERR_ARG, "tensor map encode failed (%d)", (int)r);
  return BB_OK;
}

template <int BN, int F>
int launch_bnf(bb_ctx* ctx, const CUtensorMap& ta, const CUtensorMap& tb, GemmEpilogue ep,
               TileSched ts, cudaStream_t st) {
  using C = GemmCfg<BN>;
  static std::mutex attr_mu;
  static uint64_t attr_done = 0;  // one bit per device
  {
    std::lock_guard<std::mutex> lock(attr_mu);
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (!(attr_done & bit)) {
      BB_CUDA(ctx, cudaFuncSetAttribute(gemm_bf16_tn_kernel<BN, F>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
      attr_done |= bit;
    }
  }
  const int grid = std::min(ts.total(), ctx->num_sms);
  gemm_bf16_tn_kernel<BN, F><<<grid, C::THREADS, C::SMEM, st>>>(ta, tb, ep, ts);
  return bb_check_launch(ctx, "gemm_bf16_tn_kernel");
}

// The compile-time epilogue matching the requested outputs, 0 (run-time options) if none.
int epilogue_variant(const GemmEpilogue& ep, bool split) {
  int f = 0;
  if (ep.bias) f |= kBias;
  if (ep.act == 1) f |= kAct1 | (ep.Pre ? kPreW : 0);
  if (ep.act == 2) f |= kAct2;
  if (ep.Cf) f |= split ? kCfAdd : (ep.accumulate ? 0 : kCf);
  if (ep.Cf && ep.accumulate && !split) return 0;
  if (ep.Cb) f |= kCb;
  if (ep.bias_grad) f |= kBgrad;
  switch (f) {
    case kEpiMlpHiddenTrain: case kEpiMlpHidden: case kEpiBiasF32: case kEpiGeluGradBf16:
    case kEpiGeluGrad: case kEpiSplitK: case kEpiF32: case kEpiBf16:
      return f;
    default:
      return 0;
  }
}

template <int BN>
int launch_bn(bb_ctx* ctx, const CUtensorMap& ta, const void* B, int N, int K, GemmEpilogue ep,
              TileSched ts, cudaStream_t st) {
  CUtensorMap tb;
  int rc = make_map(ctx, &tb, B, N, K, BN);
  if (rc) return rc;
  switch (epilogue_variant(ep, ts.splits > 1)) {
    case kEpiMlpHiddenTrain: return launch_bnf<BN, kEpiMlpHiddenTrain>(ctx, ta, tb, ep, ts, st);
    case kEpiMlpHidden: return launch_bnf<BN, kEpiMlpHidden>(ctx, ta, tb, ep, ts, st);
    case kEpiBiasF32: return launch_bnf<BN, kEpiBiasF32>(ctx, ta, tb, ep, ts, st);
    case kEpiGeluGradBf16: return launch_bnf<BN, kEpiGeluGradBf16>(ctx, ta, tb, ep, ts, st);
    case kEpiGeluGrad: return launch_bnf<BN, kEpiGeluGrad>(ctx, ta, tb, ep, ts, st);
    case kEpiSplitK: return launch_bnf<BN, kEpiSplitK>(ctx, ta, tb, ep, ts, st);
    case kEpiF32: return launch_bnf<BN, kEpiF32>(ctx, ta, tb, ep, ts, st);
    case kEpiBf16: return launch_bnf<BN, kEpiBf16>(ctx, ta, tb, ep, ts, st);
    default: return launch_bnf<BN, 0>(ctx, ta, tb, ep, ts, st);
  }
}

}  // namespace

int bb_gemm_launch(bb_ctx* ctx, int64_t M, int N, int K, const void* A, const void* B,
                   GemmEpilogue ep, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1) return bb_fail(ctx, BB_ERR_ARG, "GEMM sizes must be positive");
  if (K % 8 != 0) return bb_fail(ctx, BB_ERR_ARG, "GEMM K must be a multiple of 8 (16-byte rows)");
  if (((uintptr_t)A | (uintptr_t)B) & 15)
    return bb_fail(ctx, BB_ERR_ARG, "GEMM operands must be 16-byte aligned");
  if (M > ((int64_t)1 << 30) / 2) return bb_fail(ctx, BB_ERR_ARG, "GEMM M too large");
  ep.wait_iters = ctx->wait_iters;
  ep.fault = ctx->test_fault;
  int rc = get_encoder(ctx);
  if (rc) return rc;
  CUtensorMap ta;
  rc = make_map(ctx, &ta, A, M, K, 128);
  if (rc) return rc;
  ep.M = (int)M;
  ep.N = N;
  ep.K = K;
  const int nkt = (K + 63) / 64;
  int splits = 1;
  if (ep.kt_per > 0 && ep.kt_per < nkt) {
    // split-K: partial products are added into Cf (which the caller has zeroed)
    if (!ep.Cf || ep.Cb || ep.CbT || ep.Pre || ep.bias || ep.bias_grad || ep.act || ep.accumulate)
      return bb_fail(ctx, BB_ERR_ARG, "split-K GEMM writes only an FP32 sum");
    splits = (nkt + ep.kt_per - 1) / ep.kt_per;
  } else {
    ep.kt_per = nkt;
  }
  // BN = 256 unless 128-column tiles waste less of the last tile
  const int pad256 = (N + 255) / 256 * 256 - N, pad128 = (N + 127) / 128 * 128 - N;
  const int bn = pad256 <= pad128 ? 256 : 128;
  TileSched ts;
  ts.m_tiles = (int)((M + 127) / 128);
  ts.n_tiles = (N + bn - 1) / bn;
  ts.splits = splits;
  ts.kt_per = ep.kt_per;
  ts.nkt_all = nkt;
  if ((int64_t)ts.m_tiles * ts.n_tiles * splits > INT32_MAX / 2)
    return bb_fail(ctx, BB_ERR_ARG, "GEMM too large");
  return bn == 256 ? launch_bn<256>(ctx, ta, B, N, K, ep, ts, st)
                   : launch_bn<128>(ctx, ta, B, N, K, ep, ts, st);
}

int* bb_ctx_status_word(bb_ctx* ctx) {
  if (!ctx->d_status) {
    if (cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) return nullptr;
  }
  return ctx->d_status;
}

extern "C" int bb_gemm_bf16(bb_ctx* ctx, int64_t M, int N, int K, const void* A, const void* B,
                            float alpha, const float* bias, int act, float* pre, float* C_f32,
                            void* C_bf16, void* CT_bf16, float* bias_grad, int ldc, int ldt,
                            int kt_per, void* stream) {
  if (!ctx) return BB_ERR_ARG;
  if (!A || !B || (!C_f32 && !C_bf16 && !CT_bf16 && !bias_grad))
    return bb_fail(ctx, BB_ERR_ARG, "bb_gemm_bf16: null operand or no output");
  if (act < 0 || act > 2) return bb_fail(ctx, BB_ERR_ARG, "act must be 0, 1 (GELU) or 2 (GELU')");
  if (act == 2 && !pre) return bb_fail(ctx, BB_ERR_ARG, "act 2 needs the pre-activation");
  if ((C_f32 || C_bf16 || pre) && ldc < N) return bb_fail(ctx, BB_ERR_ARG, "ldc must be >= N");
  if (CT_bf16 && ldt < M) return bb_fail(ctx, BB_ERR_ARG, "ldt must be >= M");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  int* status = bb_ctx_status_word(ctx);
  if (!status) return bb_fail(ctx, BB_ERR_NOMEM, "status word allocation failed");
  GemmEpilogue ep{};
  ep.alpha = alpha;
  ep.bias = bias;
  ep.act = act;
  ep.Pre = pre;
  ep.Cf = C_f32;
  ep.accumulate = 0;
  ep.Cb = (__nv_bfloat16*)C_bf16;
  ep.CbT = (__nv_bfloat16*)CT_bf16;
  ep.bias_grad = bias_grad;
  ep.ldc = ldc;
  ep.ldt = ldt;
  ep.status = status;
  if (kt_per < 0) return bb_fail(ctx, BB_ERR_ARG, "kt_per must be >= 0");
  ep.kt_per = kt_per;
  return bb_gemm_launch(ctx, M, N, K, A, B, ep, (cudaStream_t)stream);
}

extern "C" int bb_device_status(bb_ctx* ctx, void* stream, int* out) {
  if (!ctx || !out) return BB_ERR_ARG;
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  *out = 0;
  if (!ctx->d_status) return BB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  BB_CUDA(ctx, cudaMemcpyAsync(out, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  BB_CUDA(ctx, cudaStreamSynchronize(st));
  if (*out) BB_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), st));
  return BB_OK;
}
