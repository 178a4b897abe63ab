// BF16 tensor-core GEMM for sm_103a (tcgen05 + TMEM + TMA), FP32 accumulation:
//     C[M x N] = alpha * A[M x K] * B[N x K]^T (+ bias[N]) (optionally GELU)
// A and B are row-major BF16 with K contiguous ("K-major" operands). One CTA computes one
// 128 x 128 tile: TMA loads 128 x 64 boxes of A and B with 128-byte swizzle into a 4-stage
// shared-memory ring (mbarrier full/empty pairs, every wait bounded); one thread issues
// tcgen05.mma (kind::f16, M=128, N=128, K=16) into a TMEM accumulator and releases each
// stage with tcgen05.commit; after the last K block the four warps read the accumulator with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile rows) and apply the epilogue.
// Used by the learned per-element closure (an MLP trained and evaluated in BF16).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cmath>
#include <mutex>

#include "bbdg_internal.cuh"
#include "bbdg_gemm.cuh"

namespace {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 4, UMMA_K = 16;
constexpr int A_BYTES = BM * BK * 2;  // 16 KiB per stage
constexpr int B_BYTES = BN * BK * 2;  // 16 KiB per stage
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int TMEM_COLS = BN;         // 128 FP32 accumulator columns
constexpr int GEMM_THREADS = 128;
constexpr int GEMM_SMEM = STAGES * STAGE_BYTES + 1024 /*alignment slack*/ + 256 /*barriers*/;

// tcgen05 instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

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
// Bounded wait (about a second), false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 24); ++it) {
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
// 32 lanes x 32 bit, 16 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
// d/dx [x Phi(x)] = Phi(x) + x phi(x)
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

constexpr int EPI_PITCH = BN + 1;  // staged FP32 tile pitch (conflict-free rows and columns)
static_assert(BM * EPI_PITCH * 4 <= STAGES * STAGE_BYTES, "epilogue tile must fit the ring");

__global__ void __launch_bounds__(GEMM_THREADS) gemm_bf16_tn_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
    GemmEpilogue ep) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // 1024-byte aligned stage ring (required by the 128-byte swizzle atoms)
  const uint32_t base = saddr(smem_raw);
  unsigned char* smem = smem_raw + ((1024 - (base & 1023)) & 1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
  __shared__ int s_fail, s_issued, s_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  // K blocks [kt0, kt0 + nkt) of this CTA (split-K along gridDim.z)
  const int nkt_all = (ep.K + BK - 1) / BK;
  const int kt0 = blockIdx.z * ep.kt_per;
  const int nkt = min(ep.kt_per, nkt_all - kt0);

  if (threadIdx.x == 0) {
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    int kt = 0;
    for (; kt < nkt; ++kt) {
      const int s = kt % STAGES;
      const uint32_t ph = (kt / STAGES) & 1;
      if (!mbar_wait(&empty[s], ph ^ 1)) {
        atomicOr(ep.status, 2);
        s_fail = 1;
        break;
      }
      unsigned char* st = smem + s * STAGE_BYTES;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      tma_load_2d(st, &tmA, (kt0 + kt) * BK, m0, &full[s]);
      tma_load_2d(st + A_BYTES, &tmB, (kt0 + kt) * BK, n0, &full[s]);
    }
    s_issued = kt;
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    int kt = 0;
    for (; kt < nkt; ++kt) {
      const int s = kt % STAGES;
      const uint32_t ph = (kt / STAGES) & 1;
      if (!mbar_wait(&full[s], ph)) {
        atomicOr(ep.status, 2);
        s_fail = 1;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = saddr(smem + s * STAGE_BYTES);
      const uint32_t b0 = a0 + A_BYTES;
#pragma unroll
      for (int k = 0; k < BK / UMMA_K; ++k) {
        // advance 16 BF16 = 32 bytes along K inside the 128-byte swizzle row
        umma_bf16(tmem, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), kIdesc,
                  (kt | k) != 0);
      }
      umma_commit(&empty[s]);  // frees the stage when these MMAs have read it
    }
    s_consumed = kt;
    umma_commit(accum);        // accumulator complete (tracks every MMA issued above)
  }
  __syncthreads();
  // one thread observes the accumulator barrier; the block learns the outcome uniformly
  // (the TMEM loads below are warp-collective)
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    s_ok = mbar_wait(accum, 0) ? 1 : 0;
    if (!s_ok) atomicOr(ep.status, 2);
  }
  __syncthreads();
  tc_fence_after();
  const bool ok = s_ok != 0;
  if (s_fail) {
    // a wait ran out: let the loads still in flight land before the CTA exits
    if (threadIdx.x == 0)
      for (int kt = s_consumed; kt < s_issued; ++kt) mbar_wait(&full[kt % STAGES], (kt / STAGES) & 1);
  } else if (ok && nkt > 0) {
    // 1) TMEM -> shared FP32 tile (warp w holds TMEM lanes = tile rows 32w..32w+31)
    float* S = reinterpret_cast<float*>(smem);
    const int r = warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) S[r * EPI_PITCH + c0 + j] = __uint_as_float(v[j]);
    }
    __syncthreads();
    // 2) row pass: thread t owns column t, coalesced row-major reads and writes
    const int c = n0 + threadIdx.x;
    const int rows = min(BM, ep.M - m0);
    if (c < ep.N) {
      const float b = ep.bias ? ep.bias[c] : 0.0f;
      float gsum = 0.0f;
      for (int rr = 0; rr < rows; ++rr) {
        const size_t off = (size_t)(m0 + rr) * ep.ldc + c;
        float v = fmaf(ep.alpha, S[rr * EPI_PITCH + threadIdx.x], b);
        if (ep.act == 1) {
          if (ep.Pre) ep.Pre[off] = v;
          v = gelu(v);
        } else if (ep.act == 2) {
          v *= gelu_grad(ep.Pre[off]);
        }
        if (ep.Cf) {
          if (gridDim.z > 1) atomicAdd(ep.Cf + off, v);
          else ep.Cf[off] = ep.accumulate ? ep.Cf[off] + v : v;
        }
        if (ep.Cb) ep.Cb[off] = __float2bfloat16_rn(v);
        gsum += v;
        S[rr * EPI_PITCH + threadIdx.x] = v;
      }
      if (ep.bias_grad) atomicAdd(ep.bias_grad + c, gsum);
    }
    // 3) column pass for the transposed BF16 output: thread t owns row t
    if (ep.CbT) {
      __syncthreads();
      if (threadIdx.x < rows) {
        const int cols = min(BN, ep.N - n0);
        __nv_bfloat16* o = ep.CbT + (size_t)n0 * ep.ldt + m0 + threadIdx.x;
        for (int cc = 0; cc < cols; ++cc)
          o[(size_t)cc * ep.ldt] = __float2bfloat16_rn(S[threadIdx.x * EPI_PITCH + cc]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
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
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return bb_fail(ctx, BB_ERR_ARG, "tensor map encode failed (%d)", (int)r);
  return BB_OK;
}

}  // namespace

int bb_gemm_launch(bb_ctx* ctx, int64_t M, int N, int K, const void* A, const void* B,
                   GemmEpilogue ep, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1) return bb_fail(ctx, BB_ERR_ARG, "GEMM sizes must be positive");
  if (K % 8 != 0) return bb_fail(ctx, BB_ERR_ARG, "GEMM K must be a multiple of 8 (16-byte rows)");
  if (((uintptr_t)A | (uintptr_t)B) & 15) return bb_fail(ctx, BB_ERR_ARG, "GEMM operands must be 16-byte aligned");
  if (M > (int64_t)65535 * BM) return bb_fail(ctx, BB_ERR_ARG, "GEMM M too large");
  int rc = get_encoder(ctx);
  if (rc) return rc;
  CUtensorMap ta, tb;
  rc = make_map(ctx, &ta, A, M, K, BM);
  if (rc) return rc;
  rc = make_map(ctx, &tb, B, N, K, BN);
  if (rc) return rc;
  ep.M = (int)M;
  ep.N = N;
  ep.K = K;
  const int nkt = (K + BK - 1) / BK;
  int splits = 1;
  if (ep.kt_per > 0 && ep.kt_per < nkt) {
    // split-K: partial products are added into Cf (which the caller has zeroed)
    if (!ep.Cf || ep.Cb || ep.CbT || ep.Pre || ep.bias || ep.bias_grad || ep.act || ep.accumulate)
      return bb_fail(ctx, BB_ERR_ARG, "split-K GEMM writes only an FP32 sum");
    splits = (nkt + ep.kt_per - 1) / ep.kt_per;
  } else {
    ep.kt_per = nkt;
  }
  static std::mutex attr_mu;
  static uint64_t attr_done = 0;  // one bit per device
  {
    std::lock_guard<std::mutex> lock(attr_mu);
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (!(attr_done & bit)) {
      BB_CUDA(ctx, cudaFuncSetAttribute(gemm_bf16_tn_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
      attr_done |= bit;
    }
  }
  dim3 grid((N + BN - 1) / BN, (unsigned)((M + BM - 1) / BM), splits);
  gemm_bf16_tn_kernel<<<grid, GEMM_THREADS, GEMM_SMEM, st>>>(ta, tb, ep);
  return bb_check_launch(ctx, "gemm_bf16_tn_kernel");
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
                            void* stream) {
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
