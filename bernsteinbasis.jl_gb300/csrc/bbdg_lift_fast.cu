// Degree-specialised FP32 lift operators (BernsteinLift mul! and face_lift_multiply!).
//
// One thread runs one face's whole lift chain (src/BernsteinLift.jl:139-164) with the degree
// a compile-time constant, so every multi-index is an immediate:
//   E_0 = L0 x, the 7-point stencil of (N+1)^2/2 R_{N+1} E_{N->N+1} on the face's Nfp inputs
//   E_d = R_{N-d+1} E_{d-1}, in place in registers (ascending order, as the reference)
//   layer d of the face's volume stack = l_d E_d (l_0 = 1)
// and adds each layer into the element's output tile in shared memory through the face's
// permutation (src/BernsteinLift.jl:207-218). The 4-face lift sums four chains per element
// (shared-memory atomics; the four chains of an element run in one warp); the single-face
// lift writes its stack directly. Input and output tiles move between HBM and shared memory
// with coalesced 16-byte accesses.
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

// Volume index of face f's node (i, j) at distance d (faces s=-1, r+s+t=-1, r=-1, t=-1).
template <int N>
__device__ __forceinline__ int lf_fvol(int f, int i, int j, int d) {
  const int v0 = lf_ijk(N, i, d, j), v1 = lf_ijk(N, N - i - j - d, i, j);
  const int v2 = lf_ijk(N, d, i, j), v3 = lf_ijk(N, i, j, d);
  return f == 0 ? v0 : (f == 1 ? v1 : (f == 2 ? v2 : v3));
}

template <int N, int NFACES>
struct LiftFast {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NFP = (N + 1) * (N + 2) / 2;
  static constexpr int NFPP = NFP | 1;          // odd chain stride: conflict-free reads
  static constexpr int INC = NFACES * NFP;      // input floats per element
  static constexpr int PER_ELEM = (NFACES * NFPP + NP) * 4;
  static constexpr int EPB_MAX = 128 / NFACES;
  static constexpr int EPB_FIT = (56 * 1024) / PER_ELEM;
  static constexpr int EPB = EPB_FIT >= EPB_MAX ? EPB_MAX
                             : EPB_FIT >= 16    ? 16
                             : EPB_FIT >= 8     ? 8
                             : EPB_FIT >= 4     ? 4
                                                : 2;
  static constexpr int THREADS = EPB * NFACES < 32 ? 32 : EPB * NFACES;
  static constexpr int SMEM = EPB * PER_ELEM;
};

template <int N, int NFACES>
__global__ void __launch_bounds__(LiftFast<N, NFACES>::THREADS)
    lift_fast_kernel(int64_t K, const float* __restrict__ x, const float* __restrict__ ljg,
                     float* __restrict__ out) {
  using L = LiftFast<N, NFACES>;
  constexpr int NP = L::NP, NFP = L::NFP, NFPP = L::NFPP, INC = L::INC, EPB = L::EPB;
  extern __shared__ __align__(16) float sm[];
  float* sx = sm;                        // [EPB * NFACES][NFPP] chain inputs
  float* so = sm + EPB * NFACES * NFPP;  // [EPB][NP] output tile
  float lw[N + 1];
  lw[0] = 1.0f;
#pragma unroll
  for (int d = 1; d <= N; ++d) lw[d] = __ldg(ljg + d);
  const int t = threadIdx.x;
  const int le = t / NFACES, fi = t - (t / NFACES) * NFACES;
  const int f = NFACES == 4 ? fi : 3;  // the single-face lift is the t = -1 face
  const int64_t nblk = (K + EPB - 1) / EPB;
  const bool xvec = (((uintptr_t)x) & 15) == 0 && (INC % 4) == 0;
  const bool ovec = (((uintptr_t)out) & 15) == 0 && (NP % 4) == 0;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t e0 = blk * EPB;
    const int ne = (int)min64(EPB, K - e0);
    __syncthreads();
    // input tile (contiguous in HBM) -> chain rows of stride NFPP
    const float* xs = x + e0 * INC;
    if (xvec) {
      for (int v = t; v < ne * INC / 4; v += blockDim.x) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(xs) + v);
        const float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          const int g = 4 * v + w, ch = g / NFP, m = g - ch * NFP;
          sx[ch * NFPP + m] = qq[w];
        }
      }
    } else {
      for (int g = t; g < ne * INC; g += blockDim.x) {
        const int ch = g / NFP, m = g - ch * NFP;
        sx[ch * NFPP + m] = __ldg(xs + g);
      }
    }
    if (NFACES == 4)
      for (int v = t; v < ne * NP; v += blockDim.x) so[v] = 0.0f;
    __syncthreads();
    if (le < ne) {
      const float* X = sx + t * NFPP;
      float* o = so + le * NP;
      float E[NFP];
#pragma unroll
      for (int j = 0; j <= N; ++j) {
#pragma unroll
        for (int i = 0; i + j <= N; ++i) {
          const int k = N - i - j;
          float v = float((i + 1) * (i + 1) + (j + 1) * (j + 1) + (k + 1) * (k + 1)) *
                    X[lf_ij(N, i, j)];
          if (j > 0) v = fmaf(float((i + 1) * j), X[lf_ij(N, i + 1, j - 1)], v);
          if (k > 0) v = fmaf(float((i + 1) * k), X[lf_ij(N, i + 1, j)], v);
          if (i > 0) v = fmaf(float((j + 1) * i), X[lf_ij(N, i - 1, j + 1)], v);
          if (k > 0) v = fmaf(float((j + 1) * k), X[lf_ij(N, i, j + 1)], v);
          if (i > 0) v = fmaf(float((k + 1) * i), X[lf_ij(N, i - 1, j)], v);
          if (j > 0) v = fmaf(float((k + 1) * j), X[lf_ij(N, i, j - 1)], v);
          E[lf_ij(N, i, j)] = 0.5f * v;
          if (NFACES == 4) atomicAdd(o + lf_fvol<N>(f, i, j, 0), E[lf_ij(N, i, j)]);
          else o[lf_fvol<N>(3, i, j, 0)] = E[lf_ij(N, i, j)];
        }
      }
#pragma unroll
      for (int d = 1; d <= N; ++d) {
        const int n = N - d + 1;  // input degree of this reduction
        const float inv = 1.0f / float(n);
#pragma unroll
        for (int j = 0; j < n; ++j) {
#pragma unroll
          for (int i = 0; i + j < n; ++i) {
            // reduction_multiply! (src/BernsteinLift.jl:81-85), in place, ascending
            const float v = float(i + 1) * inv * E[lf_ij(N, i + 1, j)] +
                            (float(j + 1) * inv * E[lf_ij(N, i, j + 1)] +
                             float(n - i - j) * inv * E[lf_ij(N, i, j)]);
            E[lf_ij(N, i, j)] = v;
            if (NFACES == 4) atomicAdd(o + lf_fvol<N>(f, i, j, d), lw[d] * v);
            else o[lf_fvol<N>(3, i, j, d)] = lw[d] * v;
          }
        }
      }
    }
    __syncthreads();
    float* os = out + e0 * NP;
    if (ovec) {
      for (int v = t; v < ne * NP / 4; v += blockDim.x)
        reinterpret_cast<float4*>(os)[v] = reinterpret_cast<const float4*>(so)[v];
    } else {
      for (int v = t; v < ne * NP; v += blockDim.x) os[v] = so[v];
    }
  }
}

template <int N, int NFACES>
int launch_lift_fast_t(bb_ctx* ctx, const float* lj, int64_t K, const void* x, void* out,
                       cudaStream_t st) {
  using L = LiftFast<N, NFACES>;
  auto kern = lift_fast_kernel<N, NFACES>;
  BB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L::THREADS, L::SMEM));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "lift tile does not fit");
  const int64_t nblk = (K + L::EPB - 1) / L::EPB;
  const int grid = (int)std::min<int64_t>(nblk, (int64_t)per_sm * ctx->num_sms * 4);
  kern<<<grid, L::THREADS, L::SMEM, st>>>(K, (const float*)x, lj, (float*)out);
  return bb_check_launch(ctx, "lift_fast_kernel");
}

}  // namespace

// FP32 lift of K columns with the degree-specialised kernel; nfaces 4 (BernsteinLift) or 1
// (face_lift_multiply!). Returns -1 when no specialised kernel exists for N.
int bb_lift_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int nfaces, const void* x,
                 void* out, cudaStream_t st) {
  const float* lj = t->d_ljf;
#define BB_LF(n_)                                                                  \
  case n_:                                                                         \
    return nfaces == 4 ? launch_lift_fast_t<n_, 4>(ctx, lj, K, x, out, st)         \
                       : launch_lift_fast_t<n_, 1>(ctx, lj, K, x, out, st);
  switch (t->N) {
    // above N = 12 the register chains and per-element tiles leave too few warps per SM
    // and the level-parallel kernel is as fast (measured at N = 13..15)
    BB_LF(1) BB_LF(2) BB_LF(3) BB_LF(4) BB_LF(5) BB_LF(6) BB_LF(7) BB_LF(8) BB_LF(9)
    BB_LF(10) BB_LF(11) BB_LF(12)
    default:
      return -1;
  }
#undef BB_LF
}
