// Degree-specialised FP32 derivative operators (BernsteinDerivativeMatrix_3D_{r,s,t} mul! and
// the fused gradient), N = 1..15.
//
// D_a x(alpha) = 1/2 sum_b alpha_b (x(alpha - e_b + e_a) - x(alpha - e_b + e_3)), b = 0..3,
// with e_3 the fourth barycentric direction: the four terms per row that
// BernsteinDerivativeMatrix_3D.jl:96-216 writes, each difference w_a(alpha - e_b) of the
// factored form taken straight from the inputs. All three axes read 13 points per node
// (alpha and its 12 neighbours alpha - e_b + e_c), one axis 7; the differences are formed
// before they are weighted, as in the table-driven kernel, which keeps FP32 accurate.
//
// Each thread owns fixed nodes for the whole run and keeps their neighbour indices (16-bit)
// and weights in registers, so no table is read per element. A tile of EPW elements arrives
// by cp.async (16-byte pieces, no registers) into one of two shared buffers while the other
// is worked on; outputs are stored coalesced from registers. The block shape per degree
// (deriv_shape) was chosen by measurement: what limits this streaming kernel is the bytes in
// flight per SM (blocks per SM x tile), more than idle threads.
#include <algorithm>

#include "bbdg_internal.cuh"

namespace {

// Block shape: W warps; G element groups of NP threads (G > 1 only when NP is small) or NPT
// nodes per thread (G = 1); EPW elements per tile, a multiple of G, with EPW NP a multiple of 4
// so that every tile starts on a 16-byte boundary.
struct DerivShape {
  int W, G, NPT, EPW;
};
constexpr DerivShape deriv_shape(int N) {
  constexpr DerivShape table[16] = {
      {0, 0, 0, 0},     {8, 64, 1, 768}, {10, 32, 1, 640}, {10, 16, 1, 320},
      {8, 7, 1, 112},   {7, 4, 1, 56},   {8, 3, 1, 78},    {8, 1, 1, 27},
      {16, 3, 1, 48},   {7, 1, 1, 15},   {9, 1, 1, 12},    {12, 1, 1, 18},
      {15, 1, 1, 8},    {6, 1, 3, 11},   {8, 1, 3, 9},     {13, 1, 2, 8}};
  return table[N];
}

template <int N>
struct DerivStencil {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr DerivShape S = deriv_shape(N);
  static constexpr int THREADS = 32 * S.W, G = S.G, NPT = S.NPT, EPW = S.EPW;
  static constexpr int TILE = EPW * NP;  // floats per tile
  static constexpr int NV4 = (TILE / 4 + THREADS - 1) / THREADS;  // 16-byte pieces per thread
  static constexpr int SMEM = 2 * TILE * 4;
  static_assert(TILE % 4 == 0, "tiles are whole float4s");
  static_assert(G * NP <= NPT * THREADS && (G == 1 || NPT == 1) && EPW % G == 0, "block shape");
  static_assert(NP < 65536, "16-bit node indices");
};

// 3D index (degree N) of alpha - e_b + e_c, alpha = (i, j, k, N-i-j-k); alpha itself when
// alpha_b = 0 (that term has weight 0, and x(alpha) - x(alpha) = 0 like the zero entry of w).
__device__ __forceinline__ uint32_t shifted_node(int N, int i, int j, int k, int b, int c) {
  int q[4] = {i, j, k, N - i - j - k};
  if (q[b] == 0) return (uint32_t)ijk3(N, i, j, k);
  q[b] -= 1;
  q[c] += 1;
  return (uint32_t)ijk3(N, q[0], q[1], q[2]);
}

// 16-byte global -> shared copy; bytes < 16 reads that many and zero-fills the rest.
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, int bytes) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(gsrc), "r"(bytes)
               : "memory");
}

template <int N, int MASK>  // MASK: 1, 2, 4 = one of r, s, t; 7 = all three
__global__ void __launch_bounds__(DerivStencil<N>::THREADS)
    deriv_stencil_kernel(int64_t K, const uint32_t* __restrict__ gtab, int o_node3,
                         const float* __restrict__ x, float* __restrict__ o0,
                         float* __restrict__ o1, float* __restrict__ o2) {
  using D = DerivStencil<N>;
  constexpr int NP = D::NP, THREADS = D::THREADS, NPT = D::NPT, EPW = D::EPW, TILE = D::TILE,
                NV4 = D::NV4, G = D::G;
  constexpr int A = MASK == 2 ? 1 : MASK == 4 ? 2 : 0;  // the axis when MASK != 7
  // Neighbour slots. All three axes: alpha - e_b + e_c in slot 3b + (c < b ? c : c - 1),
  // c != b. One axis A: Q_b = alpha - e_b + e_A in slot (b < A ? b : b - 1), b != A, and
  // R_b = alpha - e_b + e_3 in slot 3 + b, b < 3.
  constexpr int NI = MASK == 7 ? 12 : 6;
  extern __shared__ __align__(16) float dsm[];
  const int t = threadIdx.x;
  // element group g works on elements g, g + G, ... of a tile, at nodes n0 + THREADS r
  const int g = G > 1 ? t / NP : 0;
  const int n0 = G > 1 ? t - g * NP : t;
  uint32_t ix[NPT][NI / 2];
  uint32_t wt[NPT];
#pragma unroll
  for (int r = 0; r < NPT; ++r) {
    const int n = n0 + THREADS * r;
    uint32_t s[12];
    wt[r] = 0;
    if (n < NP && g < G) {
      const uint32_t c = gtab[o_node3 + n];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
      wt[r] = (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16) | ((uint32_t)l << 24);
      if (MASK == 7) {
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int cc = 0; cc < 4; ++cc)
            if (cc != b) s[3 * b + (cc < b ? cc : cc - 1)] = shifted_node(N, i, j, k, b, cc);
      } else {
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (b != A) s[b < A ? b : b - 1] = shifted_node(N, i, j, k, b, A);
#pragma unroll
        for (int b = 0; b < 3; ++b) s[3 + b] = shifted_node(N, i, j, k, b, 3);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 12; ++q) s[q] = 0;
    }
#pragma unroll
    for (int q = 0; q < NI / 2; ++q) ix[r][q] = s[2 * q] | (s[2 * q + 1] << 16);
  }
  float* outs[3] = {o0, o1, o2};
  const int64_t ntile = (K + EPW - 1) / EPW;
  auto tile_ne = [&](int64_t tile) { return (int)(K - tile * EPW < EPW ? K - tile * EPW : EPW); };
  auto fetch = [&](int64_t tile, float* sbuf) {
    const float* xs = x + tile * TILE;
    const int nv = tile_ne(tile) * NP;  // floats; the last tile may end inside a float4
#pragma unroll
    for (int r = 0; r < NV4; ++r) {
      const int v = t + THREADS * r;
      if (4 * v < nv) {
        const int left = nv - 4 * v;
        cp_async16(sbuf + 4 * v, xs + 4 * v, left >= 4 ? 16 : 4 * left);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  if (blockIdx.x < ntile) fetch(blockIdx.x, dsm);
  int buf = 0;
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, buf ^= 1) {
    const int ne = tile_ne(tile);
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();  // this tile has landed for every thread; the other buffer is free
    if (tile + gridDim.x < ntile) fetch(tile + gridDim.x, dsm + (buf ^ 1) * TILE);
    const float* sx = dsm + buf * TILE;
    const int64_t base = tile * TILE;
#pragma unroll
    for (int r = 0; r < NPT; ++r) {
      const int n = n0 + THREADS * r;
      if (n >= NP || g >= G) break;
      const uint32_t gw = wt[r];
      const float a0 = float(gw & 0xff), a1 = float((gw >> 8) & 0xff),
                  a2 = float((gw >> 16) & 0xff), a3 = float(gw >> 24);
      auto I = [&](int q) -> int { return (int)((ix[r][q >> 1] >> (16 * (q & 1))) & 0xffff); };
      for (int le = g; le < ne; le += G) {
        const float* xe = sx + le * NP;
        const float xa = xe[n];
        if (MASK == 7) {
          float d[4][3];  // d[b][a] = x(alpha - e_b + e_a) - x(alpha - e_b + e_3)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const float e3 = b == 3 ? xa : xe[I(3 * b + 2)];
#pragma unroll
            for (int a = 0; a < 3; ++a)
              d[b][a] = (a == b ? xa : xe[I(3 * b + (a < b ? a : a - 1))]) - e3;
          }
#pragma unroll
          for (int a = 0; a < 3; ++a)
            outs[a][base + le * NP + n] =
                0.5f * fmaf(a3, d[3][a], fmaf(a2, d[2][a], fmaf(a1, d[1][a], a0 * d[0][a])));
        } else {
          float d[4];
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const float q = b == A ? xa : xe[I(b < A ? b : b - 1)];
            const float rr = b == 3 ? xa : xe[I(3 + b)];
            d[b] = q - rr;
          }
          outs[A][base + le * NP + n] =
              0.5f * fmaf(a3, d[3], fmaf(a2, d[2], fmaf(a1, d[1], a0 * d[0])));
        }
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");  // nothing in flight at exit
}

template <int N, int MASK>
int launch_deriv_stencil_t(bb_ctx* ctx, const DegTables* t, int64_t K, const void* x, void* o0,
                           void* o1, void* o2, cudaStream_t st) {
  using D = DerivStencil<N>;
  auto kern = deriv_stencil_kernel<N, MASK>;
  BB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, D::THREADS, D::SMEM));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "derivative tile does not fit");
  const int64_t ntile = (K + D::EPW - 1) / D::EPW;
  const int grid = (int)std::min<int64_t>(ntile, (int64_t)per_sm * ctx->num_sms);
  kern<<<grid, D::THREADS, D::SMEM, st>>>(K, t->d_words, t->o_node3, (const float*)x,
                                          (float*)o0, (float*)o1, (float*)o2);
  return bb_check_launch(ctx, "deriv_stencil_kernel");
}

template <int N>
int launch_deriv_stencil_n(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x,
                           void* o0, void* o1, void* o2, cudaStream_t st) {
  switch (mask) {
    case 1: return launch_deriv_stencil_t<N, 1>(ctx, t, K, x, o0, o1, o2, st);
    case 2: return launch_deriv_stencil_t<N, 2>(ctx, t, K, x, o0, o1, o2, st);
    case 4: return launch_deriv_stencil_t<N, 4>(ctx, t, K, x, o0, o1, o2, st);
    case 7: return launch_deriv_stencil_t<N, 7>(ctx, t, K, x, o0, o1, o2, st);
    default: return -1;
  }
}

}  // namespace

// FP32 derivative(s) of K columns with the degree-specialised kernel; mask = axes (1, 2, 4 for
// one of r, s, t; 7 for all three). Returns -1 when none applies (degree above 15, another
// mask, or an input that is not 16-byte aligned), and the caller runs the generic kernel.
int bb_deriv_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x, void* o0,
                  void* o1, void* o2, cudaStream_t st) {
  if ((((uintptr_t)x) & 15) != 0 || K < 1) return -1;
#define BB_DS(n_) \
  case n_:        \
    return launch_deriv_stencil_n<n_>(ctx, t, K, mask, x, o0, o1, o2, st);
  switch (t->N) {
    BB_DS(1) BB_DS(2) BB_DS(3) BB_DS(4) BB_DS(5) BB_DS(6) BB_DS(7) BB_DS(8) BB_DS(9) BB_DS(10)
    BB_DS(11) BB_DS(12) BB_DS(13) BB_DS(14) BB_DS(15)
    default:
      return -1;
  }
#undef BB_DS
}
