// Degree-specialised FP32 derivative operators (BernsteinDerivativeMatrix_3D_{r,s,t} mul! and
// the fused gradient), N = 1..11 (at N = 12 the table-driven kernel's larger blocks keep more
// warps per SM and run faster).
//
// Same factored form as the table-driven kernel: D_a x(alpha) = 1/2 sum_b alpha_b w_a(alpha-e_b)
// with w_a(beta) = x(beta + e_a) - x(beta + e_3) at degree N-1 (BernsteinDerivativeMatrix_3D.jl:
// 96-216 writes exactly these four terms per row). One warp per block and EPW elements per
// tile: the tile's inputs go to shared memory, one pass forms w for every requested axis, one
// pass forms the outputs and stores them coalesced; the next tile's inputs are loaded into
// registers while the current one is worked on. With the degree a compile-time constant every
// division by Np or Np(N-1) is a multiply-shift.
#include <algorithm>

#include "bbdg_internal.cuh"

namespace {

template <int N, int NA>  // NA = number of axes formed (1 or 3)
struct DerivFast {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NPM1 = N * (N + 1) * (N + 2) / 6;
  static constexpr int NW = NPM1 + 1;  // w rows end with a zero entry
  // elements per tile: about 1000 inputs, a multiple of 4 when Np is odd so that every tile
  // starts on a 16-byte boundary
  static constexpr int EPW0 = 1000 / NP > 0 ? 1000 / NP : 1;
  static constexpr int EPW = (NP % 2) ? std::max(4, EPW0 / 4 * 4)
                           : (NP % 4) ? std::max(2, EPW0 / 2 * 2) : EPW0;
  static constexpr int TILE = EPW * NP;           // floats per tile
  static constexpr int NV4 = (TILE / 4 + 31) / 32;  // float4 inputs per lane
  static constexpr int X_OFF = 0;                  // [EPW][NP]
  static constexpr int W_OFF = TILE;               // [NA][EPW][NW]
  static constexpr int VN_OFF = (W_OFF + NA * EPW * NW + 3) / 4 * 4;  // [NPM1] uint2
  static constexpr int GA_OFF = VN_OFF + 2 * NPM1;  // [NP] uint2
  static constexpr int GW_OFF = GA_OFF + 2 * NP;    // [NP] uint32
  static constexpr int SMEM = (GW_OFF + NP) * 4;
  static_assert(TILE % 4 == 0, "tiles are whole float4s");
};

template <int N, int MASK>
__global__ void __launch_bounds__(32) deriv_fast_kernel(int64_t K, const uint32_t* __restrict__ gtab,
                                                        int o_node3, int o_node3m1,
                                                        const float* __restrict__ x,
                                                        float* __restrict__ o0, float* __restrict__ o1,
                                                        float* __restrict__ o2) {
  constexpr int NA = MASK == 7 ? 3 : 1;
  using D = DerivFast<N, NA>;
  constexpr int NP = D::NP, NPM1 = D::NPM1, NW = D::NW, EPW = D::EPW, TILE = D::TILE, NV4 = D::NV4;
  // w row set of axis a
  constexpr int RA0 = 0, RA1 = MASK == 7 ? 1 : 0, RA2 = MASK == 7 ? 2 : 0;
  extern __shared__ __align__(16) float dsm[];
  float* sx = dsm + D::X_OFF;
  float* sW = dsm + D::W_OFF;
  uint2* sVN = reinterpret_cast<uint2*>(dsm + D::VN_OFF);
  uint2* sGA = reinterpret_cast<uint2*>(dsm + D::GA_OFF);
  uint32_t* sGW = reinterpret_cast<uint32_t*>(dsm + D::GW_OFF);
  const int t = threadIdx.x;
  constexpr uint32_t Z = NPM1;
  for (int b = t; b < NPM1; b += 32) {
    const uint32_t c = gtab[o_node3m1 + b];
    const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
    sVN[b] = make_uint2(ijk3(N, i + 1, j, k) | (ijk3(N, i, j + 1, k) << 16),
                        ijk3(N, i, j, k + 1) | (ijk3(N, i, j, k) << 16));
  }
  for (int n = t; n < NP; n += 32) {
    const uint32_t c = gtab[o_node3 + n];
    const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
    const uint32_t m0 = i > 0 ? ijk3(N - 1, i - 1, j, k) : Z;
    const uint32_t m1 = j > 0 ? ijk3(N - 1, i, j - 1, k) : Z;
    const uint32_t m2 = k > 0 ? ijk3(N - 1, i, j, k - 1) : Z;
    const uint32_t m3 = l > 0 ? ijk3(N - 1, i, j, k) : Z;
    sGA[n] = make_uint2(m0 | (m1 << 16), m2 | (m3 << 16));
    sGW[n] = (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16) | ((uint32_t)l << 24);
  }
  for (int r = t; r < NA * EPW; r += 32) sW[r * NW + NPM1] = 0.f;
  float* outs[3] = {o0, o1, o2};
  const int64_t ntile = (K + EPW - 1) / EPW;
  auto tile_ne = [&](int64_t tile) { return (int)(K - tile * EPW < EPW ? K - tile * EPW : EPW); };
  float4 pf[NV4];
  auto fetch = [&](int64_t tile) {
    const float4* xs = reinterpret_cast<const float4*>(x + tile * TILE);
    const int nv = tile_ne(tile) * NP;  // floats; the last tile may end inside a float4
#pragma unroll
    for (int r = 0; r < NV4; ++r) {
      const int v = t + 32 * r;
      if (4 * v + 3 < nv) {
        pf[r] = __ldg(xs + v);
      } else if (4 * v < nv) {  // ragged end: scalar loads of what exists
        const float* xf = x + tile * TILE + 4 * v;
        pf[r] = make_float4(xf[0], 4 * v + 1 < nv ? xf[1] : 0.f, 4 * v + 2 < nv ? xf[2] : 0.f, 0.f);
      }
    }
  };
  if (blockIdx.x < ntile) fetch(blockIdx.x);
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int ne = tile_ne(tile);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < NV4; ++r) {
      const int v = t + 32 * r;
      if (4 * v < ne * NP) reinterpret_cast<float4*>(sx)[v] = pf[r];
    }
    __syncwarp();
    if (tile + gridDim.x < ntile) fetch(tile + gridDim.x);
    for (int it = t; it < ne * NPM1; it += 32) {
      const int le = it / NPM1, b = it - le * NPM1;
      const uint2 vn = sVN[b];
      const float* xe = sx + le * NP;
      const float x3 = xe[vn.y >> 16];
      if (MASK & 1) sW[(RA0 * EPW + le) * NW + b] = xe[vn.x & 0xffff] - x3;
      if (MASK & 2) sW[(RA1 * EPW + le) * NW + b] = xe[vn.x >> 16] - x3;
      if (MASK & 4) sW[(RA2 * EPW + le) * NW + b] = xe[vn.y & 0xffff] - x3;
    }
    __syncwarp();
    const int64_t base = tile * TILE;
    for (int it = t; it < ne * NP; it += 32) {
      const int le = it / NP, n = it - le * NP;
      const uint2 ga = sGA[n];
      const uint32_t gw = sGW[n];
      const int m0 = ga.x & 0xffff, m1 = ga.x >> 16, m2 = ga.y & 0xffff, m3 = ga.y >> 16;
      const float a0 = float(gw & 0xff), a1 = float((gw >> 8) & 0xff),
                  a2 = float((gw >> 16) & 0xff), a3 = float(gw >> 24);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (!(MASK & (1 << a))) continue;
        const float* w = sW + ((MASK == 7 ? a : 0) * EPW + le) * NW;
        outs[a][base + it] = 0.5f * (a0 * w[m0] + a1 * w[m1] + a2 * w[m2] + a3 * w[m3]);
      }
    }
  }
}

template <int N, int MASK>
int launch_deriv_fast_t(bb_ctx* ctx, const DegTables* t, int64_t K, const void* x, void* o0,
                        void* o1, void* o2, cudaStream_t st) {
  using D = DerivFast<N, MASK == 7 ? 3 : 1>;
  auto kern = deriv_fast_kernel<N, MASK>;
  BB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, D::SMEM));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, D::SMEM));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "derivative tile does not fit");
  const int64_t ntile = (K + D::EPW - 1) / D::EPW;
  const int grid = (int)std::min<int64_t>(ntile, (int64_t)per_sm * ctx->num_sms);
  kern<<<grid, 32, D::SMEM, st>>>(K, t->d_words, t->o_node3, t->o_node3m1, (const float*)x,
                                  (float*)o0, (float*)o1, (float*)o2);
  return bb_check_launch(ctx, "deriv_fast_kernel");
}

template <int N>
int launch_deriv_fast_n(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x,
                        void* o0, void* o1, void* o2, cudaStream_t st) {
  switch (mask) {
    case 1: return launch_deriv_fast_t<N, 1>(ctx, t, K, x, o0, o1, o2, st);
    case 2: return launch_deriv_fast_t<N, 2>(ctx, t, K, x, o0, o1, o2, st);
    case 4: return launch_deriv_fast_t<N, 4>(ctx, t, K, x, o0, o1, o2, st);
    case 7: return launch_deriv_fast_t<N, 7>(ctx, t, K, x, o0, o1, o2, st);
    default: return -1;
  }
}

}  // namespace

// FP32 derivative(s) of K columns with the degree-specialised kernel; mask = axes (1, 2, 4 for
// one of r, s, t; 7 for all three). Returns -1 when none applies (degree above 11, another
// mask, or an input or output that is not 16-byte aligned), and the caller runs the generic
// kernel.
int bb_deriv_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x, void* o0,
                  void* o1, void* o2, cudaStream_t st) {
  if ((((uintptr_t)x) & 15) != 0) return -1;
#define BB_DF(n_) \
  case n_:        \
    return launch_deriv_fast_n<n_>(ctx, t, K, mask, x, o0, o1, o2, st);
  switch (t->N) {
    BB_DF(1) BB_DF(2) BB_DF(3) BB_DF(4) BB_DF(5) BB_DF(6) BB_DF(7) BB_DF(8) BB_DF(9) BB_DF(10)
    BB_DF(11)
    default:
      return -1;
  }
#undef BB_DF
}
