// Registry of the degree-specialised FP32 stage kernels: lookup, tile information and launch
// by variant index. The kernels themselves are instantiated in bbdg_stage_fast_v*.cu.
#include "bbdg_stage_fast_impl.cuh"
#include "bbdg_stage_fast_variants.h"

using bbfast::FastLayout;
#define BB_EXTERN(n_, p_, e_, t_) \
  extern template int bbfast::launch_fast_t<n_, p_, e_, t_>(const FastLaunch&, const FastStageParams&, cudaStream_t);
BB_FAST_VARIANTS(BB_EXTERN)
#undef BB_EXTERN

// The public tile description is (elements per block, threads per block).
int bb_fast_find(int N, int physics, int epb, int threads, int64_t K) {
  int idx = 0;
#define BB_FIND(n_, p_, e_, t_)                                                        \
  if (N == n_ && physics == p_ && (epb == 0 || epb == e_) &&                           \
      (threads == 0 || threads == FastLayout<n_, p_, e_, t_>::NT) &&                   \
      (K <= 0 || K % e_ == 0))                                                         \
    return idx;                                                                        \
  ++idx;
  BB_FAST_VARIANTS(BB_FIND)
#undef BB_FIND
  return -1;
}

int bb_fast_variant_info(int idx, int* epb, int* threads, size_t* smem) {
  int i = 0;
#define BB_INFO(n_, p_, e_, t_)                       \
  if (idx == i) {                                     \
    *epb = e_;                                        \
    *threads = FastLayout<n_, p_, e_, t_>::NT;        \
    *smem = FastLayout<n_, p_, e_, t_>::BYTES;        \
    return BB_OK;                                     \
  }                                                   \
  ++i;
  BB_FAST_VARIANTS(BB_INFO)
#undef BB_INFO
  return BB_ERR_ARG;
}

// C ABI: the compiled variants, for tile choosers (the autotuner times every one that fits).
extern "C" int bb_fast_variant(int idx, int* N, int* physics, int* epb, int* threads) {
  if (!N || !physics || !epb || !threads) return BB_ERR_ARG;
  int i = 0;
#define BB_VAR(n_, p_, e_, t_)                        \
  if (idx == i) {                                     \
    *N = n_;                                          \
    *physics = p_;                                    \
    *epb = e_;                                        \
    *threads = FastLayout<n_, p_, e_, t_>::NT;        \
    return BB_OK;                                     \
  }                                                   \
  ++i;
  BB_FAST_VARIANTS(BB_VAR)
#undef BB_VAR
  return BB_ERR_ARG;
}

int bb_fast_launch(int idx, const FastLaunch& fl, const FastStageParams& P, cudaStream_t st) {
  int i = 0;
#define BB_LAUNCH(n_, p_, e_, t_)                                 \
  if (idx == i) return bbfast::launch_fast_t<n_, p_, e_, t_>(fl, P, st);  \
  ++i;
  BB_FAST_VARIANTS(BB_LAUNCH)
#undef BB_LAUNCH
  return BB_ERR_ARG;
}
