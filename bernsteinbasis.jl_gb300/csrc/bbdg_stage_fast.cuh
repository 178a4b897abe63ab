// Interface of the degree-specialised FP32 stage kernels (bbdg_stage_fast.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct FastStageParams {
  const uint32_t* gtab;  // degree tables (DegTables::d_words) and their word offsets
  int o_node3, o_node3m1, o_fvol, o_fperm, o_sslot;
  int64_t K;
  int64_t tile_begin, tile_end;  // tiles [tile_begin, tile_end) of EPB elements (end 0 = all)
  int mode;              // 0: rhs only, 1: LSRK stage update
  float rkA, rkB, dt, tau;
  float* q;              // [NF][K][Np]
  float* res;            // [NF][K][Np]
  float* rhs;            // mode 0 output
  const float* trace_in; // [K][4][NF][Nfp], all faces that cross a tile boundary
  float* trace_out;      // [K][4][NF][Nfp] or nullptr
  const float* geo;      // [K][BB_GEO_STRIDE]
  const int32_t* conn;   // [K][4]
  int* status;
  uint32_t wait_iters;   // polls of a bounded mbarrier wait before it gives up (0 = 2^24)
  int fault;             // test only: 1 = one bulk copy is left out (a wait then runs out)
  // volume phase: warp-round g = r * (TPE / 32) + warp forms w(beta) for beta = vstart[g] +
  // lane, lane < vlen[g] (filled by the launcher)
  uint16_t vstart[16];
  uint8_t vlen[16];
};

struct FastLaunch {
  int num_sms;
  int device;           // CUDA device ordinal (the per-device launch set-up is cached)
  uint32_t wait_iters;  // copied into FastStageParams (the context's wait limit)
  int fault;            // copied into FastStageParams (the context's test-only fault mode)
};

// Index of the compiled variant for (N, physics, elements per block, threads), 0 = any,
// usable for K elements (K must be a multiple of the tile; K <= 0: any); -1 if none.
int bb_fast_find(int N, int physics, int epb, int threads, int64_t K);
int bb_fast_variant_info(int idx, int* epb, int* threads, size_t* smem);
int bb_fast_launch(int idx, const FastLaunch& fl, const FastStageParams& P, cudaStream_t st);
