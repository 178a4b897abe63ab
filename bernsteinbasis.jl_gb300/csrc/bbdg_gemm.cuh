// BF16 tcgen05 GEMM with a fused epilogue, shared by the GEMM entry point and the closure MLP.
#pragma once

#include <cuda_bf16.h>

#include "bbdg_internal.cuh"

// C = alpha * A[M x K] * B[N x K]^T, A and B row-major BF16 (K contiguous), then per element
// (row r < M, column c < N), with v the FP32 accumulator value:
//   v = alpha * v + bias[c]                      (bias optional)
//   act 1: Pre[r][c] = v (if Pre), v = GELU(v)   (exact erf form)
//   act 2: v = v * GELU'(Pre[r][c])              (backward through GELU)
//   Cf[r][c] = v (or += v with accumulate), Cb[r][c] = bf16(v), CbT[c][r] = bf16(v),
//   bias_grad[c] += sum over rows of v
// With kt_per > 0 the K range is split over gridDim.z CTAs whose partial sums are added
// atomically into Cf (no other output allowed).
// Row-major outputs use leading dimension ldc, the transposed BF16 output leading dimension
// ldt. Every output pointer is optional.
struct GemmEpilogue {
  int M, N, K;
  float alpha;
  const float* bias;
  int act;
  float* Pre;
  float* Cf;
  int accumulate;
  __nv_bfloat16* Cb;
  __nv_bfloat16* CbT;
  float* bias_grad;
  int ldc, ldt;
  int kt_per;   // split-K: K blocks of 64 per CTA (0 = no split); split outputs add into Cf
  int* status;  // device error word: bit 1 = a pipeline wait ran out
  uint32_t wait_iters;  // polls of a bounded mbarrier wait before it gives up (0 = 2^24)
  int fault;            // test only: 1 = the second operand copy is left out
};

// Launches the GEMM on `st` (A, B device pointers, 16-byte aligned, K % 8 == 0).
int bb_gemm_launch(bb_ctx* ctx, int64_t M, int N, int K, const void* A, const void* B,
                   GemmEpilogue ep, cudaStream_t st);
