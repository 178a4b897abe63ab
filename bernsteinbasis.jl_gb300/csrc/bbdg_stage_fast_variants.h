// Registry of the compiled degree-specialised stage-kernel variants:
// X(N, physics, elements per block, threads per element). The first variant matching a query
// (and dividing the element count) is the default for that (N, physics), so each degree
// lists its fastest tile on a 16^3 x 6 mesh first; the 2-element tiles at the end serve
// meshes whose element count is not a multiple of the larger tiles. Each is instantiated in
// one bbdg_stage_fast_v*.cu.
#pragma once
#define BB_FAST_VARIANTS(X) \
  X(9, BB_WAVE, 4, 64) \
  X(9, BB_WAVE, 4, 32) \
  X(9, BB_WAVE, 2, 64) \
  X(9, BB_MAXWELL, 2, 64) \
  X(9, BB_MAXWELL, 2, 96) \
  X(5, BB_WAVE, 8, 32) \
  X(5, BB_WAVE, 4, 32) \
  X(5, BB_MAXWELL, 4, 32) \
  X(5, BB_MAXWELL, 8, 32) \
  X(10, BB_WAVE, 2, 64) \
  X(10, BB_MAXWELL, 2, 96) \
  X(10, BB_MAXWELL, 2, 64) \
  X(4, BB_WAVE, 8, 32) \
  X(4, BB_MAXWELL, 4, 32) \
  X(6, BB_WAVE, 8, 32) \
  X(6, BB_WAVE, 4, 32) \
  X(6, BB_MAXWELL, 2, 64) \
  X(7, BB_WAVE, 4, 64) \
  X(7, BB_MAXWELL, 2, 64) \
  X(8, BB_WAVE, 4, 64) \
  X(8, BB_MAXWELL, 4, 32) \
  X(11, BB_WAVE, 2, 96) \
  X(11, BB_MAXWELL, 2, 96) \
  X(5, BB_WAVE, 2, 32) \
  X(6, BB_WAVE, 2, 64) \
  X(7, BB_WAVE, 2, 64) \
  X(5, BB_MAXWELL, 2, 32)
