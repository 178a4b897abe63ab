// Degree-specialised FP32 stage-kernel variants for N = 7, 8 (split from the other
// degrees so that the variants compile in parallel).
#include "bbdg_stage_fast_impl.cuh"

template int bbfast::launch_fast_t<7, BB_WAVE, 4, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<7, BB_MAXWELL, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<8, BB_WAVE, 4, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<8, BB_MAXWELL, 4, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<7, BB_WAVE, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
