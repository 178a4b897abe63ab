// Degree-specialised FP32 stage-kernel variants for N = 4, 5, 6 (split from the other
// degrees so that the variants compile in parallel).
#include "bbdg_stage_fast_impl.cuh"

template int bbfast::launch_fast_t<5, BB_WAVE, 4, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<5, BB_WAVE, 8, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<5, BB_MAXWELL, 4, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<5, BB_MAXWELL, 8, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<4, BB_WAVE, 8, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<4, BB_MAXWELL, 4, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<6, BB_WAVE, 4, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<6, BB_WAVE, 8, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<6, BB_MAXWELL, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<5, BB_WAVE, 2, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<6, BB_WAVE, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<5, BB_MAXWELL, 2, 32>(const FastLaunch&, const FastStageParams&, cudaStream_t);
