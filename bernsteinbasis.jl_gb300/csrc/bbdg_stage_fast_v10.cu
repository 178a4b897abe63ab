// Degree-specialised FP32 stage-kernel variants for N = 10, 11 (split from the other
// degrees so that the variants compile in parallel).
#include "bbdg_stage_fast_impl.cuh"

template int bbfast::launch_fast_t<10, BB_WAVE, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<10, BB_MAXWELL, 2, 64>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<10, BB_MAXWELL, 2, 96>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<11, BB_WAVE, 2, 96>(const FastLaunch&, const FastStageParams&, cudaStream_t);
template int bbfast::launch_fast_t<11, BB_MAXWELL, 2, 96>(const FastLaunch&, const FastStageParams&, cudaStream_t);
