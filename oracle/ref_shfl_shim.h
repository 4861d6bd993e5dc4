/* Forced-include shim for building the reference GPU trainer (singleGPU/) with CUDA 13.
 * TEST INFRASTRUCTURE ONLY.  CUDA 13 dropped the maskless warp shuffles that
 * sgd_k128_kernel_hogwild_warp32.h:48,77-83 call; these two templates forward them to the
 * _sync forms with every lane of the warp named, which is what the reference's full-warp
 * calls meant.  Included after cuda_fp16.h (a macro form would rename the __shfl members
 * that cuda_fp16.h itself declares). */
#pragma once
#include <cuda_fp16.h>
template <typename T>
__device__ __forceinline__ T __shfl(T v, int src_lane) { return __shfl_sync(0xffffffffu, v, src_lane); }
template <typename T>
__device__ __forceinline__ T __shfl_down(T v, unsigned int delta) { return __shfl_down_sync(0xffffffffu, v, delta); }
