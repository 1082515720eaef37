// scf_stage.h -- host<->device staging of the callers' arrays.
//
// On GB300 the host's memory is reached over NVLink-C2C.  Measured on this
// GPU with 20 page-locked arrays of 137 MB per round, 100 rounds each:
// copies by the copy engines (cudaMemcpyAsync) ran at 210 GB/s but stalled
// in 24 of 100 rounds, taking 2 to 10 times as long; a kernel that reads the
// same buffers through their device-mapped address ran at the same 210 GB/s
// and stalled in none.  Kernels reading pageable memory directly stalled in
// 12 of 100.  So a page-locked, device-mapped array is moved by a kernel;
// anything else (pageable memory, or a pointer the device cannot address)
// goes through cudaMemcpyAsync, which stages pageable memory itself.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

// How a copy was made.
enum StageHow { STAGE_KERNEL = 0, STAGE_COPY_ENGINE = 1 };

// Copies `bytes` (a multiple of 4) from host `src` to device `dst` on
// `st`.  `max_blocks` bounds the copy kernel's grid (0: the whole GPU);
// `*how` (optional) says which path was taken; `*launches` counts kernels.
cudaError_t stage_h2d(void *dst, const void *src, size_t bytes, cudaStream_t st, int max_blocks, int *launches,
                      StageHow *how);

// The other direction, device `src` to host `dst`, by a kernel storing into
// the device-mapped address of a page-locked `dst` (the copy engines' writes
// to host memory stall now and then too), else by cudaMemcpyAsync.  The
// host sees the values once the stream has been synchronised.
cudaError_t stage_d2h(void *dst, const void *src, size_t bytes, cudaStream_t st, int max_blocks, int *launches,
                      StageHow *how);
