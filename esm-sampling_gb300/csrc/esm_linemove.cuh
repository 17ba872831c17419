// Host entry points of the line-move kernels (esm_linemove_impl.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "esm_common.cuh"

namespace esm {
template <class real>
size_t linemove_scratch_reals(const DevModel<real> &M);  // per warp
template <class real>
size_t linemove_smem_per_warp(const DevModel<real> &M);  // bytes of one move descriptor
// one colour class: the descriptors of its moves into descs ((natoms + nextra) descriptors), then
// one launch per move; the sweep index is read on the device from *sweep (graph-capturable)
template <class real>
cudaError_t launch_class_pass(const DevModel<real> &M, const int *steps, int nsteps, const uint32_t *sweep, int cls,
                              int limit, real *scratch, int wpb, int max_warps, unsigned long long *stats,
                              char *descs, unsigned int *counters, cudaStream_t s);
// resident k_move warps per SM with blocks of wpb (1, 2 or 4) warps
template <class real>
int linemove_blocks_per_sm(const DevModel<real> &M, int wpb);
}  // namespace esm
