/*
 * rt_bvh_gpu.h - the reference's SAH tree built on the GPU (rt_bvh_gpu.cu).
 * Produces exactly the nodes and primitive order of rtb::build_sah.
 */
#ifndef RT_BVH_GPU_H
#define RT_BVH_GPU_H
#include <cuda_runtime.h>
#include <vector>
#include "rt_bvh.h"

/* cudaMalloc that also counts the call in a process-wide tally (rt_host.cpp),
 * so tests can show which entry points allocate device memory */
cudaError_t rt_dev_malloc(void** p, size_t bytes);

cudaError_t rt_gpu_build_sah(const std::vector<rtb::Box>& bounds, int max_prims, rtb::BuildResult* out, cudaStream_t s);

#endif
