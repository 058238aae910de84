// Launch wrappers of the hash-split kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "gz_engine.cuh"

namespace gz {

cudaError_t launch_hash_count(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st);
cudaError_t launch_plan(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st);
cudaError_t launch_scatter(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st);
cudaError_t launch_gather(const HostCopy* jobs, uint32_t n_jobs, cudaStream_t st);
// The derived arrays of a pass's nested columns (`jobs` in device memory); errors into *err.
cudaError_t launch_nest_prep(const NestJob* jobs, uint32_t n_jobs, int32_t* err, cudaStream_t st);
size_t scatter_smem_bytes();
int max_str_columns();

}  // namespace gz
