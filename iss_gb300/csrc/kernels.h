// Launch wrappers of the sampler's CUDA kernels (host-callable).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace iss {

// kernels_cells.cu
cudaError_t launch_cell_prologue(const DevConfig& cfg, const float* fo34, int64_t n,
                                 const CellArrays& cells, cudaStream_t stream);
cudaError_t launch_yields(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                          float* yields, cudaStream_t stream);
int cdf_num_tiles(int64_t n);
// buckets of the per-species guide table (guide_len + 1 entries per species)
int cdf_guide_len(int64_t n);
cudaError_t launch_cdf(const float* yields, int n_species, int64_t n, double* tile_sum,
                       double* tile_off, double* totals, double* cdf, int32_t* guide,
                       cudaStream_t stream);

// kernels_sample.cu
cudaError_t launch_counts(const DevConfig& cfg, const double* totals, int32_t* counts,
                          int32_t* items, int* error, cudaStream_t stream);
int offsets_num_tiles(int64_t n);
cudaError_t launch_offsets_scan(const int32_t* counts, int64_t n, int64_t* tile_sum,
                                int64_t* offsets, cudaStream_t stream);
cudaError_t launch_item_map(const int32_t* items, const int64_t* item_off, int64_t nseg,
                            int32_t* item_seg, cudaStream_t stream);
cudaError_t launch_sampler(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                           const int32_t* pids, const double* cdf, const int32_t* guide,
                           int guide_len, const double* totals, const int64_t* offsets,
                           const int64_t* item_off, const int32_t* item_seg, int64_t n_items,
                           HadronRec* out, unsigned long long* work_counter,
                           SampleCounters* counters, int num_sms, cudaStream_t stream);

}  // namespace iss
