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
// fixed-point cell CDF (cdf_quantize), four launches (species maxima ymax,
// tile sums, tile offsets, scan): row s holds n + 1 entries C[0..n],
// the guide table 2^g + 1 entries per species, g = cdf_guide_bits(n)
cudaError_t launch_cdf(const float* yields, uint32_t* ymax, int n_species, int64_t n,
                       unsigned long long* tile_sum, unsigned long long* tile_off,
                       unsigned long long* qtot, double* totals, unsigned long long* cdf,
                       int32_t* guide, cudaStream_t stream);

// kernels_sample.cu
// two launches: per-species Poisson constants and inversion tables (pois,
// (kPoissonConsts + kInvTable + 1) doubles per species), then one count per
// (event, species)
cudaError_t launch_counts(const DevConfig& cfg, const double* totals, double* pois, int32_t* counts,
                          int32_t* items, int* error, cudaStream_t stream);
int offsets_num_tiles(int64_t n);
cudaError_t launch_offsets_scan(const int32_t* counts, int64_t n, int64_t* tile_sum,
                                int64_t* offsets, cudaStream_t stream);
cudaError_t launch_item_map(const int32_t* items, const int64_t* item_off, int64_t nseg,
                            int32_t* item_seg, cudaStream_t stream);
// work items [k_begin, k_end) in two launches: the first-draw cell of every
// hadron (cell_of, one int32 per slot), then the sampler; work_counter must
// be zero
cudaError_t launch_sampler(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                           const int32_t* pids, const unsigned long long* cdf,
                           const int32_t* guide, int guide_bits, const unsigned long long* qtot,
                           const int64_t* offsets,
                           const int64_t* item_off, const int32_t* item_seg, int64_t k_begin,
                           int64_t k_end, int32_t* cell_of, HadronRec* out,
                           unsigned long long* work_counter, SampleCounters* counters, int num_sms,
                           cudaStream_t stream);

}  // namespace iss
