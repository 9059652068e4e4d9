// Launch wrappers of the sampler's CUDA kernels (host-callable).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace iss {

// kernels_cells.cu
cudaError_t launch_cell_prologue(const DevConfig& cfg, const float* fo34, int64_t n,
                                 const CellArrays& cells, cudaStream_t stream);
// per-cell yields [species][cell] and, in ymax (n_surf * S rows, zeroed
// here first), the largest yield of every (surface, species) row as float bits
cudaError_t launch_yields(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                          float* yields, uint32_t* ymax, cudaStream_t stream);
int cdf_num_tiles(int64_t n);
// Fixed-point cell CDF (cdf_quantize) of every (surface, species) row of a
// batch from the yields and their row maxima (launch_yields); three launches
// over n_tiles = sum over surfaces of S * nt tiles (tile sums, tile offsets,
// scan).  Row (b, k) of the CDF holds
// n_b + 1 entries C[0..n_b] at surf[b].cdf_base + k (n_b + 1); its guide
// table 2^g_b + 1 entries at surf[b].guide_base + k (2^g_b + 1).  ymax,
// qtot and totals hold n_surf * S rows.  surf is a device array.
cudaError_t launch_cdf(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                       int64_t n_tiles, int S, uint32_t* ymax, unsigned long long* tile_sum,
                       unsigned long long* tile_off, unsigned long long* qtot, double* totals,
                       unsigned long long* cdf, int32_t* guide, cudaStream_t stream);
// the same in two parts: tile sums and tile offsets (which also give qtot and
// totals), then the scan that writes the CDF rows and guide tables
cudaError_t launch_cdf_head(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                            int64_t n_tiles, int S, uint32_t* ymax, unsigned long long* tile_sum,
                            unsigned long long* tile_off, unsigned long long* qtot, double* totals,
                            unsigned long long* cdf, int32_t* guide, cudaStream_t stream);
cudaError_t launch_cdf_scan(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                            int64_t n_tiles, int S, const uint32_t* ymax, const unsigned long long* tile_off,
                            const unsigned long long* qtot, unsigned long long* cdf, int32_t* guide,
                            cudaStream_t stream);

// kernels_sample.cu
// two launches: Poisson constants and inversion tables of every (surface,
// species) row (pois, (kPoissonConsts + kInvTable + 1) doubles per row), then
// one count per (event, species); totals has n_surfaces * S rows
cudaError_t launch_counts(const DevConfig& cfg, const SpeciesDev* species, const double* totals,
                          double* pois, int32_t* counts, int32_t* items, int* error,
                          cudaStream_t stream);
int offsets_num_tiles(int64_t n);
cudaError_t launch_offsets_scan(const int32_t* counts, int64_t n, int64_t* tile_sum,
                                int64_t* offsets, cudaStream_t stream);
cudaError_t launch_item_map(const int32_t* items, const int64_t* item_off, int64_t nseg,
                            int32_t* item_seg, cudaStream_t stream,
                            const int64_t* limits = nullptr);
// graph replays: limits[0] = the call's work items, limits[1] = 1 when the
// call does not fit the captured buffers (cap_units records, cap_items items)
cudaError_t launch_graph_limits(const int64_t* offsets, const int64_t* item_off, int64_t nseg,
                                int64_t cap_units, int64_t cap_items, int64_t* limits,
                                cudaStream_t stream);
// work items [k_begin, k_end) in two launches: the first-draw cell of every
// hadron (cell_of, one int32 per slot), then the sampler; work_counter must
// be zero
cudaError_t launch_sampler(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                           const int32_t* pids, const unsigned long long* cdf,
                           const int32_t* guide, const unsigned long long* qtot,
                           const int64_t* offsets,
                           const int64_t* item_off, const int32_t* item_seg, int64_t k_begin,
                           int64_t k_end, int32_t* cell_of, HadronRec* out,
                           unsigned long long* work_counter, SampleCounters* counters, int num_sms,
                           cudaStream_t stream, const int64_t* k_end_dev = nullptr);

// learned proposal (kernels_sample.cu): network inputs of the pairs
// (slot, cell), slot < n_slots, as bf16 rows [n_slots * n_cells][32]; the
// envelope constants of the pairs' mixture records (n_pilot proposals, times
// safety; the records come from the network's fused epilogue); training rows
// (features, (K, n) targets) from n sampled hadrons and their cells, with the
// plain proposal's negative log-likelihood of the rows added to *nll_plain
cudaError_t launch_learned_pairs(const DevConfig& cfg, const CellArrays& cells,
                                 const SpeciesDev* species, const int32_t* lspecies, int n_slots,
                                 void* x, cudaStream_t stream);
cudaError_t launch_learned_envelopes(const DevConfig& cfg, const CellArrays& cells,
                                     const SpeciesDev* species, const int32_t* lspecies, int n_slots,
                                     int n_pilot, float safety, float* lpairs, cudaStream_t stream);
cudaError_t launch_learned_train_rows(const DevConfig& cfg, const CellArrays& cells,
                                      const SpeciesDev* species, const int32_t* sorted_pid,
                                      const int32_t* sorted_idx, int S, const HadronRec* had,
                                      const int32_t* cell_of, int64_t n, void* x, void* tg,
                                      double* nll_plain, cudaStream_t stream);

// kernels_decay.cu: resonance decays, one generation over all events at a
// time: a count sweep on particle ids (sizes and final places, kept on the
// device), then a write sweep with the kinematics.  DecayMeta (int64 slots of
// `meta`): kDecayMetaNIn + g the input size of generation g (g <= g_max),
// kDecayMetaSBase + g the stable products of generations < g,
// kDecayMetaIBase + g where generation g's inputs start in the per-input
// arrays, kDecayMetaFlags (1: final lists too small, 2: one generation's
// records too small, 4: chains longer than g_max, 8: per-input arrays too
// small), kDecayMetaNeedS / NeedU / NeedI what the failing generation
// needed, kDecayMetaMaxU the largest next input seen.
constexpr int kDecayMetaFlags = 0;
constexpr int kDecayMetaNeedS = 1;
constexpr int kDecayMetaNeedU = 2;
constexpr int kDecayMetaMaxU = 3;
constexpr int kDecayMetaNeedI = 4;
constexpr int kDecayMetaNIn = 8;
constexpr int kDecayMaxGenerations = 64;
constexpr int kDecayMetaSBase = kDecayMetaNIn + kDecayMaxGenerations + 1;
constexpr int kDecayMetaIBase = kDecayMetaSBase + kDecayMaxGenerations + 1;
constexpr int kDecayMetaLen = kDecayMetaIBase + kDecayMaxGenerations + 1;

struct DecayBuffers {
    const HadronRec* rec0;      // the sampled records (generation 0's input), event-sorted
    int32_t* ev;                // [i_cap] event of every input, generations back to back
    int32_t* pid;               // [i_cap] particle id of every input of generations >= 1
    int32_t* chan;              // [i_cap] per input: (type << 16) | channel, or < 0
    int64_t* cnt;               // [largest generation] (stable products << 32) | unstable ones
    int64_t* off;               // [i_cap + g_max + 1] generation g's exclusive scan of cnt
                                // (inputs + 1 entries) from IBase + g: both offsets at once
    int64_t* tiles;             // one per scan tile of 4096 inputs
    int64_t* first;             // [g_max][n_events] input range of each event per generation
    int64_t* last;              //   (-1: none)
    int64_t* scnt;              // [g_max][n_events] stable products of each event per generation
    int64_t* shift;             // [g_max][n_events] final place of the event's first stable
                                //   product of the generation, less its stable scan offset
    int64_t* meta;              // DecayMeta
    unsigned long long* failures;
    int64_t s_cap, u_cap, i_cap;   // final lists, one generation's records, per-input arrays
    uint32_t g_max;
};

// event ids and input ranges of generation 0 from the sampled event offsets
cudaError_t launch_decay_first_generation(const int64_t* evoff, int n_events, const DecayBuffers& b,
                                          cudaStream_t s);
// count sweep of one generation: channel cache, packed scan, sizes of the
// next generation, its inputs' ids and events, per-event ranges
cudaError_t launch_decay_count_generation(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                                          const DecayBuffers& b, int n_events, int num_sms,
                                          cudaStream_t s);
// final lists of generations < n_gen: per-event totals, event offsets
// (evoff, n_events + 1) and the per (generation, event) shifts
cudaError_t launch_decay_layout(const DecayBuffers& b, int n_gen, int n_events, int32_t* ev_tot,
                                int64_t* tiles, int64_t* evoff, cudaStream_t s);
// write sweep of generation gen (n inputs from ib): stable products to out,
// unstable ones to out_u (the next generation's records)
cudaError_t launch_decay_write_generation(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                                          int64_t n, int64_t ib, const HadronRec* in, HadronRec* out_u,
                                          const DecayBuffers& b, int n_events, int num_sms,
                                          HadronRec* out, cudaStream_t s);

// kernels_output.cu: OSCAR text (FSSW::combine_samples_to_OSCAR) of hadrons
// [h0, h1), which are the whole events [e_lo, e_hi).  ev_off: the events'
// first hadrons (n_events + 1 entries); ev_byte: the byte offset of each
// event's block in the file body (sub-header, then its lines).  Writes to
// out + ev_byte[e] - byte0.
constexpr int kOscarSubHeader = 43;   // setw(10) iev, setw(10) n, two setw(8) zeros
constexpr int kOscarLine = 257;       // setw(10) ipart, setw(10) pid, nine %24.16e
cudaError_t launch_oscar_lines(const HadronRec* had, int64_t h0, int64_t h1, const int64_t* ev_off,
                               const int64_t* ev_byte, int e_lo, int e_hi, int64_t byte0,
                               char* out, int num_sms, cudaStream_t stream);

}  // namespace iss
