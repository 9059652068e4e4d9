// C ABI of the sampler (include/iss_gpu.h): the handle, the host side of
// iSS::read_in_FO_surface / generate_samples, device memory and the launch
// sequence of one generate:
//   upload surface -> cell prologue -> yields -> per-species CDF
//   -> counts -> slot offsets -> sampler -> event offsets back to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <map>
#include <mutex>
#include <tuple>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "devbuf.h"
#include "host/params.h"
#include "host/surface_io.h"
#include "host/tables.h"
#include "host/writers.h"
#include "iss_gpu.h"
#include "kernels.h"
#include "kernels_mlp.h"
#include "learned.h"

using namespace iss;

namespace {

struct TableKey {
    std::string table_path;
    int afterburner = -1, bulk_kind = -1, include_bulk = -1, include_diff = -1, neos = -9;
    int fix_c0 = -1;
    bool operator==(const TableKey& o) const {
        return table_path == o.table_path && afterburner == o.afterburner &&
               bulk_kind == o.bulk_kind && include_bulk == o.include_bulk &&
               include_diff == o.include_diff && neos == o.neos && fix_c0 == o.fix_c0;
    }
};

// Pinned host results of a graph replay: written by the graph's copies.
struct GraphHost {
    int64_t units, items, limits[2];
    int32_t count_err, pad;
    SampleCounters ctr;
    uint32_t run[4];            // seed and event offset uploaded before a replay
    int64_t event_offsets[1];   // n_events + 1 entries (allocated with the struct)
};

enum Phase { kEvStart = 0, kEvPrologue, kEvYields, kEvCdf, kEvCounts, kEvSampleStart, kEvSample,
             kEvLearnStart, kEvLearnEnd, kEvFwdStart, kEvFwdEnd, kEvCount };

}  // namespace

struct iss_handle {
    std::string work_path, table_path, particle_table_path, surface_filename;
    ParamStore params;
    std::string last_error;
    int64_t seed = 1;
    bool seed_set = false;

    // surface (host)
    std::vector<float> fo34;
    int64_t n_cells = 0;
    // a batch of surfaces (iss_gpu_set_surface_batch); empty for one surface
    std::vector<int64_t> batch_cells;     // cell offsets, n_surfaces + 1
    std::vector<int32_t> batch_events;    // events per surface
    std::vector<SurfSeg> segs;            // per-surface layout of the CDF rows
    std::vector<int32_t> ev_surf;         // surface of every event (host copy of d_ev_surf)
    // resonance decays (perform_decays = 1, not for the SMASH afterburner)
    bool decays = false;
    int decay_table_afterburner = -1;
    DevBuf<DecayParticle> d_dparticles;
    DevBuf<DecayChannel> d_dchannels;
    DevBuf<int32_t> d_dsorted;            // sorted pids, then their indices
    DevBuf<int2> d_dhash;                 // pid -> particle index (kDecayHash slots)
    int n_decay_particles = 0;
    cudaEvent_t ev_decay[2] = {nullptr, nullptr};
    // decay work buffers (grow-only): one generation's records (ping-pong),
    // the per-input arrays of all generations, per-(generation, event) tables
    // and the final lists
    DevBuf<HadronRec> dk_u[2], dk_final;
    DevBuf<int32_t> dk_ev, dk_pid, dk_chan, dk_etot;
    DevBuf<int64_t> dk_cnt, dk_coff, dk_tiles, dk_first, dk_last, dk_scnt, dk_shift, dk_meta,
        dk_off, dk_etiles, dk_evoff;
    DevBuf<unsigned long long> dk_fail;
    int64_t dk_scap_hint = 0, dk_ucap_hint = 0, dk_icap_hint = 0;   // sizes the last call needed
    int dk_gen_hint = 0;                           // generations the last call had
    int32_t dk_reruns = 0;                         // decay passes rerun in the last call
    int64_t cdf_len = 0, guide_len = 0, n_tiles = 0;
    int hydro_mode = 2;
    int iEOS = 2;
    int afterburner = 0;
    bool surface_loaded = false;
    bool surface_on_device = false;
    bool quantum_statistics = true;
    std::vector<Species> species;
    std::vector<Species> resonances;
    int species_afterburner = -1;
    bool species_qs = true;

    // device
    bool cuda_ready = false;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;     // device->host copies of iss_gpu_generate_into
    // the captured generate's second branch (the counts beside the CDF scan)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<cudaEvent_t> chunk_ev;      // end of each sampling chunk
    std::vector<cudaEvent_t> copy_ev;       // streamed generates: end of each chunk's copy
    iss_hadron_t* stream_host = nullptr;    // streamed generates: two page-locked chunk buffers
    int64_t stream_host_cap = 0;            // records per buffer
    cudaEvent_t ev[kEvCount] = {};
    DevBuf<float> d_fo34;
    DevBuf<float4> d_cells;          // 8 arrays of n_cells float4
    DevBuf<float4> d_milne;          // MC_sampling = 2: regulated Milne cells, 6 float4 each
    DevBuf<SpeciesDev> d_species;
    DevBuf<int32_t> d_pids;
    DevBuf<int32_t> d_yorder;        // yields kernel: species grouped by identical series
    DevBuf<float> d_yields;
    DevBuf<unsigned long long> d_cdf, d_tile_sum, d_tile_off, d_qtot;
    DevBuf<double> d_totals;
    DevBuf<uint32_t> d_ymax;
    DevBuf<int32_t> d_counts, d_items, d_item_seg, d_guide, d_cell_of, d_ev_surf;
    DevBuf<SurfSeg> d_surf;
    DevBuf<int64_t> d_offsets, d_off_tiles, d_item_off;
    DevBuf<HadronRec> d_hadrons;
    DevBuf<unsigned long long> d_work;
    DevBuf<SampleCounters> d_counters;
    DevBuf<int> d_error;
    // tables
    TableKey table_key;
    DevBuf<float4> d_sfK;
    DevBuf<float> d_sfE;
    DevBuf<double> d_b14c0, d_b14c1, d_b14c2, d_ce, d_qmu, d_logfact, d_pois;
    Bulk14Table b14;

    // last generate
    DevConfig cfg{};
    bool yields_valid = false;
    bool samples_valid = false;
    int n_events = 0;
    int64_t n_hadrons = 0;
    std::vector<int64_t> event_offsets;
    std::vector<iss_hadron_t> host_hadrons;
    bool host_valid = false;
    std::vector<double> totals;
    iss_timings_t timings{};
    // graph replay of a generate (gpu_graph = 1): the executable graph, the
    // call shape it was captured for, its buffer capacities, and pinned host
    // memory its copies write to
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_unavailable = false;
    std::vector<unsigned char> graph_key;
    int64_t graph_cap_units = 0, graph_cap_items = 0;
    DevBuf<uint32_t> d_run;
    DevBuf<int64_t> d_limits;
    GraphHost* gh = nullptr;
    size_t gh_events = 0;
    // launch shape of the kernels (iss_gpu_set_tuning / iss_gpu_autotune)
    iss_tuning_t tune{64, 4, 3, 8, 16};
    bool tuned = false;
    // the learned proposal: network, training set, per-pair mixture tables
    Learned learned;
    bool use_learned = false;            // gpu_sampler = 1
    DevBuf<int32_t> d_lslot, d_lspecies, d_spid;
    DevBuf<float> d_lpairs;
    iss_learned_stats_t lstats{};

    ~iss_handle() {
        if (cuda_ready) {
            DevBuf<float>* fb[] = {&d_fo34, &d_yields, &d_sfE};
            for (auto* b : fb) b->release();
            d_cells.release();
            d_milne.release();
            d_species.release();
            d_pids.release();
            d_yorder.release();
            DevBuf<double>* db[] = {&d_totals, &d_b14c0, &d_b14c1, &d_b14c2, &d_ce, &d_qmu,
                                    &d_logfact, &d_pois};
            for (auto* b : db) b->release();
            DevBuf<unsigned long long>* ub[] = {&d_cdf, &d_tile_sum, &d_tile_off, &d_qtot};
            for (auto* b : ub) b->release();
            d_ymax.release();
            d_counts.release();
            d_items.release();
            d_item_seg.release();
            d_guide.release();
            d_cell_of.release();
            d_ev_surf.release();
            d_surf.release();
            d_offsets.release();
            d_off_tiles.release();
            d_item_off.release();
            d_hadrons.release();
            d_work.release();
            d_counters.release();
            d_error.release();
            d_sfK.release();
            for (auto& e : ev)
                if (e) cudaEventDestroy(e);
            for (auto& e : chunk_ev)
                if (e) cudaEventDestroy(e);
            for (auto& e : copy_ev)
                if (e) cudaEventDestroy(e);
            if (stream_host) cudaFreeHost(stream_host);
            for (auto& e : ev_decay)
                if (e) cudaEventDestroy(e);
            d_dparticles.release();
            d_dchannels.release();
            d_dsorted.release();
            d_dhash.release();
            for (auto* b : {&dk_u[0], &dk_u[1], &dk_final}) b->release();
            for (auto* b : {&dk_ev, &dk_pid, &dk_chan, &dk_etot}) b->release();
            for (auto* b : {&dk_cnt, &dk_coff, &dk_tiles, &dk_first, &dk_last, &dk_scnt, &dk_shift,
                            &dk_meta, &dk_off, &dk_etiles, &dk_evoff})
                b->release();
            dk_fail.release();
            learned.release_all();
            if (graph_exec) cudaGraphExecDestroy(graph_exec);
            if (gh) cudaFreeHost(gh);
            d_run.release();
            d_limits.release();
            d_lslot.release();
            d_lspecies.release();
            d_spid.release();
            d_lpairs.release();
            if (copy_stream) cudaStreamDestroy(copy_stream);
            if (aux_stream) cudaStreamDestroy(aux_stream);
            if (ev_fork) cudaEventDestroy(ev_fork);
            if (ev_join) cudaEventDestroy(ev_join);
            if (stream) cudaStreamDestroy(stream);
        }
    }
};

namespace {

iss_status fail(iss_handle* h, iss_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->last_error = buf;
    return st;
}

#define CUDA_TRY(h, call)                                                                   \
    do {                                                                                    \
        cudaError_t _e = (call);                                                            \
        if (_e != cudaSuccess)                                                              \
            return fail((h), ISS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

// Species groups of the yields kernel.  The thermal series of
// calculate_dN_analytic (src/FSSW.cpp:719-848) depends on a species only
// through its mass, statistics, number of terms and chemical potential, so
// species that agree in the first three share one series per cell (isospin
// partners, particles and antiparticles).  Layout: G + 1 group starts into
// the member list, then the members (species indices, each species once).
// Groups are ordered by decreasing work (series terms, then members), so
// that the kernel's interleaving of groups over grid rows stays balanced.
std::vector<int32_t> yield_group_order(const std::vector<SpeciesDev>& sd) {
    std::vector<std::vector<int32_t>> groups;
    for (size_t k = 0; k < sd.size(); k++) {
        const SpeciesDev& a = sd[k];
        bool placed = false;
        for (auto& g : groups) {
            const SpeciesDev& b = sd[g[0]];
            if (a.m_hi == b.m_hi && a.m_lo == b.m_lo && a.sign == b.sign && a.light == b.light) {
                g.push_back(static_cast<int32_t>(k));
                placed = true;
                break;
            }
        }
        if (!placed) groups.push_back({static_cast<int32_t>(k)});
    }
    auto cost = [&](const std::vector<int32_t>& g) {
        return (sd[g[0]].light ? 20 : 2) + static_cast<int>(g.size());
    };
    std::stable_sort(groups.begin(), groups.end(),
                     [&](const auto& x, const auto& y) { return cost(x) > cost(y); });
    std::vector<int32_t> out;
    int32_t start = 0;
    for (const auto& g : groups) {
        out.push_back(start);
        start += static_cast<int32_t>(g.size());
    }
    out.push_back(start);
    for (const auto& g : groups) out.insert(out.end(), g.begin(), g.end());
    return out;
}

iss_status ensure_cuda(iss_handle* h) {
    if (h->cuda_ready) return ISS_OK;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        return fail(h, ISS_ERR_CUDA, "no CUDA device available (%s)",
                    e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    }
    CUDA_TRY(h, cudaGetDevice(&h->device));
    CUDA_TRY(h, cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (auto& ev : h->ev) CUDA_TRY(h, cudaEventCreate(&ev));
    h->cuda_ready = true;
    return ISS_OK;
}

bool need(iss_handle* h, const char* key, double* v) {
    if (h->params.get(key, v)) return true;
    h->last_error = std::string("parameter with name ") + key + " not found";
    return false;
}

iss_status load_species(iss_handle* h) {
    std::string err;
    std::vector<int32_t> missing;
    if (!load_chosen_species(h->particle_table_path, h->afterburner, h->quantum_statistics,
                             &h->species, &missing, &err)) {
        return fail(h, ISS_ERR_IO, "%s", err.c_str());
    }
    if (!load_resonances(h->particle_table_path, h->afterburner, h->quantum_statistics,
                         &h->resonances, &err)) {
        return fail(h, ISS_ERR_IO, "%s", err.c_str());
    }
    h->species_afterburner = h->afterburner;
    h->species_qs = h->quantum_statistics;
    return ISS_OK;
}

iss_status finish_surface(iss_handle* h) {
    h->n_cells = static_cast<int64_t>(h->fo34.size() / kFoSurfFloats);
    if (h->n_cells == 0) return fail(h, ISS_ERR_NO_SURFACE, "no freeze-out fluid cell");
    h->surface_loaded = true;
    h->surface_on_device = false;
    h->yields_valid = false;
    h->samples_valid = false;
    h->host_valid = false;
    return ISS_OK;
}

// sample_pT_up_to < 0: the last pT of the reference's gauss pT table
// (src/emissionfunction.cpp:3323-3326 reads it from bin_tables/pT_gauss_table.dat;
// 3.6943142 GeV in the reference's tables when the file is not at table_path)
double sampling_pt_limit(const std::string& table_path) {
    std::ifstream f(table_path + "/bin_tables/pT_gauss_table.dat");
    double last = 3.6943142, a, b;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        if (ls >> a >> b) last = a;
    }
    return last;
}

// configuration, tables and device buffers for the next generate
iss_status prepare(iss_handle* h) {
    double v;
    if (!need(h, "MC_sampling", &v)) return ISS_ERR_PARAM_MISSING;
    const int mc = static_cast<int>(v);
    if (mc != 4 && mc != 2)
        return fail(h, ISS_ERR_UNSUPPORTED,
                    "MC_sampling = %d: the GPU runs the FSSW sampler (4) and the lab-frame "
                    "EmissionFunctionArray sampler (2)", mc);
    DevConfig c{};
    c.mc_sampling = mc;
    const char* keys[] = {"hydro_mode", "include_deltaf_shear", "include_deltaf_bulk",
                          "bulk_deltaf_kind", "include_deltaf_diffusion",
                          "local_charge_conservation", "number_of_repeated_sampling",
                          "dN_dy_sampling_model", "dN_dy_sampling_para1",
                          "sample_upto_desired_particle_number", "y_LB", "y_RB"};
    double vals[12];
    for (int i = 0; i < 12; i++)
        if (!need(h, keys[i], &vals[i])) return ISS_ERR_PARAM_MISSING;
    c.hydro_mode = static_cast<int>(vals[0]);
    c.include_shear = static_cast<int>(vals[1]) == 1;
    c.include_bulk = static_cast<int>(vals[2]) == 1;
    c.bulk_kind = static_cast<int>(vals[3]);
    c.include_diff = static_cast<int>(vals[4]) == 1;
    c.neos_kind = (c.bulk_kind == 21) ? 1 : (c.bulk_kind == 20 ? 0 : -1);
    c.lcc = static_cast<int>(vals[5]) == 1;
    c.n_events = static_cast<int>(vals[6]);
    c.sampling_model = static_cast<int>(vals[7]);
    c.sampling_para1 = vals[8];
    if (c.sampling_model > 100 ||
        !(c.sampling_model == 1 || c.sampling_model == 10 || c.sampling_model == 20 ||
          c.sampling_model == 30))
        return fail(h, ISS_ERR_UNSUPPORTED, "sampling model %d is not supported", c.sampling_model);
    c.y_lb = static_cast<float>(vals[10]);
    c.y_rb = static_cast<float>(vals[11]);
    c.ymult = (c.hydro_mode != 2) ? (vals[11] - vals[10]) : 1.0;
    // the reference decays unless SMASH is the afterburner (src/FSSW.cpp:346-348)
    h->decays = h->params.get_or("perform_decays", 0) == 1 && h->afterburner != 2;
    if (h->params.get_or("include_spectators", 0) != 0)
        return fail(h, ISS_ERR_UNSUPPORTED, "include_spectators is not supported");
    if (c.n_events < 0) return fail(h, ISS_ERR_INVALID_ARG, "negative number of events");
    c.compat_fermion = static_cast<int>(h->params.get_or("gpu_compat_fermion_cdf2", 0)) != 0;
    c.max_tries = static_cast<int>(h->params.get_or("gpu_max_tries", 10000));
    c.max_redraws = static_cast<int>(h->params.get_or("gpu_max_redraws", 64));
    c.event_offset = static_cast<uint32_t>(h->params.get_or("gpu_event_offset", 0));
    {
        const int smp = static_cast<int>(h->params.get_or("gpu_sampler", 0));
        if (smp != 0 && smp != 1)
            return fail(h, ISS_ERR_UNSUPPORTED, "gpu_sampler = %d (0: plain, 1: learned)", smp);
        h->use_learned = smp == 1;
        const double alpha = h->params.get_or("gpu_learned_alpha", 0.8);
        if (h->use_learned && !(alpha > 0.0 && alpha < 1.0))
            return fail(h, ISS_ERR_INVALID_ARG, "gpu_learned_alpha = %g must lie in (0, 1)", alpha);
        c.lalpha = static_cast<float>(alpha);
        const int exact = static_cast<int>(h->params.get_or("gpu_learned_exact", 1));
        if (exact != 0 && exact != 1)
            return fail(h, ISS_ERR_INVALID_ARG, "gpu_learned_exact = %d (1: exact, 0: pilot envelope)",
                        exact);
        c.lexact = exact;
        c.lslot = nullptr;
        c.lpairs = nullptr;
    }
    if (mc == 2) {
        // sample_using_dN_dxtdy_4all_particles_conventional (src/emissionfunction.cpp:3273-3340)
        if (h->use_learned)
            return fail(h, ISS_ERR_UNSUPPORTED, "gpu_sampler = 1 needs MC_sampling = 4");
        if (c.include_bulk && c.bulk_kind != 1)
            return fail(h, ISS_ERR_UNSUPPORTED,
                        "MC_sampling = 2 with bulk_deltaf_kind = %d (the GPU supports kind 1)",
                        c.bulk_kind);
        double pt, range;
        if (!need(h, "sample_pT_up_to", &pt) || !need(h, "sample_y_minus_eta_s_range", &range))
            return ISS_ERR_PARAM_MISSING;
        if (pt < 0) pt = sampling_pt_limit(h->table_path);
        c.pt_max = static_cast<float>(pt);
        c.yme_range = static_cast<float>(range);
        c.restrict_df = static_cast<int>(h->params.get_or("restrict_deltaf", 1)) == 1;
        c.df_max_ratio = static_cast<float>(h->params.get_or("deltaf_max_ratio", 1.0));
        // the reference gives a cell 4,999 proposals before drawing another
        // (tries = 1 .. maximum_impatience - 1, src/emissionfunction.cpp:4205-4300);
        // at this sampler's acceptance the cap shapes which cells are sampled
        if (!h->params.has("gpu_max_tries")) c.max_tries = 4999;
    }
    c.item_size = h->tune.item_size;
    c.yield_groups = h->tune.yield_groups;
    c.sampler_ctas = h->tune.sampler_ctas;
    c.assign_bps = h->tune.assign_blocks;
    c.key0 = static_cast<uint32_t>(static_cast<uint64_t>(h->seed));
    c.key1 = static_cast<uint32_t>(static_cast<uint64_t>(h->seed) >> 32);
    c.n_species = static_cast<int>(h->species.size());
    c.n_cells = h->n_cells;
    // surfaces of the batch and the layout of their CDF rows
    {
        std::vector<int64_t> cells = h->batch_cells;
        std::vector<int32_t> events = h->batch_events;
        if (cells.empty()) {
            cells = {0, h->n_cells};
            events = {c.n_events};
        } else if (h->params.get_or("sample_upto_desired_particle_number", 0) == 1) {
            return fail(h, ISS_ERR_UNSUPPORTED,
                        "sample_upto_desired_particle_number with a batch of surfaces");
        }
        const int B = static_cast<int>(events.size());
        const int S = c.n_species;
        h->segs.assign(static_cast<size_t>(B), SurfSeg{});
        int64_t cdf = 0, guide = 0, tiles = 0;
        int e0 = 0;
        for (int b = 0; b < B; b++) {
            SurfSeg& g = h->segs[b];
            g.c0 = cells[b];
            g.n = cells[b + 1] - cells[b];
            g.L = cdf_log2_cells(g.n);
            g.g = cdf_guide_bits(g.n);
            g.nt = cdf_num_tiles(g.n);
            g.cdf_base = cdf;
            g.guide_base = guide;
            g.tile_base = tiles;
            g.e0 = e0;
            g.ne = events[b];
            cdf += static_cast<int64_t>(S) * (g.n + 1);
            guide += static_cast<int64_t>(S) * ((int64_t(1) << g.g) + 1);
            tiles += static_cast<int64_t>(S) * g.nt;
            e0 += events[b];
        }
        h->cdf_len = cdf;
        h->guide_len = guide;
        h->n_tiles = tiles;
        c.n_surfaces = B;
        c.n_events = e0;
        CUDA_TRY(h, h->d_surf.reserve(static_cast<size_t>(B)));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_surf.ptr, h->segs.data(), sizeof(SurfSeg) * B,
                                    cudaMemcpyHostToDevice, h->stream));
        c.surf = h->d_surf.ptr;
    }
    const int fix_c0 = static_cast<int>(h->params.get_or("gpu_fix_14mom_c0", 0)) != 0;

    // tables
    TableKey key{h->table_path, h->afterburner, c.bulk_kind, c.include_bulk, c.include_diff,
                 c.neos_kind, fix_c0};
    if (!(key == h->table_key)) {
        std::string err;
        std::vector<double> K, E;
        special_function_tables(c.include_bulk != 0, c.include_diff != 0, &K, &E);
        std::vector<float4> K4(kSfLen);
        for (int i = 0; i < kSfLen; i++)
            K4[i] = make_float4(static_cast<float>(K[3 * i]), static_cast<float>(K[3 * i + 1]),
                                static_cast<float>(K[3 * i + 2]), 0.0f);
        CUDA_TRY(h, h->d_sfK.reserve(kSfLen));
        CUDA_TRY(h, cudaMemcpy(h->d_sfK.ptr, K4.data(), sizeof(float4) * kSfLen,
                               cudaMemcpyHostToDevice));
        if (c.include_diff) {
            std::vector<float> E32(E.begin(), E.end());
            CUDA_TRY(h, h->d_sfE.reserve(E32.size()));
            CUDA_TRY(h, cudaMemcpy(h->d_sfE.ptr, E32.data(), sizeof(float) * E32.size(),
                                   cudaMemcpyHostToDevice));
        }
        if (c.include_bulk && c.bulk_kind == 11) {
            if (!load_bulk14(h->table_path, h->afterburner, fix_c0 != 0, &h->b14, &err))
                return fail(h, ISS_ERR_IO, "%s", err.c_str());
            const size_t n = h->b14.c1.size();
            CUDA_TRY(h, h->d_b14c0.reserve(n));
            CUDA_TRY(h, h->d_b14c1.reserve(n));
            CUDA_TRY(h, h->d_b14c2.reserve(n));
            CUDA_TRY(h, cudaMemcpy(h->d_b14c0.ptr, h->b14.c0.data(), 8 * n, cudaMemcpyHostToDevice));
            CUDA_TRY(h, cudaMemcpy(h->d_b14c1.ptr, h->b14.c1.data(), 8 * n, cudaMemcpyHostToDevice));
            CUDA_TRY(h, cudaMemcpy(h->d_b14c2.ptr, h->b14.c2.data(), 8 * n, cudaMemcpyHostToDevice));
        }
        if (c.neos_kind == 0) {
            return fail(h, ISS_ERR_IO, "can not find file %s/deltaf_tables/%s/NEoSBQS_22mom_deltafCoeff.dat",
                        h->table_path.c_str(), h->afterburner == 2 ? "smash" : "urqmd");
        }
        if (c.neos_kind == 1) {
            std::vector<double> ce;
            if (!load_ce_neos(h->table_path, h->afterburner, &ce, &err))
                return fail(h, ISS_ERR_IO, "%s", err.c_str());
            CUDA_TRY(h, h->d_ce.reserve(ce.size()));
            CUDA_TRY(h, cudaMemcpy(h->d_ce.ptr, ce.data(), 8 * ce.size(), cudaMemcpyHostToDevice));
        }
        if (c.include_diff) {
            std::vector<double> q;
            if (!load_qmu_coeff(h->table_path, &q, &err)) return fail(h, ISS_ERR_IO, "%s", err.c_str());
            CUDA_TRY(h, h->d_qmu.reserve(q.size()));
            CUDA_TRY(h, cudaMemcpy(h->d_qmu.ptr, q.data(), 8 * q.size(), cudaMemcpyHostToDevice));
        }
        h->table_key = key;
    }
    if (!h->d_logfact.ptr) {
        // log(k!) for k < 256, from the C library's lgamma (Poisson draws)
        std::vector<double> lf(kLogFactLen);
        for (int i = 0; i < kLogFactLen; i++) lf[i] = std::lgamma(i + 1.0);
        CUDA_TRY(h, h->d_logfact.reserve(kLogFactLen));
        CUDA_TRY(h, cudaMemcpy(h->d_logfact.ptr, lf.data(), sizeof(double) * kLogFactLen,
                               cudaMemcpyHostToDevice));
    }
    c.tab.logfact = h->d_logfact.ptr;
    c.tab.sfK = h->d_sfK.ptr;
    c.tab.sfE = h->d_sfE.ptr;
    c.tab.b14c0 = h->d_b14c0.ptr;
    c.tab.b14c1 = h->d_b14c1.ptr;
    c.tab.b14c2 = h->d_b14c2.ptr;
    c.tab.b14_nT = h->b14.nT;
    c.tab.b14_nmu = h->b14.nmu;
    c.tab.b14_T0 = h->b14.T0;
    c.tab.b14_mu0 = h->b14.mu0;
    c.tab.b14_dT = h->b14.dT;
    c.tab.b14_dmu = h->b14.dmu;
    c.tab.ce = h->d_ce.ptr;
    c.tab.qmu = h->d_qmu.ptr;

    // species
    std::vector<SpeciesDev> sd(h->species.size());
    std::vector<int32_t> pids(h->species.size());
    for (size_t k = 0; k < sd.size(); k++) {
        const Species& s = h->species[k];
        sd[k].m_hi = static_cast<float>(s.mass);
        sd[k].m_lo = static_cast<float>(s.mass - static_cast<double>(sd[k].m_hi));
        sd[k].degen = static_cast<float>(s.gspin);
        sd[k].light = s.mass < 0.7 ? 1 : 0;
        sd[k].baryon = s.baryon;
        sd[k].strange = s.strange;
        sd[k].charge = s.charge;
        sd[k].sign = s.sign;
        pids[k] = s.pid;
    }
    // species whose thermal series are the same function of the cell
    // (same float-float mass, statistics and number of terms) form one group
    // of the yields kernel; the series runs once per group and cell whenever
    // the members' chemical potentials agree in that cell
    const std::vector<int32_t> yorder = yield_group_order(sd);
    c.n_ygroups = static_cast<int>(yorder.size() - sd.size()) - 1;
    CUDA_TRY(h, h->d_species.reserve(sd.size()));
    CUDA_TRY(h, h->d_pids.reserve(sd.size()));
    CUDA_TRY(h, h->d_yorder.reserve(yorder.size()));
    c.yorder = h->d_yorder.ptr;
    if (!sd.empty()) {
        CUDA_TRY(h, cudaMemcpyAsync(h->d_species.ptr, sd.data(), sizeof(SpeciesDev) * sd.size(),
                                    cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_pids.ptr, pids.data(), 4 * pids.size(),
                                    cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_yorder.ptr, yorder.data(), 4 * yorder.size(),
                                    cudaMemcpyHostToDevice, h->stream));
    }
    h->cfg = c;
    return ISS_OK;
}

CellArrays cell_arrays(iss_handle* h) {
    CellArrays a;
    float4* b = h->d_cells.ptr;
    const int64_t n = h->n_cells;
    a.pos = b;
    a.da = b + n;
    a.u = b + 2 * n;
    a.th = b + 3 * n;
    a.th2 = b + 4 * n;
    a.pi1 = b + 5 * n;
    a.pi2 = b + 6 * n;
    a.coef = b + 7 * n;
    a.rec = b + 8 * n;   // 128-byte records, 128-byte aligned
    a.srec = b + 16 * n;  // the lean sampler's 128-byte records
    a.milne = h->cfg.mc_sampling == 2 ? h->d_milne.ptr : nullptr;
    return a;
}

// surface upload + prologue + yields + CDF (the per-cell half of generate)
iss_status run_cells(iss_handle* h) {
    const int64_t n = h->n_cells;
    const int S = static_cast<int>(h->species.size());
    DevConfig& c = h->cfg;
    cudaStream_t st = h->stream;
    if (!h->surface_on_device) {
        CUDA_TRY(h, h->d_fo34.reserve(static_cast<size_t>(n) * kFoSurfFloats));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_fo34.ptr, h->fo34.data(),
                                    sizeof(float) * static_cast<size_t>(n) * kFoSurfFloats,
                                    cudaMemcpyHostToDevice, st));
        h->surface_on_device = true;
    }
    // 8 SoA arrays, the records and the lean sampler's records
    CUDA_TRY(h, h->d_cells.reserve(static_cast<size_t>(n) * 24));
    if (c.mc_sampling == 2) CUDA_TRY(h, h->d_milne.reserve(static_cast<size_t>(n) * 6));
    CUDA_TRY(h, h->d_yields.reserve(static_cast<size_t>(n) * S));
    const size_t rows = static_cast<size_t>(c.n_surfaces) * S;
    CUDA_TRY(h, h->d_cdf.reserve(static_cast<size_t>(std::max<int64_t>(h->cdf_len, 1))));
    CUDA_TRY(h, h->d_tile_sum.reserve(static_cast<size_t>(std::max<int64_t>(h->n_tiles, 1))));
    CUDA_TRY(h, h->d_tile_off.reserve(static_cast<size_t>(std::max<int64_t>(h->n_tiles, 1))));
    CUDA_TRY(h, h->d_totals.reserve(rows));
    CUDA_TRY(h, h->d_qtot.reserve(rows));
    CUDA_TRY(h, h->d_ymax.reserve(rows));
    CUDA_TRY(h, h->d_guide.reserve(static_cast<size_t>(std::max<int64_t>(h->guide_len, 1))));
    const CellArrays cells = cell_arrays(h);
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvStart], st));
    CUDA_TRY(h, launch_cell_prologue(c, h->d_fo34.ptr, n, cells, st));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvPrologue], st));
    CUDA_TRY(h, launch_yields(c, cells, h->d_species.ptr, h->d_yields.ptr, h->d_ymax.ptr, st));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvYields], st));
    CUDA_TRY(h, launch_cdf(h->d_yields.ptr, n, h->d_surf.ptr, c.n_surfaces, h->n_tiles, S,
                           h->d_ymax.ptr, h->d_tile_sum.ptr, h->d_tile_off.ptr, h->d_qtot.ptr,
                           h->d_totals.ptr, h->d_cdf.ptr, h->d_guide.ptr, st));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvCdf], st));
    h->yields_valid = true;
    return ISS_OK;
}

float elapsed(iss_handle* h, int a, int b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[a], h->ev[b]);
    return ms;
}

// Resonance decays of the sampled records, generation by generation over
// all events (kernels_decay.cu); replaces d_hadrons and the event offsets
// with the final-state lists.  The count sweep runs on the device in batches
// of kDecayBatch generations with one host wait per batch (the sizes stay on
// the device); the layout and the write sweep follow, then one wait for the
// event offsets.  A generation whose products do not fit a buffer ends the
// count sweep with a flag; the call then reruns the sweep with buffers sized
// from what it needed (same results).  The work buffers stay allocated in the
// handle for later calls.
constexpr int kDecayBatch = 8;

iss_status run_decays(iss_handle* h, unsigned long long* failures_out) {
    DevConfig& c = h->cfg;
    cudaStream_t s = h->stream;
    const int E = c.n_events;
    if (h->decay_table_afterburner != h->afterburner) {
        DecayTable tab;
        std::string err;
        if (!load_decay_table(h->particle_table_path, h->afterburner, &tab, &err))
            return fail(h, ISS_ERR_IO, "%s", err.c_str());
        const int n = static_cast<int>(tab.particles.size());
        // the per-hadron channel cache packs (particle << 16) | channel
        if (n >= 32768 || tab.channels.size() >= 65536)
            return fail(h, ISS_ERR_UNSUPPORTED, "decay table too large (%d particles, %zu channels)", n,
                        tab.channels.size());
        std::vector<std::pair<int32_t, int32_t>> by_pid;
        for (int i = 0; i < n; i++) by_pid.push_back({tab.particles[i].pid, i});
        // first entry of a repeated pid wins, as in the reference's lookups
        std::stable_sort(by_pid.begin(), by_pid.end(),
                         [](const std::pair<int32_t, int32_t>& a, const std::pair<int32_t, int32_t>& b) {
                             return a.first < b.first;
                         });
        by_pid.erase(std::unique(by_pid.begin(), by_pid.end(),
                                 [](const std::pair<int32_t, int32_t>& a,
                                    const std::pair<int32_t, int32_t>& b) { return a.first == b.first; }),
                     by_pid.end());
        std::vector<int32_t> sorted(2 * by_pid.size());
        for (size_t i = 0; i < by_pid.size(); i++) {
            sorted[i] = by_pid[i].first;
            sorted[by_pid.size() + i] = by_pid[i].second;
        }
        CUDA_TRY(h, h->d_dparticles.reserve(tab.particles.size()));
        CUDA_TRY(h, h->d_dchannels.reserve(std::max<size_t>(tab.channels.size(), 1)));
        CUDA_TRY(h, h->d_dsorted.reserve(sorted.size()));
        CUDA_TRY(h, cudaMemcpy(h->d_dparticles.ptr, tab.particles.data(),
                               sizeof(DecayParticle) * tab.particles.size(), cudaMemcpyHostToDevice));
        if (!tab.channels.empty())
            CUDA_TRY(h, cudaMemcpy(h->d_dchannels.ptr, tab.channels.data(),
                                   sizeof(DecayChannel) * tab.channels.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(h, cudaMemcpy(h->d_dsorted.ptr, sorted.data(), 4 * sorted.size(),
                               cudaMemcpyHostToDevice));
        h->n_decay_particles = static_cast<int>(by_pid.size());
        // open-addressing hash of the first index of every pid (linear probing)
        if (by_pid.size() * 2 > static_cast<size_t>(kDecayHash))
            return fail(h, ISS_ERR_UNSUPPORTED, "decay table has %zu particles", by_pid.size());
        std::vector<int2> hash(static_cast<size_t>(kDecayHash), int2{0, -1});
        for (const auto& pi : by_pid) {
            if (pi.first == 0) continue;
            uint32_t j = decay_hash(pi.first);
            while (hash[j].x != 0) j = (j + 1) & (kDecayHash - 1);
            hash[j] = int2{pi.first, pi.second};
        }
        CUDA_TRY(h, h->d_dhash.reserve(hash.size()));
        CUDA_TRY(h, cudaMemcpy(h->d_dhash.ptr, hash.data(), sizeof(int2) * hash.size(),
                               cudaMemcpyHostToDevice));
        h->decay_table_afterburner = h->afterburner;
    }
    DecayTablesDev t;
    t.particles = h->d_dparticles.ptr;
    t.channels = h->d_dchannels.ptr;
    t.sorted_pid = h->d_dsorted.ptr;
    t.sorted_idx = h->d_dsorted.ptr + h->n_decay_particles;
    t.hash = h->d_dhash.ptr;
    t.n_particles = h->n_decay_particles;

    const int64_t n0 = h->n_hadrons;
    h->dk_reruns = 0;
    if (n0 <= 0 || E <= 0) {
        *failures_out = 0;
        return ISS_OK;
    }
    const int G = kDecayMaxGenerations;
    // first sizes: what the last call needed, else gpu_decay_arena_factor
    // (default 2.0) times the sampled hadrons for the final lists,
    // gpu_decay_next_factor (0.5) for one generation's records and the
    // sampled hadrons plus twice that for the inputs of all generations; too
    // small only costs a rerun of the count sweep
    const double fa = h->params.get_or("gpu_decay_arena_factor", 2.0);
    const double fu = h->params.get_or("gpu_decay_next_factor", 0.5);
    if (!(fa > 0.0) || !(fu > 0.0))
        return fail(h, ISS_ERR_INVALID_ARG, "gpu_decay_arena_factor / gpu_decay_next_factor must be > 0");
    int64_t s_cap = std::max<int64_t>(h->dk_scap_hint, static_cast<int64_t>(fa * static_cast<double>(n0)) + 64);
    int64_t u_cap = std::max<int64_t>(h->dk_ucap_hint, static_cast<int64_t>(fu * static_cast<double>(n0)) + 64);
    int64_t i_cap = std::max<int64_t>(h->dk_icap_hint, n0 + 2 * u_cap);
    std::vector<int64_t> meta_h(kDecayMetaLen, 0);
    // the scans add (stable << 32 | unstable) counts of at most 3 each: the
    // unstable half stays below 2^32 while a generation has < 2^32 / 3 inputs
    constexpr int64_t kMaxDecayInputs = (int64_t(1) << 32) / 3 - 1;
    if (n0 > kMaxDecayInputs)
        return fail(h, ISS_ERR_UNSUPPORTED, "resonance decays of more than %lld sampled hadrons",
                    static_cast<long long>(kMaxDecayInputs));
    const size_t GE = static_cast<size_t>(G) * static_cast<size_t>(E);
    for (int attempt = 0;; attempt++) {
        u_cap = std::min(u_cap, kMaxDecayInputs);
        i_cap = std::max(i_cap, n0);
        const int64_t gen_cap = std::max(n0, u_cap);
        for (int k = 0; k < 2; k++) CUDA_TRY(h, h->dk_u[k].reserve(static_cast<size_t>(u_cap)));
        CUDA_TRY(h, h->dk_final.reserve(static_cast<size_t>(s_cap)));
        CUDA_TRY(h, h->dk_ev.reserve(static_cast<size_t>(i_cap)));
        CUDA_TRY(h, h->dk_pid.reserve(static_cast<size_t>(i_cap)));
        CUDA_TRY(h, h->dk_chan.reserve(static_cast<size_t>(i_cap)));
        CUDA_TRY(h, h->dk_coff.reserve(static_cast<size_t>(i_cap) + G + 1));
        CUDA_TRY(h, h->dk_cnt.reserve(static_cast<size_t>(gen_cap)));
        CUDA_TRY(h, h->dk_tiles.reserve(static_cast<size_t>(gen_cap / 4096 + 1)));
        CUDA_TRY(h, h->dk_first.reserve(GE));
        CUDA_TRY(h, h->dk_last.reserve(GE));
        CUDA_TRY(h, h->dk_scnt.reserve(GE));
        CUDA_TRY(h, h->dk_shift.reserve(GE));
        CUDA_TRY(h, h->dk_meta.reserve(kDecayMetaLen));
        CUDA_TRY(h, h->dk_off.reserve(static_cast<size_t>(E) + 1));
        CUDA_TRY(h, h->dk_evoff.reserve(static_cast<size_t>(E) + 1));
        CUDA_TRY(h, h->dk_etot.reserve(static_cast<size_t>(E)));
        CUDA_TRY(h, h->dk_etiles.reserve(static_cast<size_t>(std::max(offsets_num_tiles(E), 1))));
        CUDA_TRY(h, h->dk_fail.reserve(1));

        std::fill(meta_h.begin(), meta_h.end(), 0);
        meta_h[kDecayMetaNIn] = n0;
        CUDA_TRY(h, cudaMemcpyAsync(h->dk_meta.ptr, meta_h.data(), 8 * meta_h.size(),
                                    cudaMemcpyHostToDevice, s));
        CUDA_TRY(h, cudaMemsetAsync(h->dk_first.ptr, 0xFF, 8 * GE, s));
        CUDA_TRY(h, cudaMemsetAsync(h->dk_last.ptr, 0xFF, 8 * GE, s));
        CUDA_TRY(h, cudaMemsetAsync(h->dk_fail.ptr, 0, sizeof(unsigned long long), s));
        CUDA_TRY(h, cudaMemcpyAsync(h->dk_evoff.ptr, h->event_offsets.data(), 8 * (static_cast<size_t>(E) + 1),
                                    cudaMemcpyHostToDevice, s));

        DecayBuffers b{};
        b.rec0 = h->d_hadrons.ptr;
        b.ev = h->dk_ev.ptr;
        b.pid = h->dk_pid.ptr;
        b.chan = h->dk_chan.ptr;
        b.cnt = h->dk_cnt.ptr;
        b.off = h->dk_coff.ptr;
        b.tiles = h->dk_tiles.ptr;
        b.first = h->dk_first.ptr;
        b.last = h->dk_last.ptr;
        b.scnt = h->dk_scnt.ptr;
        b.shift = h->dk_shift.ptr;
        b.meta = h->dk_meta.ptr;
        b.failures = h->dk_fail.ptr;
        b.s_cap = s_cap;
        b.u_cap = u_cap;
        b.i_cap = i_cap;
        b.g_max = static_cast<uint32_t>(G);
        CUDA_TRY(h, launch_decay_first_generation(h->dk_evoff.ptr, E, b, s));
        // count sweep: batches of generations, one wait (and a copy of the
        // sizes) per batch; the first batch has as many generations as the
        // last call had, so that a repeated workload waits once
        int g = 0;
        int batch = h->dk_gen_hint > 0 ? std::min(h->dk_gen_hint, kDecayBatch) : kDecayBatch;
        for (;;) {
            for (int k = 0; k < batch && g < G; k++, g++)
                CUDA_TRY(h, launch_decay_count_generation(c, t, static_cast<uint32_t>(g), b, E, h->num_sms, s));
            batch = kDecayBatch;
            CUDA_TRY(h, cudaMemcpyAsync(meta_h.data(), h->dk_meta.ptr, 8 * meta_h.size(),
                                        cudaMemcpyDeviceToHost, s));
            CUDA_TRY(h, cudaStreamSynchronize(s));
            if (meta_h[kDecayMetaFlags] != 0 || meta_h[kDecayMetaNIn + g] == 0 || g >= G) break;
        }
        const int64_t flags = meta_h[kDecayMetaFlags];
        if (flags & 4)
            return fail(h, ISS_ERR_SAMPLING, "decay chains longer than %d generations", G);
        if (flags & 11) {
            if (attempt >= 8) return fail(h, ISS_ERR_CUDA, "decay buffers did not settle");
            h->dk_reruns++;
            if (flags & 1) s_cap = std::max(s_cap * 2, meta_h[kDecayMetaNeedS] + meta_h[kDecayMetaNeedS] / 4);
            if (flags & 2) u_cap = std::max(u_cap * 2, meta_h[kDecayMetaNeedU] + meta_h[kDecayMetaNeedU] / 4);
            if (flags & 8) i_cap = std::max(i_cap * 2, meta_h[kDecayMetaNeedI] + meta_h[kDecayMetaNeedI] / 4);
            continue;
        }
        // generations with inputs: 0 .. n_gen - 1
        int n_gen = 0;
        while (n_gen < g && meta_h[kDecayMetaNIn + n_gen] > 0) n_gen++;
        const int64_t total = meta_h[kDecayMetaSBase + n_gen];
        CUDA_TRY(h, launch_decay_layout(b, n_gen, E, h->dk_etot.ptr, h->dk_etiles.ptr, h->dk_off.ptr, s));
        // write sweep
        for (int k = 0; k < n_gen; k++) {
            const HadronRec* in = k == 0 ? h->d_hadrons.ptr : h->dk_u[(k - 1) & 1].ptr;
            CUDA_TRY(h, launch_decay_write_generation(c, t, static_cast<uint32_t>(k), meta_h[kDecayMetaNIn + k],
                                                      meta_h[kDecayMetaIBase + k], in, h->dk_u[k & 1].ptr, b, E,
                                                      h->num_sms, h->dk_final.ptr, s));
        }
        h->event_offsets.assign(static_cast<size_t>(E) + 1, 0);
        unsigned long long nf = 0;
        CUDA_TRY(h, cudaMemcpyAsync(h->event_offsets.data(), h->dk_off.ptr, 8 * (static_cast<size_t>(E) + 1),
                                    cudaMemcpyDeviceToHost, s));
        CUDA_TRY(h, cudaMemcpyAsync(&nf, h->dk_fail.ptr, sizeof(nf), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(h, cudaStreamSynchronize(s));
        if (h->event_offsets[E] != total)
            return fail(h, ISS_ERR_CUDA, "decay lists disagree (%lld vs %lld hadrons)",
                        static_cast<long long>(h->event_offsets[E]), static_cast<long long>(total));
        *failures_out = nf;
        // sizes for the next call: what this one needed, with headroom
        const int64_t inputs = meta_h[kDecayMetaIBase + n_gen];
        h->dk_scap_hint = std::max(h->dk_scap_hint, total + total / 8 + 4096);
        h->dk_ucap_hint = std::max(h->dk_ucap_hint, meta_h[kDecayMetaMaxU] + meta_h[kDecayMetaMaxU] / 8 + 4096);
        h->dk_icap_hint = std::max(h->dk_icap_hint, inputs + inputs / 8 + 4096);
        h->dk_gen_hint = n_gen;
        std::swap(h->dk_final.ptr, h->d_hadrons.ptr);
        std::swap(h->dk_final.cap, h->d_hadrons.cap);
        h->n_hadrons = total;
        return ISS_OK;
    }
}

// host_out != nullptr: iss_gpu_generate_into -- the sampler runs in chunks of
// consecutive events and each chunk's records are copied to host_out on a
// second stream while the next chunk is sampled.

// Learned proposal of one generate: the species whose expected hadrons per
// cell (over all events) reach gpu_learned_min_hadrons_per_cell, the network
// on every (species, cell) pair of them, and the pairs' mixture records and
// envelope constants.  Sets cfg.lslot / lpairs for the sampler.
iss_status run_learned_pairs(iss_handle* h) {
    DevConfig& c = h->cfg;
    const int S = c.n_species;
    cudaStream_t s = h->stream;
    if (!h->learned.have_weights)
        return fail(h, ISS_ERR_NO_SAMPLES,
                    "gpu_sampler = 1 needs network weights (iss_gpu_learned_train or "
                    "iss_gpu_learned_set_weights)");
    const double thr = h->params.get_or("gpu_learned_min_hadrons_per_cell", 1.0);
    // pilot proposals per pair: in exact mode M only trades the network's
    // share of the tries against the excess branch's (the output is the
    // target for every M), and few pilots measured fastest (4: 15.3 ms per
    // step on the 200k-cell surface, 64: 23.9 ms); the pilot-envelope mode
    // needs M close to the true sup, so it keeps 64
    const int n_pilot = static_cast<int>(h->params.get_or("gpu_learned_pilot", c.lexact ? 4 : 64));
    const float safety = static_cast<float>(h->params.get_or("gpu_learned_safety", 1.15));
    if (n_pilot < 1 || n_pilot > 4096 || !(safety >= 1.0f))
        return fail(h, ISS_ERR_INVALID_ARG, "gpu_learned_pilot = %d, gpu_learned_safety = %g", n_pilot,
                    static_cast<double>(safety));
    std::vector<int32_t> slot(static_cast<size_t>(S), -1), lspecies;
    for (int k = 0; k < S; k++) {
        double n = 0.0;
        for (int b = 0; b < c.n_surfaces; b++)
            n += h->totals[static_cast<size_t>(b) * S + k] * c.ymult * h->segs[b].ne;
        if (n >= thr * static_cast<double>(c.n_cells)) {
            slot[k] = static_cast<int32_t>(lspecies.size());
            lspecies.push_back(k);
        }
    }
    const int n_slots = static_cast<int>(lspecies.size());
    const int64_t n_pairs = static_cast<int64_t>(n_slots) * c.n_cells;
    h->lstats.n_species = n_slots;
    h->lstats.n_pairs = n_pairs;
    CUDA_TRY(h, h->d_lslot.reserve(static_cast<size_t>(std::max(S, 1))));
    CUDA_TRY(h, h->d_lspecies.reserve(static_cast<size_t>(std::max(n_slots, 1))));
    CUDA_TRY(h, cudaMemcpyAsync(h->d_lslot.ptr, slot.data(), 4 * slot.size(), cudaMemcpyHostToDevice, s));
    if (n_slots > 0)
        CUDA_TRY(h, cudaMemcpyAsync(h->d_lspecies.ptr, lspecies.data(), 4 * lspecies.size(),
                                    cudaMemcpyHostToDevice, s));
    Learned& L = h->learned;
    CUDA_TRY(h, L.x.reserve(static_cast<size_t>(std::max<int64_t>(n_pairs, 1)) * mlp::kIn0));
    CUDA_TRY(h, h->d_lpairs.reserve(static_cast<size_t>(std::max<int64_t>(n_pairs, 1)) * kPairFloats));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvLearnStart], s));
    const CellArrays cells = cell_arrays(h);
    CUDA_TRY(h, launch_learned_pairs(c, cells, h->d_species.ptr, h->d_lspecies.ptr, n_slots, L.x.ptr, s));
    CUDA_TRY(h, cudaMemsetAsync(L.err.ptr, 0, sizeof(int), s));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvFwdStart], s));
    CUDA_TRY(h, launch_mlp_forward(L.img.ptr, L.params.ptr, L.x.ptr, n_pairs, nullptr, nullptr,
                                   L.err.ptr, h->num_sms, s, h->d_lpairs.ptr));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvFwdEnd], s));
    c.lslot = h->d_lslot.ptr;
    c.lpairs = h->d_lpairs.ptr;
    CUDA_TRY(h, launch_learned_envelopes(c, cells, h->d_species.ptr, h->d_lspecies.ptr, n_slots,
                                         n_pilot, safety, h->d_lpairs.ptr, s));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvLearnEnd], s));
    return ISS_OK;
}

// ---------------------------------------------------------------------------
// Graph replay of a generate (gpu_graph = 1).  The first eligible call runs
// eagerly, then captures the whole device sequence of a generate -- cell
// prologue, yields, CDF, counts, slot scans, the bound check, item map, cell
// assignment, sampler and the copies of the sizes, counters and event
// offsets into pinned host memory -- as one CUDA graph.  Later calls of the
// same shape upload their seed and event offset (12 bytes, read by the
// kernels through DevConfig::run), launch the graph and wait once.  The
// graph's buffers have 15 % headroom over the captured call; a call whose
// draws do not fit samples nothing (graph_limits_kernel) and runs eagerly.

bool graph_eligible(iss_handle* h, const iss_hadron_t* host_out, bool streamed = false) {
    return h->params.get_or("gpu_graph", 0) == 1 && !h->graph_unavailable && host_out == nullptr &&
           !streamed &&
           !h->decays &&
           !h->use_learned && h->params.get_or("sample_upto_desired_particle_number", 0) != 1;
}

void drop_graph(iss_handle* h) {
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
    h->graph_key.clear();
}

// everything a captured generate depends on besides the seed and event offset
std::vector<unsigned char> graph_key_of(iss_handle* h) {
    DevConfig c = h->cfg;
    c.key0 = c.key1 = 0;
    c.event_offset = 0;
    c.run = h->d_run.ptr;
    c.ev_surf = h->d_ev_surf.ptr;
    c.chunk_events = std::max(c.n_events, 1);
    std::vector<unsigned char> k(sizeof(c));
    std::memcpy(k.data(), &c, sizeof(c));
    const void* ptrs[] = {h->d_fo34.ptr,     h->d_cells.ptr,    h->d_yields.ptr,   h->d_cdf.ptr,
                          h->d_tile_sum.ptr, h->d_tile_off.ptr, h->d_qtot.ptr,     h->d_totals.ptr,
                          h->d_ymax.ptr,     h->d_guide.ptr,    h->d_counts.ptr,   h->d_items.ptr,
                          h->d_offsets.ptr,  h->d_off_tiles.ptr, h->d_item_off.ptr, h->d_item_seg.ptr,
                          h->d_hadrons.ptr,  h->d_cell_of.ptr,  h->d_work.ptr,     h->d_counters.ptr,
                          h->d_error.ptr,    h->d_pois.ptr,     h->d_species.ptr,  h->d_pids.ptr,
                          h->d_surf.ptr,     h->d_limits.ptr,   h->gh,            h->d_milne.ptr};
    const unsigned char* pb = reinterpret_cast<const unsigned char*>(ptrs);
    k.insert(k.end(), pb, pb + sizeof(ptrs));
    const int64_t nums[] = {h->n_cells, h->n_tiles, h->cdf_len, h->guide_len, h->graph_cap_units,
                            h->graph_cap_items, h->num_sms, static_cast<int64_t>(h->gh_events)};
    const unsigned char* nb = reinterpret_cast<const unsigned char*>(nums);
    k.insert(k.end(), nb, nb + sizeof(nums));
    const unsigned char* tb = reinterpret_cast<const unsigned char*>(&h->tune);
    k.insert(k.end(), tb, tb + sizeof(h->tune));
    return k;
}

void record(iss_handle* h, int ev, bool capturing) {
    if (capturing)
        cudaEventRecordWithFlags(h->ev[ev], h->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(h->ev[ev], h->stream);
}

// The device sequence of one generate, with device-side sizes (no host
// sync).  The counts need only the per-species totals, which the CDF's tile
// offsets give, so they run on a second branch beside the CDF scan; the
// sampler waits for both.  kEvCounts then marks the join: the counts phase
// reports the part of the counts the scan did not cover.
cudaError_t enqueue_generate(iss_handle* h, const DevConfig& c) {
    cudaStream_t s = h->stream;
    cudaStream_t a = h->aux_stream;
    const int64_t n = h->n_cells;
    const int S = c.n_species;
    const int64_t nseg = static_cast<int64_t>(c.n_events) * S;
    const CellArrays cells = cell_arrays(h);
    cudaError_t e;
#define GTRY(call)                      \
    if ((e = (call)) != cudaSuccess) {  \
        return e;                       \
    }
    record(h, kEvStart, true);
    GTRY(launch_cell_prologue(c, h->d_fo34.ptr, n, cells, s));
    record(h, kEvPrologue, true);
    GTRY(launch_yields(c, cells, h->d_species.ptr, h->d_yields.ptr, h->d_ymax.ptr, s));
    record(h, kEvYields, true);
    GTRY(launch_cdf_head(h->d_yields.ptr, n, h->d_surf.ptr, c.n_surfaces, h->n_tiles, S, h->d_ymax.ptr,
                         h->d_tile_sum.ptr, h->d_tile_off.ptr, h->d_qtot.ptr, h->d_totals.ptr, h->d_cdf.ptr,
                         h->d_guide.ptr, s));
    GTRY(cudaEventRecord(h->ev_fork, s));
    GTRY(cudaStreamWaitEvent(a, h->ev_fork, 0));
    GTRY(cudaMemsetAsync(h->d_error.ptr, 0, sizeof(int), a));
    GTRY(launch_counts(c, h->d_species.ptr, h->d_totals.ptr, h->d_pois.ptr, h->d_counts.ptr,
                       h->d_items.ptr, h->d_error.ptr, a));
    GTRY(launch_offsets_scan(h->d_counts.ptr, nseg, h->d_off_tiles.ptr, h->d_offsets.ptr, a));
    GTRY(launch_offsets_scan(h->d_items.ptr, nseg, h->d_off_tiles.ptr, h->d_item_off.ptr, a));
    GTRY(launch_graph_limits(h->d_offsets.ptr, h->d_item_off.ptr, nseg, h->graph_cap_units,
                             h->graph_cap_items, h->d_limits.ptr, a));
    GTRY(launch_item_map(h->d_items.ptr, h->d_item_off.ptr, nseg, h->d_item_seg.ptr, a, h->d_limits.ptr));
    GTRY(cudaEventRecord(h->ev_join, a));
    GTRY(launch_cdf_scan(h->d_yields.ptr, n, h->d_surf.ptr, c.n_surfaces, h->n_tiles, S, h->d_ymax.ptr,
                         h->d_tile_off.ptr, h->d_qtot.ptr, h->d_cdf.ptr, h->d_guide.ptr, s));
    record(h, kEvCdf, true);
    GTRY(cudaStreamWaitEvent(s, h->ev_join, 0));
    record(h, kEvCounts, true);
    GTRY(cudaMemsetAsync(h->d_work.ptr, 0, sizeof(unsigned long long), s));
    GTRY(cudaMemsetAsync(h->d_counters.ptr, 0, sizeof(SampleCounters), s));
    record(h, kEvSampleStart, true);
    GTRY(launch_sampler(c, cells, h->d_species.ptr, h->d_pids.ptr, h->d_cdf.ptr, h->d_guide.ptr,
                        h->d_qtot.ptr, h->d_offsets.ptr, h->d_item_off.ptr, h->d_item_seg.ptr, 0,
                        h->graph_cap_items, h->d_cell_of.ptr, h->d_hadrons.ptr, h->d_work.ptr,
                        h->d_counters.ptr, h->num_sms, s, h->d_limits.ptr));
    record(h, kEvSample, true);
    GraphHost* g = h->gh;
    GTRY(cudaMemcpyAsync(&g->units, h->d_offsets.ptr + nseg, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GTRY(cudaMemcpyAsync(&g->items, h->d_item_off.ptr + nseg, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GTRY(cudaMemcpyAsync(g->limits, h->d_limits.ptr, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GTRY(cudaMemcpyAsync(&g->count_err, h->d_error.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    GTRY(cudaMemcpyAsync(&g->ctr, h->d_counters.ptr, sizeof(SampleCounters), cudaMemcpyDeviceToHost, s));
    if (S > 0)
        GTRY(cudaMemcpy2DAsync(g->event_offsets, sizeof(int64_t), h->d_offsets.ptr,
                               sizeof(int64_t) * static_cast<size_t>(S), sizeof(int64_t),
                               static_cast<size_t>(c.n_events) + 1, cudaMemcpyDeviceToHost, s));
#undef GTRY
    return cudaSuccess;
}

// after an eager generate that fitted: capture the call's graph
iss_status capture_graph(iss_handle* h, int64_t n_items) {
    drop_graph(h);
    DevConfig c = h->cfg;
    const int E = c.n_events;
    CUDA_TRY(h, h->d_run.reserve(4));
    CUDA_TRY(h, h->d_limits.reserve(2));
    if (!h->gh || h->gh_events < static_cast<size_t>(E)) {
        if (h->gh) cudaFreeHost(h->gh);
        h->gh = nullptr;
        CUDA_TRY(h, cudaMallocHost(reinterpret_cast<void**>(&h->gh),
                                   sizeof(GraphHost) + sizeof(int64_t) * static_cast<size_t>(E + 1)));
        h->gh_events = static_cast<size_t>(E);
    }
    h->graph_cap_units = static_cast<int64_t>(h->d_hadrons.cap);
    h->graph_cap_items = static_cast<int64_t>(h->d_item_seg.cap);
    if (h->graph_cap_items < n_items) return ISS_OK;
    c.run = h->d_run.ptr;
    c.chunk_events = std::max(E, 1);
    cudaStream_t s = h->stream;
    if (!h->aux_stream) {
        // the counts branch at the highest priority: its blocks go first
        // whenever the CDF scan's blocks leave room (the graph keeps stream
        // priorities as node priorities)
        int least = 0, greatest = 0;
        CUDA_TRY(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CUDA_TRY(h, cudaStreamCreateWithPriority(&h->aux_stream, cudaStreamNonBlocking, greatest));
    }
    for (cudaEvent_t* e : {&h->ev_fork, &h->ev_join})
        if (!*e) CUDA_TRY(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    cudaGraph_t graph = nullptr;
    CUDA_TRY(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const cudaError_t ce = enqueue_generate(h, c);
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    // a graph that cannot be captured leaves the calls eager (the samples of
    // this call are complete either way)
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        h->graph_unavailable = true;
        h->last_error = std::string("generate runs eagerly: graph capture failed: ") +
                        cudaGetErrorString(ce != cudaSuccess ? ce : ee);
        return ISS_OK;
    }
    const cudaError_t ie =
        cudaGraphInstantiateWithFlags(&h->graph_exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        h->graph_exec = nullptr;
        cudaGetLastError();
        h->graph_unavailable = true;
        h->last_error = std::string("generate runs eagerly: graph instantiation failed: ") +
                        cudaGetErrorString(ie);
        return ISS_OK;
    }
    h->graph_key = graph_key_of(h);
    return ISS_OK;
}

// a call of the captured shape: upload the seed, launch, read the results;
// *done = false (graph dropped) when the call has to run eagerly
iss_status replay_graph(iss_handle* h, bool* done) {
    *done = false;
    DevConfig& c = h->cfg;
    cudaStream_t s = h->stream;
    if (!h->surface_on_device) {
        CUDA_TRY(h, h->d_fo34.reserve(static_cast<size_t>(h->n_cells) * kFoSurfFloats));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_fo34.ptr, h->fo34.data(),
                                    sizeof(float) * static_cast<size_t>(h->n_cells) * kFoSurfFloats,
                                    cudaMemcpyHostToDevice, s));
        h->surface_on_device = true;
    }
    if (graph_key_of(h) != h->graph_key) {
        drop_graph(h);
        return ISS_OK;
    }
    // the surface of every event (a batch may spread the same total
    // differently over its surfaces)
    {
        std::vector<int32_t>& ev_surf = h->ev_surf;
        ev_surf.assign(static_cast<size_t>(std::max(c.n_events, 1)), 0);
        for (int b = 0; b < c.n_surfaces; b++)
            for (int e = 0; e < h->segs[b].ne; e++) ev_surf[h->segs[b].e0 + e] = b;
        CUDA_TRY(h, cudaMemcpyAsync(h->d_ev_surf.ptr, ev_surf.data(), 4 * ev_surf.size(),
                                    cudaMemcpyHostToDevice, s));
    }
    GraphHost* g = h->gh;
    g->run[0] = c.key0;
    g->run[1] = c.key1;
    g->run[2] = c.event_offset;
    CUDA_TRY(h, cudaMemcpyAsync(h->d_run.ptr, g->run, 3 * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaGraphLaunch(h->graph_exec, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    h->yields_valid = true;
    if (g->count_err == 2) return fail(h, ISS_ERR_OUT_OF_RANGE, "negative particle yield (dN < 0)");
    if (g->count_err != 0) return fail(h, ISS_ERR_SAMPLING, "count draw did not converge");
    if (g->limits[1] != 0) {
        // more draws than the captured buffers hold: nothing was sampled
        drop_graph(h);
        return ISS_OK;
    }
    const int E = c.n_events;
    h->event_offsets.assign(g->event_offsets, g->event_offsets + E + 1);
    h->n_events = E;
    h->n_hadrons = g->units;
    const SampleCounters ctr = g->ctr;
    iss_timings_t& t = h->timings;
    t.ms_decays = 0.0;
    t.ms_prologue = elapsed(h, kEvStart, kEvPrologue);
    t.ms_yields = elapsed(h, kEvPrologue, kEvYields);
    t.ms_cdf = elapsed(h, kEvYields, kEvCdf);
    t.ms_counts = elapsed(h, kEvCdf, kEvCounts);
    t.ms_sample = elapsed(h, kEvSampleStart, kEvSample);
    t.ms_total = elapsed(h, kEvStart, kEvSample);
    t.n_hadrons = h->n_hadrons;
    t.n_sampled = h->n_hadrons;
    t.decay_reruns = 0;
    t.n_tries = static_cast<int64_t>(ctr.tries);
    t.n_cell_redraws = static_cast<int64_t>(ctr.redraws);
    t.n_failures = static_cast<int64_t>(ctr.failures);
    t.kernel_launches = 18;   // one graph launch of the 18 kernels of a generate
    h->samples_valid = true;
    *done = true;
    if (ctr.error_code == 1) {
        const int k = ctr.error_species;
        return fail(h, ISS_ERR_OUT_OF_RANGE,
                    "momentum sampler out of range for species %d (m/T - mu/T off the tables)",
                    (k >= 0 && k < c.n_species) ? h->species[k].pid : 0);
    }
    if (ctr.failures > 0)
        return fail(h, ISS_ERR_SAMPLING, "%llu hadrons abandoned after %d cell redraws",
                    static_cast<unsigned long long>(ctr.failures), c.max_redraws);
    return ISS_OK;
}

// A streamed generate (iss_gpu_generate_stream): the hadrons of every chunk
// of chunk_events events go to fn, the device keeping two chunks at a time.
struct StreamSink {
    int32_t chunk_events;
    iss_stream_fn fn;
    void* user;
};

iss_status run_generate(iss_handle* h, iss_hadron_t* host_out = nullptr, int64_t capacity = 0,
                        bool* copied = nullptr, const StreamSink* sink = nullptr) {
    if (copied) *copied = false;
    if (!h->surface_loaded) return fail(h, ISS_ERR_NO_SURFACE, "no surface: call iss_gpu_read_surface first");
    iss_status st = ensure_cuda(h);
    if (st != ISS_OK) return st;
    st = prepare(h);
    if (st != ISS_OK) return st;
    if (sink && h->decays)
        return fail(h, ISS_ERR_UNSUPPORTED, "perform_decays needs every event's hadrons on the device: "
                    "not with a streamed generate");
    h->samples_valid = false;
    h->host_valid = false;
    if (graph_eligible(h, host_out, sink != nullptr) && h->graph_exec) {
        bool done = false;
        st = replay_graph(h, &done);
        if (st != ISS_OK || done) return st;
    }
    st = run_cells(h);
    if (st != ISS_OK) return st;
    DevConfig& c = h->cfg;
    const int S = c.n_species;
    cudaStream_t s = h->stream;

    // number of events from the thermal pi+ yield when asked for
    // (FSSW::compute_number_of_sampling_needed, src/FSSW.cpp:851-869)
    if (h->params.get_or("sample_upto_desired_particle_number", 0) == 1) {
        double needed, max_ev;
        if (!need(h, "number_of_particles_needed", &needed) ||
            !need(h, "maximum_sampling_events", &max_ev))
            return ISS_ERR_PARAM_MISSING;
        std::vector<double> tot(static_cast<size_t>(S));
        CUDA_TRY(h, cudaMemcpyAsync(tot.data(), h->d_totals.ptr, 8 * static_cast<size_t>(S),
                                    cudaMemcpyDeviceToHost, s));
        CUDA_TRY(h, cudaStreamSynchronize(s));
        double dn_pion = 0.0;
        for (int k = 0; k < S; k++)
            if (h->species[k].real_idx == 1) dn_pion = tot[k];
        int nev = static_cast<int>(static_cast<long>(needed) / (6. * dn_pion));
        if (c.hydro_mode == 2) nev *= 10;
        nev = std::max(1, std::min(static_cast<int>(max_ev), nev));
        c.n_events = nev;
        h->segs[0].ne = nev;
    }
    // surface of every event
    {
        std::vector<int32_t>& ev_surf = h->ev_surf;
        ev_surf.assign(static_cast<size_t>(std::max(c.n_events, 1)), 0);
        for (int b = 0; b < c.n_surfaces; b++)
            for (int e = 0; e < h->segs[b].ne; e++) ev_surf[h->segs[b].e0 + e] = b;
        CUDA_TRY(h, h->d_ev_surf.reserve(ev_surf.size()));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_ev_surf.ptr, ev_surf.data(), 4 * ev_surf.size(),
                                    cudaMemcpyHostToDevice, s));
        c.ev_surf = h->d_ev_surf.ptr;
    }

    const int64_t nseg = static_cast<int64_t>(c.n_events) * S;
    CUDA_TRY(h, h->d_counts.reserve(static_cast<size_t>(std::max<int64_t>(nseg, 1))));
    CUDA_TRY(h, h->d_items.reserve(static_cast<size_t>(std::max<int64_t>(nseg, 1))));
    CUDA_TRY(h, h->d_offsets.reserve(static_cast<size_t>(nseg + 1)));
    CUDA_TRY(h, h->d_item_off.reserve(static_cast<size_t>(nseg + 1)));
    CUDA_TRY(h, h->d_off_tiles.reserve(static_cast<size_t>(std::max(offsets_num_tiles(nseg), 1))));
    // sampling chunks: one without a host destination, else up to kMaxChunks
    const int E = c.n_events;
    int n_chunks = (host_out && !h->decays) ? std::min(h->tune.copy_chunks, std::max(E, 1)) : 1;
    c.chunk_events = std::max(1, (E + n_chunks - 1) / n_chunks);
    if (sink) c.chunk_events = std::max(1, std::min(sink->chunk_events, std::max(E, 1)));
    n_chunks = std::max(1, (E + c.chunk_events - 1) / c.chunk_events);
    CUDA_TRY(h, h->d_error.reserve(1));
    CUDA_TRY(h, h->d_work.reserve(static_cast<size_t>(n_chunks)));
    CUDA_TRY(h, h->d_counters.reserve(1));
    CUDA_TRY(h, cudaMemsetAsync(h->d_error.ptr, 0, sizeof(int), s));
    // per species: kPoissonConsts constants, then an inversion table of
    // kInvTable + 1 doubles (the last holds the length)
    CUDA_TRY(h, h->d_pois.reserve(static_cast<size_t>(std::max(S * c.n_surfaces, 1)) *
                                  (kPoissonConsts + kInvTable + 1)));
    CUDA_TRY(h, launch_counts(c, h->d_species.ptr, h->d_totals.ptr, h->d_pois.ptr, h->d_counts.ptr,
                              h->d_items.ptr, h->d_error.ptr, s));
    CUDA_TRY(h, launch_offsets_scan(h->d_counts.ptr, nseg, h->d_off_tiles.ptr, h->d_offsets.ptr, s));
    CUDA_TRY(h, launch_offsets_scan(h->d_items.ptr, nseg, h->d_off_tiles.ptr, h->d_item_off.ptr, s));
    int64_t sizes[2] = {0, 0};   // hadrons, work items
    int count_err = 0;
    std::vector<int64_t> chunk_item(static_cast<size_t>(n_chunks) + 1, 0);
    h->event_offsets.assign(static_cast<size_t>(E) + 1, 0);
    CUDA_TRY(h, cudaMemcpyAsync(&sizes[0], h->d_offsets.ptr + nseg, sizeof(int64_t),
                                cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(&sizes[1], h->d_item_off.ptr + nseg, sizeof(int64_t),
                                cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(&count_err, h->d_error.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (h->use_learned) {
        // per-species totals: which species the learned proposal takes
        h->totals.resize(static_cast<size_t>(S) * c.n_surfaces);
        CUDA_TRY(h, cudaMemcpyAsync(h->totals.data(), h->d_totals.ptr, 8 * h->totals.size(),
                                    cudaMemcpyDeviceToHost, s));
    }
    if (S > 0) {
        // event offsets: offsets[e * S] for e = 0..n_events
        CUDA_TRY(h, cudaMemcpy2DAsync(h->event_offsets.data(), sizeof(int64_t), h->d_offsets.ptr,
                                      sizeof(int64_t) * static_cast<size_t>(S), sizeof(int64_t),
                                      static_cast<size_t>(E) + 1, cudaMemcpyDeviceToHost, s));
        // first work item of each chunk: item_off at segment c * chunk_events * S
        CUDA_TRY(h, cudaMemcpy2DAsync(chunk_item.data(), sizeof(int64_t), h->d_item_off.ptr,
                                      sizeof(int64_t) * static_cast<size_t>(c.chunk_events) * S,
                                      sizeof(int64_t), static_cast<size_t>(n_chunks),
                                      cudaMemcpyDeviceToHost, s));
    }
    CUDA_TRY(h, cudaStreamSynchronize(s));
    const int64_t n_units = sizes[0], n_items = sizes[1];
    chunk_item[n_chunks] = n_items;
    if (count_err == 2) return fail(h, ISS_ERR_OUT_OF_RANGE, "negative particle yield (dN < 0)");
    if (count_err != 0) return fail(h, ISS_ERR_SAMPLING, "count draw did not converge");
    const bool graph_mode = graph_eligible(h, host_out, sink != nullptr);
    // a call that will be captured gets 15 % headroom in the buffers whose
    // size depends on the draws, so that later calls fit the same graph
    const auto headroom = [&](int64_t v) { return graph_mode ? v + v / 7 + 1024 : std::max<int64_t>(v, 1); };
    CUDA_TRY(h, h->d_item_seg.reserve(static_cast<size_t>(headroom(n_items))));
    CUDA_TRY(h, launch_item_map(h->d_items.ptr, h->d_item_off.ptr, nseg, h->d_item_seg.ptr, s));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvCounts], s));
    {
        // per-generate fields; the training fields stay
        const iss_learned_stats_t keep = h->lstats;
        h->lstats = iss_learned_stats_t{};
        h->lstats.n_train_rows = keep.n_train_rows;
        h->lstats.ms_train = keep.ms_train;
        h->lstats.train_events_per_seed = keep.train_events_per_seed;
        h->lstats.train_nll_plain = keep.train_nll_plain;
    }
    if (h->use_learned) {
        const iss_status lst = run_learned_pairs(h);
        if (lst != ISS_OK) return lst;
    }

    // with decays the records change after sampling: no copies during it
    const bool to_host = host_out != nullptr && n_units <= capacity && n_units > 0 && !h->decays;
    if (to_host) {
        if (!h->copy_stream)
            CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        while (static_cast<int>(h->chunk_ev.size()) < n_chunks) {
            cudaEvent_t e;
            CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            h->chunk_ev.push_back(e);
        }
    }
    // streamed: the record buffer and cell_of hold two chunks (ring slots
    // ch & 1), the largest chunk sets their size
    int64_t ring = 0;
    if (sink) {
        for (int ch = 0; ch < n_chunks; ch++) {
            const int e0 = ch * c.chunk_events, e1 = std::min(E, e0 + c.chunk_events);
            ring = std::max(ring, h->event_offsets[e1] - h->event_offsets[e0]);
        }
        ring = std::max<int64_t>(ring, 1);
        if (!h->copy_stream)
            CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        while (static_cast<int>(h->chunk_ev.size()) < n_chunks) {
            cudaEvent_t e;
            CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            h->chunk_ev.push_back(e);
        }
        while (static_cast<int>(h->copy_ev.size()) < n_chunks) {
            cudaEvent_t e;
            CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            h->copy_ev.push_back(e);
        }
        if (h->stream_host_cap < ring) {
            if (h->stream_host) cudaFreeHost(h->stream_host);
            h->stream_host = nullptr;
            h->stream_host_cap = 0;
            CUDA_TRY(h, cudaMallocHost(reinterpret_cast<void**>(&h->stream_host),
                                       2 * sizeof(iss_hadron_t) * static_cast<size_t>(ring)));
            h->stream_host_cap = ring;
        }
    }
    CUDA_TRY(h, h->d_hadrons.reserve(static_cast<size_t>(sink ? 2 * ring : headroom(n_units))));
    CUDA_TRY(h, h->d_cell_of.reserve(static_cast<size_t>(sink ? 2 * ring : headroom(n_units))));
    CUDA_TRY(h, cudaMemsetAsync(h->d_work.ptr, 0, sizeof(unsigned long long) * n_chunks, s));
    CUDA_TRY(h, cudaMemsetAsync(h->d_counters.ptr, 0, sizeof(SampleCounters), s));
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvSampleStart], s));
    // hands chunk ch's records (already copied to the host) to the sink
    std::vector<int64_t> rel;
    const auto deliver = [&](int ch) -> iss_status {
        CUDA_TRY(h, cudaEventSynchronize(h->copy_ev[ch]));
        const int e0 = ch * c.chunk_events, e1 = std::min(E, e0 + c.chunk_events);
        const int64_t b = h->event_offsets[e0];
        rel.assign(static_cast<size_t>(e1 - e0) + 1, 0);
        for (int e = e0; e <= e1; e++) rel[e - e0] = h->event_offsets[e] - b;
        sink->fn(sink->user, h->stream_host + (ch & 1) * ring, rel[e1 - e0], e0, e1 - e0, rel.data());
        return ISS_OK;
    };
    for (int ch = 0; ch < n_chunks && sink; ch++) {
        const int e0 = ch * c.chunk_events, e1 = std::min(E, e0 + c.chunk_events);
        const int64_t b = h->event_offsets[e0], n = h->event_offsets[e1] - b;
        const int slot = ch & 1;
        // ring slot `slot` was last read by the copy of chunk ch - 2
        if (ch >= 2) CUDA_TRY(h, cudaStreamWaitEvent(s, h->copy_ev[ch - 2], 0));
        DevConfig cc = c;
        cc.slot_base = b;
        CUDA_TRY(h, launch_sampler(cc, cell_arrays(h), h->d_species.ptr, h->d_pids.ptr, h->d_cdf.ptr,
                                   h->d_guide.ptr, h->d_qtot.ptr, h->d_offsets.ptr, h->d_item_off.ptr,
                                   h->d_item_seg.ptr, chunk_item[ch], chunk_item[ch + 1],
                                   h->d_cell_of.ptr + slot * ring, h->d_hadrons.ptr + slot * ring,
                                   h->d_work.ptr + ch, h->d_counters.ptr, h->num_sms, s));
        CUDA_TRY(h, cudaEventRecord(h->chunk_ev[ch], s));
        // the previous chunk's records reach the caller while this one samples
        // (its host buffer, slot ^ 1, is free again once the sink returns)
        if (ch >= 1) {
            const iss_status dst = deliver(ch - 1);
            if (dst != ISS_OK) return dst;
        }
        CUDA_TRY(h, cudaStreamWaitEvent(h->copy_stream, h->chunk_ev[ch], 0));
        if (n > 0)
            CUDA_TRY(h, cudaMemcpyAsync(h->stream_host + slot * ring, h->d_hadrons.ptr + slot * ring,
                                        sizeof(iss_hadron_t) * static_cast<size_t>(n),
                                        cudaMemcpyDeviceToHost, h->copy_stream));
        CUDA_TRY(h, cudaEventRecord(h->copy_ev[ch], h->copy_stream));
    }
    if (sink && n_chunks > 0) {
        const iss_status dst = deliver(n_chunks - 1);
        if (dst != ISS_OK) return dst;
    }
    for (int ch = 0; ch < n_chunks && !sink; ch++) {
        CUDA_TRY(h, launch_sampler(c, cell_arrays(h), h->d_species.ptr, h->d_pids.ptr, h->d_cdf.ptr,
                                   h->d_guide.ptr, h->d_qtot.ptr,
                                   h->d_offsets.ptr, h->d_item_off.ptr, h->d_item_seg.ptr,
                                   chunk_item[ch], chunk_item[ch + 1], h->d_cell_of.ptr,
                                   h->d_hadrons.ptr, h->d_work.ptr + ch, h->d_counters.ptr,
                                   h->num_sms, s));
        if (to_host) {
            // records of events [e0, e1) are final: copy them while the next chunk runs
            const int e0 = ch * c.chunk_events, e1 = std::min(E, e0 + c.chunk_events);
            const int64_t b = h->event_offsets[e0], n = h->event_offsets[e1] - b;
            CUDA_TRY(h, cudaEventRecord(h->chunk_ev[ch], s));
            CUDA_TRY(h, cudaStreamWaitEvent(h->copy_stream, h->chunk_ev[ch], 0));
            if (n > 0)
                CUDA_TRY(h, cudaMemcpyAsync(host_out + b, h->d_hadrons.ptr + b,
                                            sizeof(iss_hadron_t) * static_cast<size_t>(n),
                                            cudaMemcpyDeviceToHost, h->copy_stream));
        }
    }
    CUDA_TRY(h, cudaEventRecord(h->ev[kEvSample], s));
    SampleCounters ctr{};
    CUDA_TRY(h, cudaMemcpyAsync(&ctr, h->d_counters.ptr, sizeof(ctr), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    if (to_host) {
        CUDA_TRY(h, cudaStreamSynchronize(h->copy_stream));
        if (copied) *copied = true;
    }
    CUDA_TRY(h, cudaGetLastError());

    h->n_events = c.n_events;
    h->n_hadrons = n_units;
    const bool streamed = sink != nullptr;
    unsigned long long decay_failures = 0;
    float ms_decays = 0.f;
    if (h->decays) {
        for (auto& e : h->ev_decay)
            if (!e) CUDA_TRY(h, cudaEventCreate(&e));
        CUDA_TRY(h, cudaEventRecord(h->ev_decay[0], s));
        const iss_status dst = run_decays(h, &decay_failures);
        if (dst != ISS_OK) return dst;
        CUDA_TRY(h, cudaEventRecord(h->ev_decay[1], s));
        CUDA_TRY(h, cudaEventSynchronize(h->ev_decay[1]));
        cudaEventElapsedTime(&ms_decays, h->ev_decay[0], h->ev_decay[1]);
        if (host_out && h->n_hadrons <= capacity && h->n_hadrons > 0) {
            CUDA_TRY(h, cudaMemcpy(host_out, h->d_hadrons.ptr,
                                   sizeof(iss_hadron_t) * static_cast<size_t>(h->n_hadrons),
                                   cudaMemcpyDeviceToHost));
            if (copied) *copied = true;
        }
    }

    iss_timings_t& t = h->timings;
    t.ms_decays = ms_decays;
    t.decay_reruns = h->decays ? h->dk_reruns : 0;
    t.ms_prologue = elapsed(h, kEvStart, kEvPrologue);
    t.ms_yields = elapsed(h, kEvPrologue, kEvYields);
    t.ms_cdf = elapsed(h, kEvYields, kEvCdf);
    t.ms_counts = elapsed(h, kEvCdf, kEvCounts);
    t.ms_sample = elapsed(h, kEvSampleStart, kEvSample);
    t.ms_total = elapsed(h, kEvStart, kEvSample);
    t.n_hadrons = h->n_hadrons;
    t.n_sampled = n_units;
    t.n_tries = static_cast<int64_t>(ctr.tries);
    t.n_cell_redraws = static_cast<int64_t>(ctr.redraws);
    t.n_failures = static_cast<int64_t>(ctr.failures + decay_failures);
    t.kernel_launches = 15 + 2 * n_chunks;
    if (h->use_learned) {
        t.kernel_launches += 4;
        h->lstats.n_tries = static_cast<int64_t>(ctr.learned_tries);
        h->lstats.n_hadrons = static_cast<int64_t>(ctr.learned_hadrons);
        h->lstats.n_violations = static_cast<int64_t>(ctr.learned_violations);
        h->lstats.n_excess_tries = static_cast<int64_t>(ctr.learned_excess_tries);
        h->lstats.n_excess_hadrons = static_cast<int64_t>(ctr.learned_excess_hadrons);
        h->lstats.n_over_one = static_cast<int64_t>(ctr.learned_over_one);
        h->lstats.ms_network = elapsed(h, kEvLearnStart, kEvLearnEnd);
        h->lstats.ms_forward = elapsed(h, kEvFwdStart, kEvFwdEnd);
    }
    h->samples_valid = !streamed;   // a streamed generate keeps no records
    if (ctr.error_code == 1) {
        const int k = ctr.error_species;
        return fail(h, ISS_ERR_OUT_OF_RANGE,
                    "momentum sampler out of range for species %d (m/T - mu/T off the tables)",
                    (k >= 0 && k < S) ? h->species[k].pid : 0);
    }
    if (h->use_learned && h->learned.device_error(s) != 0)
        return fail(h, ISS_ERR_SAMPLING, "a tensor-core wait of the proposal network timed out");
    if (ctr.failures > 0)
        return fail(h, ISS_ERR_SAMPLING, "%llu hadrons abandoned after %d cell redraws",
                    static_cast<unsigned long long>(ctr.failures), c.max_redraws);
    if (graph_mode) return capture_graph(h, n_items);
    return ISS_OK;
}

bool tuning_valid(const iss_tuning_t& t) {
    return t.item_size >= 32 && t.item_size <= 1024 && t.item_size % 32 == 0 && t.yield_groups >= 1 &&
           t.yield_groups <= 32 && t.sampler_ctas >= 1 && t.sampler_ctas <= 3 && t.assign_blocks >= 1 &&
           t.assign_blocks <= 32 && t.copy_chunks >= 1 && t.copy_chunks <= 64;
}

// Tuning results per workload shape, shared by the handles of the process.
using TuneKey = std::tuple<int64_t, int64_t, int, int, int, int, int>;
std::mutex g_tune_mutex;
std::map<TuneKey, iss_tuning_t> g_tune_cache;

TuneKey tune_key(iss_handle* h) {
    return TuneKey{h->n_cells, static_cast<int64_t>(h->batch_events.size()),
                   static_cast<int>(h->params.get_or("number_of_repeated_sampling", 0)),
                   static_cast<int>(h->species.size()),
                   static_cast<int>(h->params.get_or("local_charge_conservation", 0)),
                   static_cast<int>(h->params.get_or("gpu_sampler", 0)),
                   static_cast<int>(h->params.get_or("hydro_mode", 2))};
}

// Coordinate descent over the launch shape on the handle's own workload:
// species groups per cell (objective: the yields phase), then draws per work
// item, sampler CTAs per SM and cell-assignment blocks per SM (objective: the
// sample phase).  Each candidate runs two generates and keeps the faster
// device time; a candidate replaces the incumbent only when it is 2 % faster.
iss_status autotune(iss_handle* h, double* ms_before, double* ms_after) {
    auto measure = [&](const iss_tuning_t& t, double* y, double* smp, double* tot) -> iss_status {
        h->tune = t;
        *y = *smp = *tot = 1e300;
        for (int r = 0; r < 2; r++) {
            const iss_status st = run_generate(h);
            if (st != ISS_OK) return st;
            *y = std::min(*y, h->timings.ms_yields);
            *smp = std::min(*smp, h->timings.ms_sample);
            *tot = std::min(*tot, h->timings.ms_total);
        }
        return ISS_OK;
    };
    iss_tuning_t best = h->tune;
    double by, bs, bt;
    iss_status st = measure(best, &by, &bs, &bt);
    if (st != ISS_OK) return st;
    if (ms_before) *ms_before = bt;
    const int groups[] = {1, 2, 4, 8, 16};
    for (int g : groups) {
        if (g == best.yield_groups || g > static_cast<int>(h->species.size())) continue;
        iss_tuning_t t = best;
        t.yield_groups = g;
        double y, smp, tot;
        if ((st = measure(t, &y, &smp, &tot)) != ISS_OK) return st;
        if (y < 0.98 * by) {
            best = t;
            by = y;
        }
    }
    // the sample phase: re-measure the incumbent with the chosen groups
    if ((st = measure(best, &by, &bs, &bt)) != ISS_OK) return st;
    const int items[] = {32, 64, 128, 256, 512};
    for (int it : items) {
        if (it == best.item_size) continue;
        iss_tuning_t t = best;
        t.item_size = it;
        double y, smp, tot;
        if ((st = measure(t, &y, &smp, &tot)) != ISS_OK) return st;
        if (smp < 0.98 * bs) {
            best = t;
            bs = smp;
        }
    }
    const int ctas[] = {2, 3};
    for (int c : ctas) {
        if (c == best.sampler_ctas) continue;
        iss_tuning_t t = best;
        t.sampler_ctas = c;
        double y, smp, tot;
        if ((st = measure(t, &y, &smp, &tot)) != ISS_OK) return st;
        if (smp < 0.98 * bs) {
            best = t;
            bs = smp;
        }
    }
    const int assign[] = {4, 8, 16};
    for (int a : assign) {
        if (a == best.assign_blocks) continue;
        iss_tuning_t t = best;
        t.assign_blocks = a;
        double y, smp, tot;
        if ((st = measure(t, &y, &smp, &tot)) != ISS_OK) return st;
        if (smp < 0.98 * bs) {
            best = t;
            bs = smp;
        }
    }
    if ((st = measure(best, &by, &bs, &bt)) != ISS_OK) return st;
    if (ms_after) *ms_after = bt;
    h->tuned = true;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[tune_key(h)] = best;
    return ISS_OK;
}

// gpu_autotune = 1: the first generate of a workload shape takes the cached
// launch shape or tunes one
iss_status maybe_autotune(iss_handle* h) {
    if (h->tuned || h->params.get_or("gpu_autotune", 0) != 1) return ISS_OK;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        const auto it = g_tune_cache.find(tune_key(h));
        if (it != g_tune_cache.end()) {
            h->tune = it->second;
            h->tuned = true;
            return ISS_OK;
        }
    }
    return autotune(h, nullptr, nullptr);
}

iss_status ensure_host_copy(iss_handle* h) {
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples: call iss_gpu_generate first");
    if (h->host_valid) return ISS_OK;
    h->host_hadrons.resize(static_cast<size_t>(h->n_hadrons));
    if (h->n_hadrons > 0) {
        CUDA_TRY(h, cudaMemcpy(h->host_hadrons.data(), h->d_hadrons.ptr,
                               sizeof(iss_hadron_t) * static_cast<size_t>(h->n_hadrons),
                               cudaMemcpyDeviceToHost));
    }
    h->host_valid = true;
    return ISS_OK;
}

// OSCAR output with the text made on the GPU: the header file is copied,
// then chunks of whole events are formatted on the device, copied to
// page-locked host memory and written, two chunks in flight.
iss_status write_oscar_gpu(iss_handle* h, const char* filename) {
    const std::string header_file = h->table_path + "/OSCAR_header.txt";
    std::ifstream header(header_file);
    if (!header) return fail(h, ISS_ERR_IO, "OSCAR header file %s not found", header_file.c_str());
    std::remove(filename);
    std::FILE* f = std::fopen(filename, "w");
    if (!f) return fail(h, ISS_ERR_IO, "can not open %s", filename);
    std::string line;
    while (std::getline(header, line)) std::fprintf(f, "%s\n", line.c_str());
    const int E = h->n_events;
    const std::vector<int64_t>& off = h->event_offsets;
    std::vector<int64_t> ev_byte(static_cast<size_t>(E) + 1, 0);
    for (int e = 0; e < E; e++) {
        const int64_t n = off[e + 1] - off[e];
        ev_byte[e + 1] = ev_byte[e] + (n > 0 ? kOscarSubHeader + n * kOscarLine : 0);
    }
    const int64_t kChunk = int64_t(256) << 20;
    DevBuf<int64_t> d_off, d_byte;
    DevBuf<char> d_text[2];
    char* host[2] = {nullptr, nullptr};
    cudaStream_t s = h->stream;
    cudaEvent_t done[2] = {nullptr, nullptr};
    iss_status st = ISS_OK;
    auto cleanup = [&]() {
        for (int k = 0; k < 2; k++) {
            if (done[k]) cudaEventDestroy(done[k]);
            if (host[k]) cudaFreeHost(host[k]);
            d_text[k].release();
        }
        d_off.release();
        d_byte.release();
        std::fclose(f);
    };
#define OSCAR_TRY(x)                                                                   \
    do {                                                                               \
        const cudaError_t e_ = (x);                                                    \
        if (e_ != cudaSuccess) {                                                       \
            cleanup();                                                                 \
            return fail(h, ISS_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));        \
        }                                                                              \
    } while (0)
    // chunks: runs of whole events of at most kChunk bytes (an event larger
    // than that is a chunk by itself)
    std::vector<std::pair<int, int>> chunks;
    int64_t max_bytes = 0;
    for (int e = 0; e < E;) {
        int e1 = e + 1;
        while (e1 < E && ev_byte[e1 + 1] - ev_byte[e] <= kChunk) e1++;
        chunks.push_back({e, e1});
        max_bytes = std::max(max_bytes, ev_byte[e1] - ev_byte[e]);
        e = e1;
    }
    OSCAR_TRY(d_off.reserve(off.size()));
    OSCAR_TRY(d_byte.reserve(ev_byte.size()));
    OSCAR_TRY(cudaMemcpyAsync(d_off.ptr, off.data(), 8 * off.size(), cudaMemcpyHostToDevice, s));
    OSCAR_TRY(cudaMemcpyAsync(d_byte.ptr, ev_byte.data(), 8 * ev_byte.size(), cudaMemcpyHostToDevice, s));
    for (int k = 0; k < 2 && k < static_cast<int>(chunks.size()); k++) {
        OSCAR_TRY(d_text[k].reserve(static_cast<size_t>(std::max<int64_t>(max_bytes, 1))));
        OSCAR_TRY(cudaHostAlloc(reinterpret_cast<void**>(&host[k]),
                                static_cast<size_t>(std::max<int64_t>(max_bytes, 1)), cudaHostAllocDefault));
        OSCAR_TRY(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
    }
    auto enqueue = [&](size_t c) -> cudaError_t {
        const int k = static_cast<int>(c & 1);
        const int ea = chunks[c].first, eb = chunks[c].second;
        const int64_t bytes = ev_byte[eb] - ev_byte[ea];
        cudaError_t e = launch_oscar_lines(h->d_hadrons.ptr, off[ea], off[eb], d_off.ptr, d_byte.ptr,
                                           ea, eb, ev_byte[ea], d_text[k].ptr, h->num_sms, s);
        if (e != cudaSuccess) return e;
        if (bytes > 0) e = cudaMemcpyAsync(host[k], d_text[k].ptr, static_cast<size_t>(bytes),
                                           cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return e;
        return cudaEventRecord(done[k], s);
    };
    if (!chunks.empty()) OSCAR_TRY(enqueue(0));
    for (size_t c = 0; c < chunks.size(); c++) {
        // chunk c + 1 is formatted while chunk c is written; chunk c + 1 uses
        // the other buffer, which chunk c - 1 released when it was written
        if (c + 1 < chunks.size()) OSCAR_TRY(enqueue(c + 1));
        const int k = static_cast<int>(c & 1);
        OSCAR_TRY(cudaEventSynchronize(done[k]));
        const int64_t bytes = ev_byte[chunks[c].second] - ev_byte[chunks[c].first];
        if (bytes > 0 && std::fwrite(host[k], 1, static_cast<size_t>(bytes), f) != static_cast<size_t>(bytes)) {
            cleanup();
            return fail(h, ISS_ERR_IO, "write error on %s", filename);
        }
    }
#undef OSCAR_TRY
    cleanup();
    return st;
}

}  // namespace

static_assert(sizeof(iss_hadron_t) == 40, "iss_hadron_t must be 40 bytes");
static_assert(sizeof(HadronRec) == sizeof(iss_hadron_t), "device record layout");

extern "C" {

const char* iss_gpu_status_string(int status) {
    switch (status) {
        case ISS_OK: return "ok";
        case ISS_ERR_INVALID_ARG: return "invalid argument";
        case ISS_ERR_IO: return "file not found or unreadable";
        case ISS_ERR_PARAM_MISSING: return "parameter missing";
        case ISS_ERR_UNSUPPORTED: return "unsupported option";
        case ISS_ERR_CUDA: return "CUDA error";
        case ISS_ERR_OUT_OF_RANGE: return "value out of range";
        case ISS_ERR_NO_SURFACE: return "no surface";
        case ISS_ERR_NO_SAMPLES: return "no samples";
        case ISS_ERR_CAPACITY: return "buffer too small";
        case ISS_ERR_SAMPLING: return "sampling failure";
        default: return "unknown status";
    }
}

const char* iss_gpu_last_error(const iss_handle* h) { return h ? h->last_error.c_str() : ""; }

iss_status iss_gpu_create(const char* work_path, const char* table_path,
                          const char* particle_table_path, const char* param_file,
                          const char* surface_filename, iss_handle** out) {
    if (!out || !work_path) return ISS_ERR_INVALID_ARG;
    *out = nullptr;
    std::unique_ptr<iss_handle> h(new iss_handle);
    h->work_path = work_path;
    h->table_path = table_path ? table_path : "iSS_tables";
    h->particle_table_path = particle_table_path ? particle_table_path : "iSS_tables";
    h->surface_filename = surface_filename ? surface_filename : "surface.dat";
    const std::string pf = param_file ? param_file : "iSS_parameters.dat";
    if (!pf.empty() && !h->params.read_file(pf)) {
        return ISS_ERR_IO;
    }
    *out = h.release();
    return ISS_OK;
}

iss_status iss_gpu_destroy(iss_handle* h) {
    delete h;
    return ISS_OK;
}

iss_status iss_gpu_set_param(iss_handle* h, const char* key, double value) {
    if (!h || !key) return ISS_ERR_INVALID_ARG;
    h->params.set(key, value);
    return ISS_OK;
}

iss_status iss_gpu_get_param(iss_handle* h, const char* key, double* value) {
    if (!h || !key || !value) return ISS_ERR_INVALID_ARG;
    if (!h->params.get(key, value))
        return fail(h, ISS_ERR_PARAM_MISSING, "parameter with name %s not found", key);
    return ISS_OK;
}

iss_status iss_gpu_parse_param_line(iss_handle* h, const char* line) {
    if (!h || !line) return ISS_ERR_INVALID_ARG;
    h->params.parse_line(line);
    return ISS_OK;
}

iss_status iss_gpu_set_seed(iss_handle* h, int64_t seed) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (seed == -1) {
        std::random_device rd;
        seed = (static_cast<int64_t>(rd()) << 32) ^ rd();
    }
    h->seed = seed;
    h->seed_set = true;
    h->samples_valid = false;
    return ISS_OK;
}

iss_status iss_gpu_set_seed_from_params(iss_handle* h) {
    if (!h) return ISS_ERR_INVALID_ARG;
    double v;
    if (!need(h, "randomSeed", &v)) return ISS_ERR_PARAM_MISSING;
    return iss_gpu_set_seed(h, static_cast<int64_t>(v));
}

iss_status iss_gpu_read_surface(iss_handle* h) {
    if (!h) return ISS_ERR_INVALID_ARG;
    h->batch_cells.clear();
    h->batch_events.clear();
    double mode, qs;
    if (!need(h, "hydro_mode", &mode) || !need(h, "quantum_statistics", &qs))
        return ISS_ERR_PARAM_MISSING;
    h->hydro_mode = static_cast<int>(mode);
    h->quantum_statistics = static_cast<int>(qs) == 1;
    if (h->hydro_mode != 1 && h->hydro_mode != 2)
        return fail(h, ISS_ERR_UNSUPPORTED, "hydro_mode %d: only MUSIC surfaces (1, 2) are read",
                    h->hydro_mode);
    MusicSettings ms;
    std::string err;
    if (!read_music_input(h->work_path, h->params, &ms, &err)) return fail(h, ISS_ERR_IO, "%s", err.c_str());
    if (!eos_is_known(ms.iEOS)) return fail(h, ISS_ERR_INVALID_ARG, "invalid EOS_to_use %d", ms.iEOS);
    if (!eos_is_chemical_equilibrium(ms.iEOS))
        return fail(h, ISS_ERR_UNSUPPORTED,
                    "EOS_to_use %d is partially chemically equilibrated (PCE); not supported", ms.iEOS);
    h->iEOS = ms.iEOS;
    h->afterburner = select_afterburner(h->params, ms.iEOS);
    if (!read_music_surface(h->work_path + "/" + h->surface_filename, h->hydro_mode, ms, &h->fo34,
                            &err))
        return fail(h, ISS_ERR_IO, "%s", err.c_str());
    if (ms.iEOS == 9 || ms.iEOS == 91 || ms.iEOS == 12 || ms.iEOS == 14) {
        HrgEos eos;
        if (!load_hrg_eos(h->table_path, ms.iEOS, h->afterburner, &eos, &err))
            return fail(h, ISS_ERR_IO, "%s", err.c_str());
        regulate_temperature(eos, &h->fo34);
    }
    iss_status st = load_species(h);
    if (st != ISS_OK) return st;
    return finish_surface(h);
}

iss_status iss_gpu_set_surface(iss_handle* h, const float* records, int64_t n_cells) {
    if (!h || (!records && n_cells > 0) || n_cells < 0) return ISS_ERR_INVALID_ARG;
    double mode, qs;
    if (!need(h, "hydro_mode", &mode) || !need(h, "quantum_statistics", &qs))
        return ISS_ERR_PARAM_MISSING;
    h->hydro_mode = static_cast<int>(mode);
    h->quantum_statistics = static_cast<int>(qs) == 1;
    h->iEOS = 2;
    h->afterburner = select_afterburner(h->params, 2);
    if (h->species.empty() || h->species_afterburner != h->afterburner ||
        h->species_qs != h->quantum_statistics) {
        iss_status st = load_species(h);
        if (st != ISS_OK) return st;
    }
    if (n_cells == 0) return fail(h, ISS_ERR_NO_SURFACE, "no freeze-out fluid cell");
    h->batch_cells.clear();
    h->batch_events.clear();
    // With a device, the records go straight from the caller's buffer (pinned
    // or pageable) to HBM; without one a host copy is kept for inspection.
    if (ensure_cuda(h) == ISS_OK) {
        const size_t bytes = sizeof(float) * static_cast<size_t>(n_cells) * kFoSurfFloats;
        CUDA_TRY(h, h->d_fo34.reserve(static_cast<size_t>(n_cells) * kFoSurfFloats));
        CUDA_TRY(h, cudaMemcpyAsync(h->d_fo34.ptr, records, bytes, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        h->fo34.clear();
        h->n_cells = n_cells;
        h->surface_loaded = true;
        h->surface_on_device = true;
        h->yields_valid = false;
        h->samples_valid = false;
        h->host_valid = false;
        h->last_error.clear();
        return ISS_OK;
    }
    h->last_error.clear();
    h->fo34.assign(records, records + static_cast<size_t>(n_cells) * kFoSurfFloats);
    return finish_surface(h);
}

iss_status iss_gpu_set_surface_batch(iss_handle* h, const float* records,
                                     const int64_t* cell_offsets, const int32_t* events,
                                     int32_t n_surfaces) {
    if (!h || !records || !cell_offsets || !events || n_surfaces <= 0)
        return ISS_ERR_INVALID_ARG;
    if (cell_offsets[0] != 0) return fail(h, ISS_ERR_INVALID_ARG, "cell_offsets[0] must be 0");
    int64_t total_events = 0;
    for (int32_t b = 0; b < n_surfaces; b++) {
        if (cell_offsets[b + 1] <= cell_offsets[b])
            return fail(h, ISS_ERR_NO_SURFACE, "surface %d of the batch has no cell", b);
        if (events[b] < 0) return fail(h, ISS_ERR_INVALID_ARG, "surface %d: negative events", b);
        total_events += events[b];
    }
    if (cell_offsets[n_surfaces] >= (int64_t(1) << 31))
        return fail(h, ISS_ERR_INVALID_ARG, "a batch holds fewer than 2^31 cells");
    if (total_events >= (int64_t(1) << 31))
        return fail(h, ISS_ERR_INVALID_ARG, "a batch holds fewer than 2^31 events");
    iss_status st = iss_gpu_set_surface(h, records, cell_offsets[n_surfaces]);
    if (st != ISS_OK) return st;
    h->batch_cells.assign(cell_offsets, cell_offsets + n_surfaces + 1);
    h->batch_events.assign(events, events + n_surfaces);
    return ISS_OK;
}

iss_status iss_gpu_generate(iss_handle* h) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!h->seed_set) {
        iss_status st = iss_gpu_set_seed_from_params(h);
        if (st != ISS_OK) return st;
    }
    const iss_status st = maybe_autotune(h);
    if (st != ISS_OK) return st;
    return run_generate(h);
}

iss_status iss_gpu_generate_into(iss_handle* h, iss_hadron_t* out, int64_t capacity,
                                 int64_t* n_total) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (n_total) *n_total = 0;
    if (capacity < 0 || (capacity > 0 && !out)) return fail(h, ISS_ERR_INVALID_ARG, "bad output buffer");
    if (!h->seed_set) {
        iss_status st = iss_gpu_set_seed_from_params(h);
        if (st != ISS_OK) return st;
    }
    const iss_status tst = maybe_autotune(h);
    if (tst != ISS_OK) return tst;
    bool copied = false;
    const iss_status st = run_generate(h, out, capacity, &copied);
    if (n_total && h->samples_valid) *n_total = h->n_hadrons;
    if (st != ISS_OK) return st;
    if (!copied && h->n_hadrons > 0)
        return fail(h, ISS_ERR_CAPACITY, "%lld hadrons do not fit in %lld records (samples kept "
                    "on the device)", static_cast<long long>(h->n_hadrons),
                    static_cast<long long>(capacity));
    return ISS_OK;
}

iss_status iss_gpu_generate_stream(iss_handle* h, int32_t chunk_events, iss_stream_fn fn, void* user) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!fn || chunk_events < 1) return fail(h, ISS_ERR_INVALID_ARG, "no sink or chunk_events < 1");
    if (!h->seed_set) {
        iss_status st = iss_gpu_set_seed_from_params(h);
        if (st != ISS_OK) return st;
    }
    const iss_status tst = maybe_autotune(h);
    if (tst != ISS_OK) return tst;
    const StreamSink sink{chunk_events, fn, user};
    return run_generate(h, nullptr, 0, nullptr, &sink);
}

iss_status iss_gpu_shell(iss_handle* h) {
    if (!h) return ISS_ERR_INVALID_ARG;
    iss_status st = iss_gpu_read_surface(h);
    if (st != ISS_OK) return st;
    st = iss_gpu_set_seed_from_params(h);
    if (st != ISS_OK) return st;
    return run_generate(h);
}

iss_status iss_gpu_clear(iss_handle* h) {
    if (!h) return ISS_ERR_INVALID_ARG;
    h->fo34.clear();
    h->n_cells = 0;
    h->surface_loaded = false;
    h->surface_on_device = false;
    h->yields_valid = false;
    h->samples_valid = false;
    h->host_valid = false;
    h->host_hadrons.clear();
    h->event_offsets.clear();
    h->species.clear();
    h->species_afterburner = -1;
    return ISS_OK;
}

iss_status iss_gpu_num_events(iss_handle* h, int32_t* n) {
    if (!h || !n) return ISS_ERR_INVALID_ARG;
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples");
    *n = h->n_events;
    return ISS_OK;
}

iss_status iss_gpu_num_particles(iss_handle* h, int32_t iev, int64_t* n) {
    if (!h || !n) return ISS_ERR_INVALID_ARG;
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples");
    if (iev < 0 || iev >= h->n_events) return fail(h, ISS_ERR_INVALID_ARG, "event %d out of range", iev);
    *n = h->event_offsets[iev + 1] - h->event_offsets[iev];
    return ISS_OK;
}

iss_status iss_gpu_get_hadron(iss_handle* h, int32_t iev, int64_t ipart, iss_hadron_t* out) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    iss_status st = ensure_host_copy(h);
    if (st != ISS_OK) return st;
    if (iev < 0 || iev >= h->n_events) return fail(h, ISS_ERR_INVALID_ARG, "event %d out of range", iev);
    const int64_t n = h->event_offsets[iev + 1] - h->event_offsets[iev];
    if (ipart < 0 || ipart >= n) return fail(h, ISS_ERR_INVALID_ARG, "particle %lld out of range",
                                             static_cast<long long>(ipart));
    *out = h->host_hadrons[static_cast<size_t>(h->event_offsets[iev] + ipart)];
    return ISS_OK;
}

iss_status iss_gpu_copy_event(iss_handle* h, int32_t iev, iss_hadron_t* out, int64_t capacity,
                              int64_t* n_written) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples");
    if (iev < 0 || iev >= h->n_events) return fail(h, ISS_ERR_INVALID_ARG, "event %d out of range", iev);
    const int64_t b = h->event_offsets[iev], n = h->event_offsets[iev + 1] - b;
    if (n_written) *n_written = n;
    if (!out) return ISS_OK;
    if (capacity < n) return fail(h, ISS_ERR_CAPACITY, "event %d has %lld hadrons", iev,
                                  static_cast<long long>(n));
    if (n == 0) return ISS_OK;
    if (h->host_valid) {
        std::memcpy(out, h->host_hadrons.data() + b, sizeof(iss_hadron_t) * static_cast<size_t>(n));
        return ISS_OK;
    }
    CUDA_TRY(h, cudaMemcpy(out, h->d_hadrons.ptr + b, sizeof(iss_hadron_t) * static_cast<size_t>(n),
                           cudaMemcpyDeviceToHost));
    return ISS_OK;
}

iss_status iss_gpu_copy_all(iss_handle* h, iss_hadron_t* out, int64_t capacity,
                            int64_t* event_offsets, int64_t* n_total) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples");
    if (n_total) *n_total = h->n_hadrons;
    if (event_offsets)
        std::memcpy(event_offsets, h->event_offsets.data(), sizeof(int64_t) * h->event_offsets.size());
    if (!out) return ISS_OK;
    if (capacity < h->n_hadrons) return fail(h, ISS_ERR_CAPACITY, "%lld hadrons do not fit",
                                             static_cast<long long>(h->n_hadrons));
    if (h->n_hadrons == 0) return ISS_OK;
    if (h->host_valid) {
        std::memcpy(out, h->host_hadrons.data(), sizeof(iss_hadron_t) * static_cast<size_t>(h->n_hadrons));
        return ISS_OK;
    }
    CUDA_TRY(h, cudaMemcpyAsync(out, h->d_hadrons.ptr,
                                sizeof(iss_hadron_t) * static_cast<size_t>(h->n_hadrons),
                                cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return ISS_OK;
}

iss_status iss_gpu_write_output(iss_handle* h, int format, const char* filename) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (format == ISS_OUTPUT_OSCAR && h->samples_valid && h->cuda_ready &&
        h->params.get_or("gpu_oscar_on_host", 0) == 0)
        return write_oscar_gpu(h, filename ? filename : "OSCAR.DAT");
    iss_status st = ensure_host_copy(h);
    if (st != ISS_OK) return st;
    std::string err;
    bool ok = false;
    const iss_hadron_t* hd = h->host_hadrons.data();
    const int64_t* off = h->event_offsets.data();
    if (format == ISS_OUTPUT_OSCAR) {
        ok = write_oscar(filename ? filename : "OSCAR.DAT", h->table_path + "/OSCAR_header.txt", hd,
                         off, h->n_events, &err);
    } else if (format == ISS_OUTPUT_GZIP) {
        ok = write_gzip(filename ? filename : "particle_samples.gz", hd, off, h->n_events, &err);
    } else if (format == ISS_OUTPUT_BINARY) {
        ok = write_binary(filename ? filename : "particle_samples.bin", hd, off, h->n_events, &err);
    } else {
        return fail(h, ISS_ERR_INVALID_ARG, "unknown output format %d", format);
    }
    return ok ? ISS_OK : fail(h, ISS_ERR_IO, "%s", err.c_str());
}

iss_status iss_gpu_write_hadron_list(int format, const char* filename, const char* table_path,
                                     const iss_hadron_t* hadrons, const int64_t* event_offsets,
                                     int32_t n_events) {
    if (n_events < 0 || !event_offsets || (event_offsets[n_events] > 0 && !hadrons))
        return ISS_ERR_INVALID_ARG;
    for (int32_t e = 0; e < n_events; e++)
        if (event_offsets[e + 1] < event_offsets[e] || event_offsets[e] < 0) return ISS_ERR_INVALID_ARG;
    const std::string tables = table_path ? table_path : "iSS_tables";
    std::string err;
    bool ok = false;
    if (format == ISS_OUTPUT_OSCAR) {
        ok = write_oscar(filename ? filename : "OSCAR.DAT", tables + "/OSCAR_header.txt", hadrons,
                         event_offsets, n_events, &err);
    } else if (format == ISS_OUTPUT_GZIP) {
        ok = write_gzip(filename ? filename : "particle_samples.gz", hadrons, event_offsets, n_events,
                        &err);
    } else if (format == ISS_OUTPUT_BINARY) {
        ok = write_binary(filename ? filename : "particle_samples.bin", hadrons, event_offsets,
                          n_events, &err);
    } else {
        return ISS_ERR_INVALID_ARG;
    }
    return ok ? ISS_OK : ISS_ERR_IO;
}

iss_status iss_gpu_species(iss_handle* h, int32_t* n_species, int32_t* pids, int32_t capacity) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!h->surface_loaded) return fail(h, ISS_ERR_NO_SURFACE, "no surface");
    const int32_t n = static_cast<int32_t>(h->species.size());
    if (n_species) *n_species = n;
    if (!pids) return ISS_OK;
    if (capacity < n) return fail(h, ISS_ERR_CAPACITY, "%d species", n);
    for (int32_t k = 0; k < n; k++) pids[k] = h->species[k].pid;
    return ISS_OK;
}

iss_status iss_gpu_species_yields(iss_handle* h, double* dn_dy, int32_t capacity) {
    if (!h || !dn_dy) return ISS_ERR_INVALID_ARG;
    if (!h->yields_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no yields: call iss_gpu_generate first");
    const int32_t n = static_cast<int32_t>(h->species.size()) * h->cfg.n_surfaces;
    if (capacity < n) return fail(h, ISS_ERR_CAPACITY, "%d (surface, species) rows", n);
    CUDA_TRY(h, cudaMemcpy(dn_dy, h->d_totals.ptr, 8 * static_cast<size_t>(n), cudaMemcpyDeviceToHost));
    return ISS_OK;
}

iss_status iss_gpu_num_cells(iss_handle* h, int64_t* n_cells) {
    if (!h || !n_cells) return ISS_ERR_INVALID_ARG;
    *n_cells = h->n_cells;
    return ISS_OK;
}

iss_status iss_gpu_copy_lrf_cells(iss_handle* h, float* out, int64_t capacity_cells) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    if (!h->yields_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no cells on the device yet");
    if (capacity_cells < h->n_cells) return fail(h, ISS_ERR_CAPACITY, "too small");
    const int64_t n = h->n_cells;
    std::vector<float4> buf(static_cast<size_t>(n) * 8);
    CUDA_TRY(h, cudaMemcpy(buf.data(), h->d_cells.ptr, sizeof(float4) * buf.size(),
                           cudaMemcpyDeviceToHost));
    for (int64_t l = 0; l < n; l++) {
        const float4 pos = buf[l], da = buf[n + l], u = buf[2 * n + l], th = buf[3 * n + l];
        const float4 th2 = buf[4 * n + l], p1 = buf[5 * n + l], p2 = buf[6 * n + l];
        float* o = out + 28 * l;
        const float v[28] = {pos.x, pos.y, pos.z, pos.w, da.x, da.y, da.z, da.w, u.x, u.y,
                             u.z, u.w, th2.x, th.x, th2.y, th2.z, th.y, th.z, th.w, th2.w,
                             p1.x, p1.y, p1.z, p1.w, p2.x, p2.y, p2.z, p2.w};
        std::memcpy(o, v, sizeof(v));
    }
    return ISS_OK;
}

iss_status iss_gpu_copy_cell_yields(iss_handle* h, int32_t species_index, float* out,
                                    int64_t capacity_cells) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    if (!h->yields_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no yields yet");
    if (species_index < 0 || species_index >= static_cast<int32_t>(h->species.size()))
        return fail(h, ISS_ERR_INVALID_ARG, "species index %d out of range", species_index);
    if (capacity_cells < h->n_cells) return fail(h, ISS_ERR_CAPACITY, "too small");
    CUDA_TRY(h, cudaMemcpy(out, h->d_yields.ptr + static_cast<size_t>(species_index) * h->n_cells,
                           sizeof(float) * static_cast<size_t>(h->n_cells), cudaMemcpyDeviceToHost));
    return ISS_OK;
}

iss_status iss_gpu_copy_counts(iss_handle* h, int32_t* out, int64_t capacity) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    if (!h->samples_valid) return fail(h, ISS_ERR_NO_SAMPLES, "no samples");
    const int64_t n = static_cast<int64_t>(h->n_events) * static_cast<int64_t>(h->species.size());
    if (capacity < n) return fail(h, ISS_ERR_CAPACITY, "need %lld", static_cast<long long>(n));
    if (n > 0)
        CUDA_TRY(h, cudaMemcpy(out, h->d_counts.ptr, 4 * static_cast<size_t>(n), cudaMemcpyDeviceToHost));
    return ISS_OK;
}

iss_status iss_gpu_get_timings(iss_handle* h, iss_timings_t* out) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    *out = h->timings;
    return ISS_OK;
}


// ---- the learned proposal network -------------------------------------------

iss_status iss_gpu_mma_selftest(const uint16_t* a, const uint16_t* b, int32_t n, int32_t k,
                                float* c) {
    if (!a || !b || !c || n < 32 || n > 256 || (n % 32) != 0 || k < 16 || k > 256 || (k % 16) != 0)
        return ISS_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ISS_ERR_CUDA;
    void *da = nullptr, *db = nullptr;
    float* dc = nullptr;
    int* derr = nullptr;
    cudaStream_t s = nullptr;
    iss_status st = ISS_ERR_CUDA;
    int herr = 0;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
        cudaMalloc(&da, 2 * 128 * static_cast<size_t>(k)) == cudaSuccess &&
        cudaMalloc(&db, 2 * static_cast<size_t>(n) * k) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&dc), 4 * 128 * static_cast<size_t>(n)) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&derr), sizeof(int)) == cudaSuccess &&
        cudaMemcpyAsync(da, a, 2 * 128 * static_cast<size_t>(k), cudaMemcpyHostToDevice, s) == cudaSuccess &&
        cudaMemcpyAsync(db, b, 2 * static_cast<size_t>(n) * k, cudaMemcpyHostToDevice, s) == cudaSuccess &&
        cudaMemsetAsync(derr, 0, sizeof(int), s) == cudaSuccess &&
        launch_mma_selftest(da, db, n, k, dc, derr, s) == cudaSuccess &&
        cudaMemcpyAsync(c, dc, 4 * 128 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
        cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
        cudaStreamSynchronize(s) == cudaSuccess)
        st = herr == 0 ? ISS_OK : ISS_ERR_SAMPLING;
    if (da) cudaFree(da);
    if (db) cudaFree(db);
    if (dc) cudaFree(dc);
    if (derr) cudaFree(derr);
    if (s) cudaStreamDestroy(s);
    return st;
}

int64_t iss_gpu_learned_num_weights(void) { return mlp::kNumParams; }

iss_status iss_gpu_learned_init_weights(iss_handle* h, uint64_t seed) {
    if (!h) return ISS_ERR_INVALID_ARG;
    iss_status st = ensure_cuda(h);
    if (st != ISS_OK) return st;
    std::vector<float> p;
    Learned::initial_params(seed, &p);
    CUDA_TRY(h, h->learned.set_params(p.data(), h->stream));
    return ISS_OK;
}

iss_status iss_gpu_learned_set_weights(iss_handle* h, const float* weights, int64_t n) {
    if (!h || !weights) return ISS_ERR_INVALID_ARG;
    if (n != mlp::kNumParams)
        return fail(h, ISS_ERR_INVALID_ARG, "%lld weights given, the network has %lld",
                    static_cast<long long>(n), static_cast<long long>(mlp::kNumParams));
    iss_status st = ensure_cuda(h);
    if (st != ISS_OK) return st;
    CUDA_TRY(h, h->learned.set_params(weights, h->stream));
    return ISS_OK;
}

iss_status iss_gpu_learned_get_weights(iss_handle* h, float* out, int64_t capacity) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    if (!h->learned.have_weights) return fail(h, ISS_ERR_NO_SAMPLES, "the network has no weights yet");
    if (capacity < mlp::kNumParams) return fail(h, ISS_ERR_CAPACITY, "need %lld floats",
                                                static_cast<long long>(mlp::kNumParams));
    CUDA_TRY(h, h->learned.get_params(out, h->stream));
    return ISS_OK;
}

iss_status iss_gpu_learned_forward(iss_handle* h, const float* features, int64_t n, float* out) {
    if (!h || !features || !out || n < 0) return ISS_ERR_INVALID_ARG;
    if (!h->learned.have_weights) return fail(h, ISS_ERR_NO_SAMPLES, "the network has no weights yet");
    CUDA_TRY(h, h->learned.forward_host(features, n, out, h->num_sms, h->stream));
    if (h->learned.device_error(h->stream) != 0)
        return fail(h, ISS_ERR_SAMPLING, "a tensor-core wait of the forward pass timed out");
    return ISS_OK;
}

iss_status iss_gpu_learned_loss_grad(iss_handle* h, const float* features, const float* targets,
                                     int64_t n, double* loss, float* grad) {
    if (!h || !features || !targets || !loss || !grad || n <= 0) return ISS_ERR_INVALID_ARG;
    if (!h->learned.have_weights) return fail(h, ISS_ERR_NO_SAMPLES, "the network has no weights yet");
    CUDA_TRY(h, h->learned.loss_grad_host(features, targets, n, loss, grad, h->num_sms, h->stream));
    if (h->learned.device_error(h->stream) != 0)
        return fail(h, ISS_ERR_SAMPLING, "a tensor-core wait of the backward pass timed out");
    return ISS_OK;
}

iss_status iss_gpu_learned_stats(iss_handle* h, iss_learned_stats_t* out) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    *out = h->lstats;
    return ISS_OK;
}

iss_status iss_gpu_learned_train(iss_handle* h, const iss_learned_train_t* opt, double* loss_curve,
                                 int32_t capacity) {
    if (!h || !opt) return ISS_ERR_INVALID_ARG;
    if (opt->n_momenta < 0 || opt->n_seeds <= 0 || opt->n_steps < 0 || opt->batch <= 0 ||
        !(opt->learning_rate > 0.0))
        return fail(h, ISS_ERR_INVALID_ARG, "training options out of range");
    if (opt->n_momenta == 0) {
        // more steps on the rows already held
        Learned& L0 = h->learned;
        if (L0.n_data <= 0 || !L0.have_weights)
            return fail(h, ISS_ERR_NO_SAMPLES, "n_momenta = 0 needs training rows and weights");
        iss_status st0 = ensure_cuda(h);
        if (st0 != ISS_OK) return st0;
        const auto t0 = std::chrono::steady_clock::now();
        CUDA_TRY(h, L0.train(opt->n_steps, opt->batch, static_cast<float>(opt->learning_rate),
                             static_cast<uint32_t>(opt->init_seed),
                             static_cast<uint32_t>(opt->init_seed >> 32) ^ 0x7A11u, loss_curve,
                             h->num_sms, h->stream));
        h->lstats.ms_train =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (L0.device_error(h->stream) != 0)
            return fail(h, ISS_ERR_SAMPLING, "a tensor-core wait of the training step timed out");
        return ISS_OK;
    }
    if (loss_curve && capacity < opt->n_steps)
        return fail(h, ISS_ERR_CAPACITY, "the loss curve needs %d entries", opt->n_steps);
    if (!h->surface_loaded) return fail(h, ISS_ERR_NO_SURFACE, "no surface: call iss_gpu_read_surface first");
    iss_status st = ensure_cuda(h);
    if (st != ISS_OK) return st;
    if (h->params.get_or("local_charge_conservation", 0) == 1)
        return fail(h, ISS_ERR_UNSUPPORTED, "training rows with local_charge_conservation");
    if (!h->batch_cells.empty())
        return fail(h, ISS_ERR_UNSUPPORTED, "training rows from a batch of surfaces");
    // the plain sampler draws the training momenta; the caller's settings come back afterwards
    const char* keys[] = {"gpu_sampler", "perform_decays", "number_of_repeated_sampling",
                          "sample_upto_desired_particle_number", "gpu_event_offset"};
    double saved[5];
    bool had[5];
    for (int i = 0; i < 5; i++) had[i] = h->params.get(keys[i], &saved[i]);
    const int64_t saved_seed = h->seed;
    const bool saved_seed_set = h->seed_set;
    auto restore = [&]() {
        for (int i = 0; i < 5; i++) {
            if (had[i]) h->params.set(keys[i], saved[i]);
            else h->params.erase(keys[i]);
        }
        h->seed = saved_seed;
        h->seed_set = saved_seed_set;
        h->samples_valid = false;
    };
    h->params.set("gpu_sampler", 0);
    h->params.set("perform_decays", 0);
    h->params.set("sample_upto_desired_particle_number", 0);
    h->params.set("gpu_event_offset", 0);
    Learned& L = h->learned;
    // hadrons per event from a one-event generate
    h->params.set("number_of_repeated_sampling", 1);
    h->seed = opt->first_seed;
    st = run_generate(h);
    if (st != ISS_OK) {
        restore();
        return st;
    }
    double per_event = 0.0;
    {
        std::vector<double> tot(h->species.size());
        CUDA_TRY(h, cudaMemcpy(tot.data(), h->d_totals.ptr, 8 * tot.size(), cudaMemcpyDeviceToHost));
        for (double v : tot) per_event += v * h->cfg.ymult;
    }
    if (!(per_event > 0.0)) {
        restore();
        return fail(h, ISS_ERR_SAMPLING, "the surface emits no hadrons");
    }
    const int64_t per_seed = (opt->n_momenta + opt->n_seeds - 1) / opt->n_seeds;
    const int ev = static_cast<int>(std::min<double>(1e7, std::ceil(1.02 * per_seed / per_event) + 1));
    // sorted PDG ids -> species index
    {
        std::vector<std::pair<int32_t, int32_t>> sp;
        for (size_t k = 0; k < h->species.size(); k++)
            sp.emplace_back(h->species[k].pid, static_cast<int32_t>(k));
        std::sort(sp.begin(), sp.end());
        std::vector<int32_t> tab(2 * sp.size());
        for (size_t k = 0; k < sp.size(); k++) {
            tab[k] = sp[k].first;
            tab[sp.size() + k] = sp[k].second;
        }
        CUDA_TRY(h, h->d_spid.reserve(std::max<size_t>(tab.size(), 1)));
        CUDA_TRY(h, cudaMemcpy(h->d_spid.ptr, tab.data(), 4 * tab.size(), cudaMemcpyHostToDevice));
    }
    const int S = static_cast<int>(h->species.size());
    CUDA_TRY(h, L.data_x.reserve(static_cast<size_t>(opt->n_momenta) * mlp::kIn0));
    CUDA_TRY(h, L.data_t.reserve(static_cast<size_t>(opt->n_momenta)));
    CUDA_TRY(h, L.loss.reserve(std::max<size_t>(static_cast<size_t>(opt->n_steps), 1)));
    CUDA_TRY(h, cudaMemsetAsync(L.loss.ptr, 0, sizeof(double), h->stream));
    int64_t filled = 0;
    for (int k = 0; k < opt->n_seeds && filled < opt->n_momenta; k++) {
        h->params.set("number_of_repeated_sampling", ev);
        h->seed = static_cast<int64_t>(opt->first_seed) + k;
        st = run_generate(h);
        if (st != ISS_OK) {
            restore();
            return st;
        }
        const int64_t take = std::min<int64_t>({h->n_hadrons, per_seed, opt->n_momenta - filled});
        CUDA_TRY(h, launch_learned_train_rows(h->cfg, cell_arrays(h), h->d_species.ptr, h->d_spid.ptr,
                                              h->d_spid.ptr + S, S, h->d_hadrons.ptr, h->d_cell_of.ptr,
                                              take, L.data_x.ptr + filled * mlp::kIn0,
                                              L.data_t.ptr + filled, L.loss.ptr, h->stream));
        filled += take;
    }
    double nll_plain = 0.0;
    CUDA_TRY(h, cudaMemcpyAsync(&nll_plain, L.loss.ptr, sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    restore();
    L.n_data = filled;
    h->lstats.train_nll_plain = filled > 0 ? nll_plain / static_cast<double>(filled) : 0.0;
    h->lstats.n_train_rows = filled;
    h->lstats.train_events_per_seed = ev;
    if (!L.have_weights) {
        std::vector<float> p;
        Learned::initial_params(opt->init_seed, &p);
        CUDA_TRY(h, L.set_params(p.data(), h->stream));
    }
    const auto t0 = std::chrono::steady_clock::now();
    CUDA_TRY(h, L.train(opt->n_steps, opt->batch, static_cast<float>(opt->learning_rate),
                        static_cast<uint32_t>(opt->init_seed), static_cast<uint32_t>(opt->init_seed >> 32) ^ 0x7A11u,
                        loss_curve, h->num_sms, h->stream));
    h->lstats.ms_train = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (L.device_error(h->stream) != 0)
        return fail(h, ISS_ERR_SAMPLING, "a tensor-core wait of the training step timed out");
    return ISS_OK;
}

iss_status iss_gpu_learned_copy_rows(iss_handle* h, int64_t first, int64_t count, float* features,
                                     float* targets) {
    if (!h || first < 0 || count < 0) return ISS_ERR_INVALID_ARG;
    Learned& L = h->learned;
    if (first + count > L.n_data)
        return fail(h, ISS_ERR_CAPACITY, "%lld training rows held", static_cast<long long>(L.n_data));
    if (count == 0) return ISS_OK;
    if (features) {
        std::vector<uint16_t> x(static_cast<size_t>(count) * mlp::kIn0);
        CUDA_TRY(h, cudaMemcpy(x.data(), L.data_x.ptr + first * mlp::kIn0, 2 * x.size(),
                               cudaMemcpyDeviceToHost));
        for (int64_t r = 0; r < count; r++)
            for (int j = 0; j < mlp::kFeatures; j++) {
                const uint32_t b = static_cast<uint32_t>(x[r * mlp::kIn0 + j]) << 16;
                float v;
                std::memcpy(&v, &b, 4);
                features[r * mlp::kFeatures + j] = v;
            }
    }
    if (targets)
        CUDA_TRY(h, cudaMemcpy(targets, L.data_t.ptr + first, sizeof(float4) * count,
                               cudaMemcpyDeviceToHost));
    return ISS_OK;
}

// ---- launch shape -------------------------------------------------------------

iss_status iss_gpu_get_tuning(iss_handle* h, iss_tuning_t* out) {
    if (!h || !out) return ISS_ERR_INVALID_ARG;
    *out = h->tune;
    return ISS_OK;
}

iss_status iss_gpu_set_tuning(iss_handle* h, const iss_tuning_t* t) {
    if (!h || !t) return ISS_ERR_INVALID_ARG;
    if (!tuning_valid(*t))
        return fail(h, ISS_ERR_INVALID_ARG,
                    "launch shape out of range (item_size %d, yield_groups %d, sampler_ctas %d, "
                    "assign_blocks %d, copy_chunks %d)",
                    t->item_size, t->yield_groups, t->sampler_ctas, t->assign_blocks, t->copy_chunks);
    h->tune = *t;
    h->tuned = true;
    return ISS_OK;
}

iss_status iss_gpu_autotune(iss_handle* h, iss_tuning_t* best, double* ms_before, double* ms_after) {
    if (!h) return ISS_ERR_INVALID_ARG;
    if (!h->seed_set) {
        iss_status st = iss_gpu_set_seed_from_params(h);
        if (st != ISS_OK) return st;
    }
    const iss_status st = autotune(h, ms_before, ms_after);
    if (st != ISS_OK) return st;
    if (best) *best = h->tune;
    return ISS_OK;
}

}  // extern "C"
