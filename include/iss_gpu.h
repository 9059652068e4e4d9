/*
 * iss_gpu.h -- C ABI of the GB300 Cooper-Frye sampler (the "FSSW" path of
 * iSS, MC_sampling = 4).
 *
 * Every entry point replaces one public member of the reference's driver class
 * `iSS` (src/iSS.h:16-102) or one step behind it; the citation next to each
 * declaration names the reference interface it stands in for.  The ABI uses
 * plain pointers and sizes only.  Every call returns an iss_status instead of
 * calling exit() the way the reference does (src/iSS.cpp:45-53,
 * src/ParameterReader.cpp:150-159, src/readindata.cpp:50-55, 411-415, 933-935,
 * src/FSSW.cpp:254-259, 897-902, src/MomentumSamplerBase.cpp:35-43); the
 * message of the last failure is available from iss_gpu_last_error().
 *
 * Threading: a handle owns its CUDA stream, its device buffers and its host
 * copies; handles are independent, one handle must not be used from two
 * threads at the same time.  There is no CPU fallback: when no CUDA device is
 * usable, the calls that need one return ISS_ERR_CUDA.
 */
#ifndef ISS_GPU_H
#define ISS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct iss_handle iss_handle;

typedef enum iss_status {
    ISS_OK = 0,
    ISS_ERR_INVALID_ARG = 1,   /* NULL handle/pointer, bad index, bad size     */
    ISS_ERR_IO = 2,            /* a parameter, surface or table file missing   */
    ISS_ERR_PARAM_MISSING = 3, /* ParameterReader::getVal of an unknown key    */
    ISS_ERR_UNSUPPORTED = 4,   /* MC_sampling != 4, PCE surfaces, missing 22-moment table, ... */
    ISS_ERR_CUDA = 5,          /* no device, launch or allocation failure      */
    ISS_ERR_OUT_OF_RANGE = 6,  /* m/T - mu/T outside the momentum tables, negative yield, NaN */
    ISS_ERR_NO_SURFACE = 7,    /* generate before a surface was read           */
    ISS_ERR_NO_SAMPLES = 8,    /* hadron access before generate                */
    ISS_ERR_CAPACITY = 9,      /* caller buffer too small                      */
    ISS_ERR_SAMPLING = 10      /* a bounded device loop gave up (counted, see timings) */
} iss_status;

/* Layout-identical to the reference's iSS_Hadron (src/data_struct.h:79-84):
 * int pid followed by nine floats, 40 bytes. */
typedef struct iss_hadron {
    int32_t pid;
    float mass;
    float E, px, py, pz;
    float t, x, y, z;
} iss_hadron_t;

/* Output formats of iss_gpu_write_output, as selected in the reference by
 * use_OSCAR_format / use_gzip_format / use_binary_format (src/FSSW.cpp:354-360). */
typedef enum iss_output_format {
    ISS_OUTPUT_OSCAR = 1,   /* FSSW::combine_samples_to_OSCAR,       src/FSSW.cpp:365-494 */
    ISS_OUTPUT_GZIP = 2,    /* FSSW::combine_samples_to_gzip_file,   src/FSSW.cpp:497-526 */
    ISS_OUTPUT_BINARY = 3   /* FSSW::combine_samples_to_binary_file, src/FSSW.cpp:529-561 */
} iss_output_format;

/* Device-side time of the phases of the last iss_gpu_generate, measured with
 * CUDA events on the handle's stream, plus the counters of the bounded loops. */
typedef struct iss_timings {
    double ms_prologue;   /* local-rest-frame transform + per-cell delta-f coefficients */
    double ms_yields;     /* per (cell, species) yields                               */
    double ms_cdf;        /* per-species fixed-point prefix sums (cell CDF), totals   */
    double ms_counts;     /* per (event, species) counts + slot scan                  */
    double ms_sample;     /* momentum sampling, boost, emission                       */
    double ms_total;      /* first event to last event of iss_gpu_generate            */
    int64_t n_hadrons;    /* hadrons written                                          */
    int64_t n_tries;      /* proposals made by the sampler                            */
    int64_t n_cell_redraws;  /* cells redrawn after the try cap (src/FSSW.cpp:1017-1021) */
    int64_t n_failures;   /* hadrons abandoned after the redraw cap (never expected)  */
    int32_t kernel_launches; /* kernels launched by the last iss_gpu_generate (without decays) */
    double ms_decays;     /* resonance decays (perform_decays = 1), not in ms_total   */
    int32_t decay_reruns; /* decay passes rerun because a buffer was too small (the
                             sizes are then kept for later calls; results unchanged) */
    int64_t n_sampled;    /* hadrons the sampler wrote (before resonance decays)      */
} iss_timings_t;

/* ---- construction, parameters ------------------------------------------ */

/* iSS::iSS(path, table_path, particle_table_path, inputfile, surface_filename)
 * (src/iSS.h:43-46, src/iSS.cpp:14-24): reads `param_file` with the
 * ParameterReader rules (src/ParameterReader.cpp:33-106).  NULL strings take
 * the reference defaults ("iSS_tables", "iSS_tables", "iSS_parameters.dat",
 * "surface.dat"); work_path has no default. */
iss_status iss_gpu_create(const char* work_path, const char* table_path,
                          const char* particle_table_path, const char* param_file,
                          const char* surface_filename, iss_handle** out);

/* iSS::~iSS (src/iSS.cpp:27-30); accepts NULL. */
iss_status iss_gpu_destroy(iss_handle* h);

/* paraRdr_ptr->setVal(name, value) (src/ParameterReader.cpp:130-144). */
iss_status iss_gpu_set_param(iss_handle* h, const char* key, double value);

/* paraRdr_ptr->getVal(name) (src/ParameterReader.cpp:150-159); an unknown key
 * returns ISS_ERR_PARAM_MISSING instead of exiting. */
iss_status iss_gpu_get_param(iss_handle* h, const char* key, double* value);

/* paraRdr_ptr->readFromArguments for one "key=value  # comment" string
 * (src/ParameterReader.cpp:76-83, 110-116; src/main.cpp:61). */
iss_status iss_gpu_parse_param_line(iss_handle* h, const char* line);

/* ---- seed, surface, sampling --------------------------------------------- */

/* iSS::set_random_seed(int) (src/iSS.cpp:123-127).  seed == -1 draws a seed
 * from the OS like std::random_device (src/Random.cpp:10-12). */
iss_status iss_gpu_set_seed(iss_handle* h, int64_t seed);

/* iSS::set_random_seed() (src/iSS.cpp:116-120): seed from key randomSeed. */
iss_status iss_gpu_set_seed_from_params(iss_handle* h);

/* iSS::read_in_FO_surface (src/iSS.cpp:86-113): reads <work_path>/music_input
 * and the MUSIC surface (text or 34-float binary, hydro_mode 1 or 2,
 * src/readindata.cpp:25-111, 395-546, 626-765), the species tables
 * (src/readindata.cpp:971-1116) and uploads the cells; the local-rest-frame
 * transform (src/iSS.cpp:170-293) runs on the device at generate time. */
iss_status iss_gpu_read_surface(iss_handle* h);

/* In-memory surface: n_cells records in the reference's FO_surf field order
 * and units (src/data_struct.h:53-63 without the PCE vector: tau, x, y, eta,
 * da0..da3, u0..u3, Edec, Tdec, Pdec, Bn, muB, muS, muQ, pi00, pi01, pi02,
 * pi03, pi11, pi12, pi13, pi22, pi23, pi33, bulkPi, qmu0..qmu3 -- 34 floats,
 * GeV and fm), i.e. what read_FOdata produces before regulate_surface_cells
 * (src/readindata.cpp:768-842) runs.  Species tables are read as in
 * iss_gpu_read_surface; music_input is not needed (EOS_to_use = 2). */
iss_status iss_gpu_set_surface(iss_handle* h, const float* fo_surf_records,
                               int64_t n_cells);

/* A batch of independent surfaces sampled by one iss_gpu_generate (no
 * counterpart in the reference, which holds one surface per iSS object).
 *   - Surface b has the FO_surf records
 *     [cell_offsets[b], cell_offsets[b+1]) of `fo_surf_records`.
 *   - cell_offsets[0] = 0, n_surfaces + 1 entries.
 *   - Surface b gets events[b] events, which replaces
 *     number_of_repeated_sampling.
 *   - Events are numbered across the batch: surface 0's events come first,
 *     then surface 1's, and so on. iss_gpu_num_events returns the sum.
 *   - Every kernel runs once over the whole batch.
 *   - Surface b's events are bit-identical to a single-surface run of b with
 *     the same seed and gpu_event_offset raised by the events of surfaces
 *     0 .. b-1.
 *   - iss_gpu_species_yields then returns n_surfaces * n_species values,
 *     row b * n_species + k.
 *   - Fewer than 2^31 cells and events in total.
 *   - iss_gpu_set_surface or iss_gpu_read_surface ends batch mode. */
iss_status iss_gpu_set_surface_batch(iss_handle* h, const float* fo_surf_records,
                                     const int64_t* cell_offsets, const int32_t* events,
                                     int32_t n_surfaces);

/* iSS::generate_samples (src/iSS.cpp:130-165) for MC_sampling = 4, i.e.
 * FSSW::shell (src/FSSW.cpp:344-361) without the optional decays and
 * spectators: yields, counts, momenta and the hadron lists, all on the GPU. */
iss_status iss_gpu_generate(iss_handle* h);

/* iSS::generate_samples followed by reading every event's hadron list
 * (get_hadron_list_iev for iev = 0 .. n_events-1, src/iSS.h:85-91) in one call.
 *   - The sampler runs in up to 16 chunks of consecutive events.
 *   - Each chunk's records are copied into out[0 .. n_total) while the next
 *     chunk is sampled.
 *   - `out` should be page-locked (cudaHostAlloc or cudaHostRegister). Then
 *     the copies run beside the sampling.
 *   - The hadrons and their order are those of iss_gpu_generate followed by
 *     iss_gpu_copy_all.
 *   - If capacity is too small, the samples stay on the device. The call
 *     returns ISS_ERR_CAPACITY and sets *n_total to the size needed.
 *   - Event offsets come from iss_gpu_copy_all(h, NULL, 0, offsets, NULL). */
iss_status iss_gpu_generate_into(iss_handle* h, iss_hadron_t* out, int64_t capacity,
                                 int64_t* n_total);

/* Streamed generate (no counterpart in the reference, whose hadron lists all
 * stay in host memory): the same sampling as iss_gpu_generate, with the
 * hadrons handed to `fn` chunk by chunk instead of kept.  Events are taken
 * chunk_events at a time; fn(user, hadrons, n, first_event, n_events,
 * offsets) receives the n hadrons of events [first_event, first_event +
 * n_events) in a page-locked buffer of the library, event k's records at
 * [offsets[k], offsets[k+1]).  The buffer is valid until fn returns.  fn runs
 * on the calling thread while the next chunk is being sampled on the device,
 * and the device holds the records of two chunks only, so runs whose hadrons
 * would not fit in device memory at once (large batches, many oversampled
 * events) stream through a bounded buffer.  The hadrons are the ones
 * iss_gpu_generate draws for the same seed, bit for bit.  Afterwards the
 * handle holds timings and counts but no hadrons (the accessors return
 * ISS_ERR_NO_SAMPLES).  perform_decays needs every event on the device and
 * returns ISS_ERR_UNSUPPORTED here.  fn must not call the library with the
 * same handle (the generate is still running) and must not let a C++
 * exception escape into this C call. */
typedef void (*iss_stream_fn)(void* user, const iss_hadron_t* hadrons, int64_t n_hadrons,
                              int32_t first_event, int32_t n_events, const int64_t* event_offsets);
iss_status iss_gpu_generate_stream(iss_handle* h, int32_t chunk_events, iss_stream_fn fn, void* user);

/* iSS::shell (src/iSS.cpp:41-56): read_surface + set_seed_from_params +
 * generate. */
iss_status iss_gpu_shell(iss_handle* h);

/* iSS::clear (src/iSS.cpp:33-38): drops the surface and the samples. */
iss_status iss_gpu_clear(iss_handle* h);

/* ---- results --------------------------------------------------------------- */

/* iSS::get_number_of_sampled_events (src/iSS.h:61-67, src/FSSW.h:173). */
iss_status iss_gpu_num_events(iss_handle* h, int32_t* n_events);

/* iSS::get_number_of_particles(iev) (src/iSS.h:69-75, src/FSSW.h:174-176). */
iss_status iss_gpu_num_particles(iss_handle* h, int32_t iev, int64_t* n);

/* iSS::get_hadron(iev, ipart) (src/iSS.h:77-83, src/FSSW.h:178-180). */
iss_status iss_gpu_get_hadron(iss_handle* h, int32_t iev, int64_t ipart,
                              iss_hadron_t* out);

/* iSS::get_hadron_list_iev(iev) (src/iSS.h:85-91, src/FSSW.h:182-184): copies
 * event iev (species in mass order, then draw order) into `out`. */
iss_status iss_gpu_copy_event(iss_handle* h, int32_t iev, iss_hadron_t* out,
                              int64_t capacity, int64_t* n_written);

/* All events at once: out[0 .. n_total), event_offsets[0 .. n_events]
 * (event iev is out[event_offsets[iev] .. event_offsets[iev+1])).  Either
 * output pointer may be NULL to query sizes only. */
iss_status iss_gpu_copy_all(iss_handle* h, iss_hadron_t* out, int64_t capacity,
                            int64_t* event_offsets, int64_t* n_total);

/* Writes the hadron lists in one of the reference's output formats
 * (src/FSSW.cpp:365-561) to `filename` (NULL: the reference's default name in
 * the current directory: OSCAR.DAT, particle_samples.gz, particle_samples.bin). */
iss_status iss_gpu_write_output(iss_handle* h, int format, const char* filename);

/* The same writers on a caller's host hadron list (no device work, no
 * handle): FSSW::combine_samples_to_OSCAR / _gzip_file / _binary_file
 * (src/FSSW.cpp:365-561) applied to events [event_offsets[i],
 * event_offsets[i+1]) of `hadrons`, i < n_events.  For example the
 * concatenated hadrons of event shards sampled on several GPUs.  The OSCAR
 * header is read from <table_path>/OSCAR_header.txt, as the reference reads
 * it (src/FSSW.cpp:164); table_path NULL means "iSS_tables".  filename NULL
 * takes the reference's default name. */
iss_status iss_gpu_write_hadron_list(int format, const char* filename, const char* table_path,
                                     const iss_hadron_t* hadrons, const int64_t* event_offsets,
                                     int32_t n_events);

/* ---- inspection (parity tests, run reports) ---------------------------- */

/* Number of chosen species and their PDG ids in the sampler's mass-sorted
 * order (src/FSSW.cpp:115-162). */
iss_status iss_gpu_species(iss_handle* h, int32_t* n_species, int32_t* pids,
                           int32_t capacity);

/* Per-species FP64 yields dN/dy summed over cells (the value the reference
 * logs as "Sampling using dN_dy=", src/FSSW.cpp:943-961), in mass order. */
iss_status iss_gpu_species_yields(iss_handle* h, double* dn_dy, int32_t capacity);

/* Number of cells held on the device (after the T > 0.01 GeV filter of
 * src/readindata.cpp:751-761; cells dropped by the u.dsigma < 0 rule of
 * src/iSS.cpp:226 are kept with zero yield). */
iss_status iss_gpu_num_cells(iss_handle* h, int64_t* n_cells);

/* Local-rest-frame cells, 28 floats per cell in the FO_surf_LRF order of
 * src/data_struct.h:66-76 (tau, x, y, eta, da_mu_LRF[4], u_tz[4], Edec, Tdec,
 * Pdec, Bn, muB, muS, muQ, bulkPi, pi_xx, pi_xy, pi_xz, pi_yy, pi_yz, q_x, q_y,
 * q_z); dropped cells have da_mu_LRF[0] < 0. */
iss_status iss_gpu_copy_lrf_cells(iss_handle* h, float* out, int64_t capacity_cells);

/* Per-cell yields dN/(dx_t dy) of species `species_index` (mass order), the
 * vector FSSW::calculate_dN_dxtdy_for_one_particle_species fills
 * (src/FSSW.cpp:565-715). */
iss_status iss_gpu_copy_cell_yields(iss_handle* h, int32_t species_index,
                                    float* out, int64_t capacity_cells);

/* Hadron records per (event, species), event-major, of the last generate
 * (src/FSSW.cpp:970-977).  Under local_charge_conservation, a positively
 * charged species counts two records per draw (hadron and partner), and a
 * negatively charged one counts 0. */
iss_status iss_gpu_copy_counts(iss_handle* h, int32_t* out, int64_t capacity);

/* Timings and loop counters of the last iss_gpu_generate. */
iss_status iss_gpu_get_timings(iss_handle* h, iss_timings_t* out);

/* Message of the last failure on this handle ("" if none). */
const char* iss_gpu_last_error(const iss_handle* h);

/* Static name of a status code. */
const char* iss_gpu_status_string(int status);

/* ---- launch shape and autotuning -----------------------------------------
 *
 * No counterpart in the reference (its loops are serial).  The launch shape
 * of the kernels never changes a result: every random number is keyed by
 * (draw, hadron, event, species), so any shape gives the same hadrons bit
 * for bit.  It changes only the time. */
typedef struct iss_tuning {
    int32_t item_size;      /* draws per sampler work item: 32, 64, ..., 1024 (default 64) */
    int32_t yield_groups;   /* species groups per cell in the yields kernel: 1..32 (4)     */
    int32_t sampler_ctas;   /* sampler blocks of 256 threads per SM: 1..3 (3)               */
    int32_t assign_blocks;  /* cell-assignment blocks per SM: 1..32 (8)                     */
    int32_t copy_chunks;    /* event chunks copied out by iss_gpu_generate_into: 1..64 (16) */
} iss_tuning_t;
iss_status iss_gpu_get_tuning(iss_handle* h, iss_tuning_t* out);
iss_status iss_gpu_set_tuning(iss_handle* h, const iss_tuning_t* tuning);
/* Times the handle's own workload (its surface and parameters) under
 * candidate launch shapes and keeps the fastest: species groups per cell by
 * the yields phase, then draws per work item, sampler blocks per SM and
 * cell-assignment blocks per SM by the sample phase (coordinate descent, two
 * generates per candidate, a 2 % margin to switch).  The result is cached per
 * workload shape (cells, surfaces, events, species, local charge
 * conservation, sampler, hydro mode) for every handle of the process; with
 * gpu_autotune = 1 the first generate of a new shape tunes or takes the
 * cached shape.  Leaves the samples of its last trial; ms_before / ms_after
 * (optional) are the device times of one generate. */
iss_status iss_gpu_autotune(iss_handle* h, iss_tuning_t* best, double* ms_before, double* ms_after);

/* ---- the learned proposal ------------------------------------------------
 *
 * No counterpart in the reference: the reference has one momentum sampler
 * (FSSW::sample_momemtum_from_a_fluid_cell, src/FSSW.cpp:1852-1966).  The
 * learned sampler keeps that sampler's target density and accept step and
 * changes only where proposals come from: a mixture of the plain proposal
 * and a conditional density network (18 features of the cell and species ->
 * 4 x 128 ReLU -> an 8-component log-normal x von Mises-Fisher mixture over
 * the rest-frame momentum).  The network runs on the tensor cores (bf16
 * weights, FP32 accumulation) for training and inference.
 *
 * Features of a (cell, species) pair, in this order (rest-frame cell values):
 *   (T - 0.15) / 0.02, (mu / T) / 2, pi_xx, pi_xy, pi_xz, pi_yy, pi_yz each
 *   / (e + P) / 0.1, Pi / (e + P) / 0.05, (0, q_x, q_y, q_z) / (e + P) / 0.1,
 *   dsigma_mu / (|dsigma_0| + |dsigma_vec|), (m / T) / 10, statistics sign.
 * Targets: (K, n_x, n_y, n_z) with K = (E - m) / T and n = p / |p|.
 * Network outputs (64 per row, 48 used): 8 logits, 8 locations of ln K,
 * 8 ln sigma, 8 x 3 vectors v (direction v / |v|, concentration |v|). */

/* Number of FP32 weights of the network (flat layout: per layer W[out][in]
 * row-major, then b[out]). */
int64_t iss_gpu_learned_num_weights(void);
/* Deterministic initial weights from a seed. */
iss_status iss_gpu_learned_init_weights(iss_handle* h, uint64_t seed);
iss_status iss_gpu_learned_set_weights(iss_handle* h, const float* weights, int64_t n);
iss_status iss_gpu_learned_get_weights(iss_handle* h, float* out, int64_t capacity);
/* Network outputs for n feature rows (host FP32 [n][18] -> host FP32 [n][64]). */
iss_status iss_gpu_learned_forward(iss_handle* h, const float* features, int64_t n, float* out);
/* Mean negative log-likelihood of n targets (host FP32 [n][4]) and its
 * gradient with respect to the weights (host FP32 [num_weights]). */
iss_status iss_gpu_learned_loss_grad(iss_handle* h, const float* features, const float* targets,
                                     int64_t n, double* loss, float* grad);
/* Training of the network (no counterpart in the reference).  The plain
 * sampler draws n_momenta hadrons on the handle's surface with the handle's
 * parameters, split evenly over the seeds first_seed .. first_seed + n_seeds
 * - 1 (resonance decays off); each hadron becomes one training row: its
 * (cell, species) features and its rest-frame (K, n).  Then n_steps Adam
 * steps minimise the mean negative log-likelihood of the mixture on batches
 * of `batch` rows drawn with replacement (forward, loss, backward and update
 * on the tensor cores, replayed as one CUDA graph per step).  A network
 * without weights starts from iss_gpu_learned_init_weights(init_seed).  The
 * handle's parameters and seed are restored afterwards; the rows stay on the
 * device for further calls.  loss_curve (optional, capacity >= n_steps)
 * receives the mean loss of every step. */
typedef struct iss_learned_train {
    int64_t n_momenta;       /* training rows (the rows of the last call are replaced);
                                0: more steps on the rows and weights already held */
    int32_t first_seed;
    int32_t n_seeds;
    int32_t n_steps;
    int32_t batch;
    double learning_rate;
    uint64_t init_seed;      /* initial weights and batch draws */
} iss_learned_train_t;
iss_status iss_gpu_learned_train(iss_handle* h, const iss_learned_train_t* options,
                                 double* loss_curve, int32_t capacity);

/* Sampling with the learned proposal: gpu_sampler = 1.  Species whose
 * expected hadrons per cell over all events reach
 * gpu_learned_min_hadrons_per_cell (default 1) are proposed from
 * gpu_learned_alpha (default 0.8) x network mixture + (1 - alpha) x the
 * plain proposal q_P; the others keep the plain sampler.  M per (species,
 * cell) is gpu_learned_safety (default 1.15) times the largest ratio
 * P a / q over gpu_learned_pilot pilot proposals (default 4 in exact mode,
 * 64 with gpu_learned_exact = 0), capped by 1 / (1 - alpha).  Target: the plain sampler's P a (a <= 1 its acceptance).
 *   gpu_learned_exact = 1 (default): exact rejection for every M.  A try is
 *     the mixture branch with probability M / (M + c): x from q, accepted
 *     with min(1, P a / (M q)); else the excess branch: x from the plain
 *     proposal, accepted with (P a - M q) / (c P), c = 1 - M (1 - alpha)
 *     (plus a rounding margin) >= sup (a - M q / P).  The accepted density
 *     is min(P a, M q) + (P a - M q)+ = P a whatever M is.  n_violations
 *     counts excess-branch ratios above 1 (none by construction).
 *   gpu_learned_exact = 0: the mixture branch alone; ratios above 1 are
 *     accepted and counted as violations (the output is then the target
 *     only where M q >= P a). */
typedef struct iss_learned_stats {
    int32_t n_species;       /* species sampled with the learned proposal   */
    int64_t n_pairs;         /* (species, cell) pairs evaluated by the network */
    double ms_network;       /* pair inputs + network + mixture records + envelopes */
    int64_t n_tries;         /* proposals made for those species           */
    int64_t n_hadrons;       /* hadrons of those species                    */
    int64_t n_violations;    /* proposals whose ratio exceeded 1            */
    int64_t n_train_rows;    /* training rows held on the device            */
    double ms_train;         /* wall time of the Adam steps of the last training */
    int32_t train_events_per_seed;  /* events of each plain run that drew training rows */
    double train_nll_plain;  /* mean -ln P of the training rows under the plain proposal
                                (same units as the network's loss) */
    double ms_forward;       /* the network's forward pass alone (part of ms_network) */
    int64_t n_excess_tries;  /* exact mode: proposals of the excess branch (in n_tries) */
    int64_t n_excess_hadrons;/* exact mode: hadrons accepted by the excess branch      */
    int64_t n_over_one;      /* exact mode: mixture-branch ratios above 1 (their
                                missing mass is what the excess branch supplies) */
} iss_learned_stats_t;
iss_status iss_gpu_learned_stats(iss_handle* h, iss_learned_stats_t* out);
/* Training rows first .. first + count - 1 of the last training: features
 * (FP32 [count][18], the bf16 values the network reads) and targets
 * (FP32 [count][4]); either pointer may be NULL. */
iss_status iss_gpu_learned_copy_rows(iss_handle* h, int64_t first, int64_t count, float* features,
                                     float* targets);

/* Self-test of the tensor-core GEMM the network is built from:
 * c[128][n] = a[128][k] * b[n][k]^T with bf16 inputs (raw 16-bit patterns,
 * row-major) and FP32 output; n in {32, 64, ..., 256}, k in {16, 32, ..., 256}. */
iss_status iss_gpu_mma_selftest(const uint16_t* a, const uint16_t* b, int32_t n, int32_t k,
                                float* c);

/* ---- count-to-slot scan without allocation ----------------------------- */

/* No counterpart in the reference.  Callers that cannot allocate device
 * memory use it: a program whose memory pool already holds the device, or a
 * pipeline where cudaFree's device-wide wait would stall other streams.
 *
 * Exclusive prefix sum of n hadron counts (device pointer d_counts) into
 * d_offsets[0 .. n] (device pointer; d_offsets[n] = total).  It is the scan
 * iss_gpu_generate uses to turn per-(event, species) counts into output
 * slots.  Its tile partial sums live in one fixed device array of 128 KiB
 * instead of a handle buffer, so it allocates nothing.
 *   - n > ISS_GPU_NOALLOC_SCAN_MAX_SEGMENTS returns ISS_ERR_CAPACITY before
 *     any device work.
 *   - The work is enqueued on `stream` (a cudaStream_t; NULL is the legacy
 *     default stream).  The results are ready when that stream reaches this
 *     point.
 *   - Nothing has to be zeroed before the call.
 *   - The fixed array is shared by all calls on one device.  Calls on one
 *     device must not overlap in time; issue them on one stream.
 *   - Counts must be >= 0; negative counts give wrong offsets (not checked).
 *   - The first call on each device looks up the array's address.  With
 *     CUDA's lazy module loading (the default) that lookup loads the module
 *     holding the array, which takes its 128 KiB of device memory then.  So
 *     make the first call on a device before a memory pool claims that
 *     device's memory, and before starting any stream capture on it.  Later
 *     calls allocate nothing.
 *   - A CUDA error that earlier work left pending makes the call return
 *     ISS_ERR_CUDA without launching anything; that error stays pending. */
#define ISS_GPU_NOALLOC_SCAN_MAX_SEGMENTS ((int64_t)16384 * 4096)
iss_status iss_gpu_scan_counts_noalloc(const int32_t* d_counts, int64_t n,
                                       int64_t* d_offsets, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ISS_GPU_H */
