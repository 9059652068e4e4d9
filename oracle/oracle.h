/* Test infrastructure only -- the ORACLE for the GB300 sampler.
 *
 * A CPU restatement, in FP64 C, of the reference's Cooper-Frye sampling path
 * (iSS, MC_sampling = 4, "FSSW").  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline; the product library never links or calls it.
 *
 * Three parts:
 *  1. orc_lrf_cells / orc_cell_coeffs / orc_yields: a direct restatement of
 *     regulate_surface_cells + transform_to_local_rest_frame + the delta-f
 *     coefficient lookups + calculate_dN_dxtdy_for_one_particle_species, pinned
 *     against per-cell yields dumped by the reference itself (tests/golden).
 *  2. orc_counts / orc_sample_replay: a replay, in FP64, of the GPU algorithm
 *     on the same Philox4x32-10 streams, so that integer outputs (counts, cell
 *     choices, species, PDG ids) can be compared bit for bit and momenta to
 *     FP32 rounding.
 *  3. orc_reference_sampler: the reference's own sampling algorithm
 *     (inverse-CDF momentum tables, nested rejection loops, per-hadron
 *     coefficient lookups, Mersenne-twister uniforms), used as the timed CPU
 *     baseline and as an independent statistical check.
 *
 * Parity: part 1 is pinned by the golden per-cell yields generated with the
 * reference compiled from its own sources (tests/golden/make_golden.py);
 * part 3 is compared with the reference's samples statistically. */
#ifndef ISS_ORACLE_H
#define ISS_ORACLE_H
#include <stdint.h>

#define ORC_HBARC 0.197327053
#define ORC_SF_LEN 7991        /* x in [0.5, 400], dx = 0.05 (src/FSSW.cpp:1611-1615) */
#define ORC_SF_X0 0.5
#define ORC_SF_DX 0.05
#define ORC_SF_XMAX 400.0
#define ORC_N_EXPINT 9         /* E_2, E_4, ..., E_18 (src/FSSW.cpp:1636-1640) */

typedef struct orc_species {
    int32_t pid;
    int32_t real_idx;
    double mass;
    int32_t gspin, baryon, strange, charge, sign;
} orc_species;

typedef struct orc_cfg {
    int32_t hydro_mode;
    int32_t include_shear, include_bulk, include_diff;
    int32_t bulk_kind;          /* bulk_deltaf_kind */
    int32_t neos_kind;          /* -1 none, 0: 22-moment, 1: Chapman-Enskog */
    double y_lb, y_rb;
    int32_t sampling_model;     /* dN_dy_sampling_model */
    double sampling_para1;
    int64_t n_events;
    int64_t event_offset;       /* first global event index (sharded runs) */
    uint64_t seed;
    int32_t compat_fermion;     /* 1: reproduce the reference's fermion CDF_2 term */
    int32_t max_tries;          /* proposals per cell before the cell is redrawn */
    int32_t max_redraws;
    int32_t lcc;                /* local_charge_conservation */
    /* special-function tables, ORC_SF_LEN rows */
    const double* sf_K;         /* [row][3] = K1, K2, K3 */
    const double* sf_E;         /* [row][9] = E_2, E_4, ..., E_18 */
    /* OSU 14-moment bulk tables, [iT * nmu + imu] */
    int32_t b14_nT, b14_nmu;
    double b14_T0, b14_mu0, b14_dT, b14_dmu;
    const double *b14_c0, *b14_c1, *b14_c2;
    /* NEoS-BQS Chapman-Enskog table: 200 x 200 rows of (e, nB, c2, zeta, eta) */
    const double* ce_tb;
    /* diffusion coefficient table, [iT * 100 + imu], 150 x 100 */
    const double* qmu_tb;
} orc_cfg;

/* Hadron record of the replay: same field order as iSS_Hadron. */
typedef struct orc_hadron {
    int32_t pid;
    float mass, E, px, py, pz, t, x, y, z;
} orc_hadron;

typedef struct orc_stats {
    int64_t n_tries;
    int64_t n_redraws;
    int64_t n_failures;
    int64_t n_bound_violations;
} orc_stats;

/* Part 1 */
void orc_sf_tables(int include_bulk, int include_diff, double* sf_K, double* sf_E);
double orc_sf_K(const orc_cfg* c, int which, double arg);   /* which = 1, 2, 3 */
void orc_lrf_cells(const float* fo34, int64_t n, float* lrf28, int32_t* keep);
void orc_cell_coeffs(const orc_cfg* c, const float* lrf28, int64_t n, double* coef4);
int orc_yields(const orc_cfg* c, const orc_species* sp, int32_t n_sp,
               const float* lrf28, const int32_t* keep, int64_t n, double* yields);
void orc_cdf(const float* yields_f32, int32_t n_sp, int64_t n, uint64_t* cdf, uint64_t* qtot,
             double* totals);

/* Part 2 */
int orc_counts(const orc_cfg* c, const orc_species* sp, int32_t n_sp, const double* totals,
               int32_t* counts);
int64_t orc_sample_replay(const orc_cfg* c, const orc_species* sp, int32_t n_sp,
                          const float* lrf28, int64_t n_cells, const float* coef4,
                          const uint64_t* cdf, const uint64_t* qtot, const int32_t* counts,
                          orc_hadron* out, int64_t capacity, orc_stats* stats);

/* Part 2c: resonance decays (oracle_decay.c).  The decay table as
 * particle_decay::read_resonances_list reads it (src/particle_decay.cpp:33-160):
 * one entry per particle, anti-baryons appended after their baryon; stable
 * when the first channel has one daughter; daughters as indices of the first
 * entry with their pid (-1: unknown); cum53 = ceil(2^53 x the FP64 partial
 * sum of the particle's branching ratios in channel order). */
typedef struct orc_dparticle {
    int32_t pid;
    double mass, width;
    int32_t stable, first_channel, n_channels;
} orc_dparticle;

typedef struct orc_dchannel {
    int32_t n_daughters;
    int32_t daughter[5];
    uint64_t cum53;
} orc_dchannel;

/* the final-state lists of events [0, n_events) whose sampled hadrons are
 * in[ev_off[e] .. ev_off[e + 1]): out (capacity records) and out_off
 * (n_events + 1); returns the number of records, -1 when out is too small,
 * -2 on allocation failure; *failures counts 3-body decays without an
 * accepted (E1, E2) */
int64_t orc_decay_replay(const orc_dparticle* parts, int32_t n_parts, const orc_dchannel* chans,
                         uint64_t seed, int64_t event_offset, int32_t n_events, const int64_t* ev_off,
                         const orc_hadron* in, int64_t capacity, orc_hadron* out, int64_t* out_off,
                         int64_t* failures);

/* Part 3 */
int64_t orc_reference_sampler(const orc_cfg* c, const orc_species* sp, int32_t n_sp,
                              const float* lrf28, const int32_t* keep, int64_t n_cells,
                              int32_t n_threads, uint64_t seed, orc_hadron* out,
                              int64_t capacity, double* seconds);

#endif
