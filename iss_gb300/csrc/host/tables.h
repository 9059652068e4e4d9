// Species lists, delta-f coefficient tables, special-function tables and the
// hadron-resonance-gas tables used to regulate cell temperatures, read in the
// reference's file formats with the reference's parsing rules.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "device_common.cuh"

namespace iss {

struct Species {
    int32_t pid;
    int32_t real_idx;   // index in the full resonance list
    double mass;
    int32_t gspin, baryon, strange, charge, sign;
};

// read_resonances_list (src/readindata.cpp:971-1116, anti-baryons appended
// after each baryon, statistics sign at :1103-1113), the chosen table
// selected by the afterburner (src/iSS.cpp:133-142) and FSSW's stable bubble
// sort by mass (src/FSSW.cpp:115-162).  Returns false with `err` set if a
// file is missing.
bool load_chosen_species(const std::string& particle_table_path, int afterburner,
                         bool quantum_statistics, std::vector<Species>* out,
                         std::vector<int32_t>* unidentified, std::string* err);

// Resonance decay table of particle_decay::read_resonances_list
// (src/particle_decay.cpp:33-170): every entry of the pdg file, each baryon
// followed by its anti-baryon, whose channels negate every daughter that is
// not a neutral, non-strange meson (looked up among the entries read so far).
// stable = the first channel has one daughter.  Daughters are indices into
// `particles` (-1 when the pid is not in the table).
struct DecayTable {
    std::vector<DecayParticle> particles;
    std::vector<DecayChannel> channels;
};
bool load_decay_table(const std::string& particle_table_path, int afterburner, DecayTable* out,
                      std::string* err);

// Full resonance list (for quantum-number lookups).
bool load_resonances(const std::string& particle_table_path, int afterburner,
                     bool quantum_statistics, std::vector<Species>* out, std::string* err);

// Special functions on the reference's grid x = 0.5 + 0.05 i, i < 7991
// (src/FSSW.cpp:1609-1643), computed in FP64 from their integral
// representations.
constexpr int kSfLen = 7991;
constexpr double kSfX0 = 0.5;
constexpr double kSfDx = 0.05;
constexpr int kNumExpint = 9;   // E_2, E_4, ..., E_18
double bessel_k(int n, double x);
double expint_en(int n, double x);
void special_function_tables(bool with_bulk, bool with_diffusion, std::vector<double>* K,
                             std::vector<double>* E);

// OSU 14-moment bulk tables (src/FSSW.cpp:1215-1300), [iT * nmu + imu].
struct Bulk14Table {
    int nT = 0, nmu = 0;
    double T0 = 0, mu0 = 0, dT = 0, dmu = 0;
    std::vector<double> c0, c1, c2;
};
// fix_c0 == false reproduces the reference: it reads c0.dat's two size lines
// but not the column-title line after them, so every c0 read fails and the
// c0 coefficients stay zero.
bool load_bulk14(const std::string& table_path, int afterburner, bool fix_c0,
                 Bulk14Table* out, std::string* err);

// NEoS-BQS Chapman-Enskog coefficients (src/FSSW.cpp:1303-1338): 200 x 200
// rows of (e, n_B, c2_hat, zeta_hat, eta_hat).
bool load_ce_neos(const std::string& table_path, int afterburner, std::vector<double>* out,
                  std::string* err);

// RTA diffusion coefficient kappa_B (src/FSSW.cpp:1546-1568), [iT * 100 + imu].
bool load_qmu_coeff(const std::string& table_path, std::vector<double>* out, std::string* err);

// Pure hadron-resonance-gas EoS used to regulate T and mu for EOS_to_use in
// {9, 91, 12, 14} (read_in_HRG_EOS, src/readindata.cpp:913-968; rows of
// {e, nB, P, T, muB, muS, muQ}).
struct HrgEos {
    int iEOS = 0;
    std::vector<std::vector<double>> rows;
};
bool load_hrg_eos(const std::string& table_path, int iEOS, int afterburner, HrgEos* out,
                  std::string* err);
// getValuesFromHRGEOS (src/readindata.cpp:1249-1309): {P, T, muB, muS, muQ};
// returns false when e is outside the table (the cell is left unchanged).
bool hrg_eos_values(const HrgEos& eos, double ed, double nB, double* vars5);

}  // namespace iss
