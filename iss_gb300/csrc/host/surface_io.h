// MUSIC freeze-out surface reader: music_input settings, binary and text
// surfaces for hydro_mode 1 (boost-invariant) and 2 (3+1D), the reference's
// unit conversions and T > 0.01 GeV filter, and the HRG temperature
// regulation.  Output rows are FO_surf records (34 floats, GeV and fm) in the
// field order of src/data_struct.h:53-63.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "params.h"
#include "tables.h"

namespace iss {

constexpr int kFoSurfFloats = 34;

struct MusicSettings {
    int turn_on_bulk = 0, turn_on_rhob = 0, turn_on_diff = 0;
    bool binary = true;
    int iEOS = 0;
};

// The read_FOdata constructor's music_input parsing (src/readindata.cpp:25-94):
// starts from the parameter-file values of turn_on_bulk/rhob/diff and lets
// <work_path>/music_input override them.
bool read_music_input(const std::string& work_path, const ParamStore& params, MusicSettings* s,
                      std::string* err);

// Afterburner selected by afterburner_type and forced by EOS 9 / 91
// (src/readindata.cpp:96-109): 0 PDG decays, 1 UrQMD, 2 SMASH.
int select_afterburner(const ParamStore& params, int iEOS);

// read_FOsurfdat_MUSIC (src/readindata.cpp:626-765) for hydro_mode 2 and
// read_FOsurfdat_MUSIC_boost_invariant (src/readindata.cpp:395-546) for
// hydro_mode 1.
bool read_music_surface(const std::string& filename, int hydro_mode, const MusicSettings& s,
                        std::vector<float>* fo34, std::string* err);

// Temperature / chemical-potential regulation with the pure HRG EoS for
// EOS_to_use in {9, 91, 12, 14} (src/readindata.cpp:773-801).
void regulate_temperature(const HrgEos& eos, std::vector<float>* fo34);

// EOS_to_use values whose species tables the sampler supports: chemical
// equilibrium ones (src/readindata.cpp:222-264 with N_stable = 0).
bool eos_is_chemical_equilibrium(int iEOS);
bool eos_is_known(int iEOS);

}  // namespace iss
