#include "surface_io.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace iss {

namespace {
constexpr double kHbarC = 0.197327053;
}

bool read_music_input(const std::string& work_path, const ParamStore& params, MusicSettings* s,
                      std::string* err) {
    s->turn_on_bulk = static_cast<int>(params.get_or("turn_on_bulk", 0));
    s->turn_on_rhob = static_cast<int>(params.get_or("turn_on_rhob", 0));
    s->turn_on_diff = static_cast<int>(params.get_or("turn_on_diff", 0));
    s->binary = true;
    s->iEOS = 0;
    const std::string fn = work_path + "/music_input";
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find configuration file " + fn;
        return false;
    }
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key)) continue;
        int v = 0;
        if (key == "Include_Bulk_Visc_Yes_1_No_0") {
            if (ss >> v) s->turn_on_bulk = v;
        } else if (key == "Include_Rhob_Yes_1_No_0") {
            if (ss >> v) s->turn_on_rhob = v;
        } else if (key == "turn_on_baryon_diffusion") {
            if (ss >> v) s->turn_on_diff = v;
        } else if (key == "freeze_surface_in_binary") {
            if (ss >> v) s->binary = (v == 1);
        } else if (key == "EOS_to_use") {
            if (ss >> v) s->iEOS = v;
        }
    }
    return true;
}

int select_afterburner(const ParamStore& params, int iEOS) {
    const int id = static_cast<int>(params.get_or("afterburner_type", 0));
    int ab = (id == 1) ? 1 : (id == 2 ? 2 : 0);
    if (iEOS == 9) ab = 1;
    if (iEOS == 91) ab = 2;
    return ab;
}

bool eos_is_known(int iEOS) {
    return iEOS == 2 || (iEOS >= 3 && iEOS <= 9) || iEOS == 91 ||
           (iEOS >= 10 && iEOS <= 15) || iEOS == 17;
}

bool eos_is_chemical_equilibrium(int iEOS) {
    return eos_is_known(iEOS) && !(iEOS >= 3 && iEOS <= 6);
}

namespace {

// unit conversions of the reference reader: float members assigned from
// float*double products, P = (e+P)/T * T - e in float arithmetic
void fill_record(const float* a, int hydro_mode, float* r) {
    r[0] = a[0];
    r[1] = a[1];
    r[2] = a[2];
    r[3] = (hydro_mode == 2) ? a[3] : 0.0f;
    r[4] = a[4];
    r[5] = a[5];
    r[6] = a[6];
    r[7] = (hydro_mode == 2) ? a[7] : 0.0f;
    r[8] = a[8];
    r[9] = a[9];
    r[10] = a[10];
    r[11] = a[11];
    const float E = static_cast<float>(a[12] * kHbarC);
    const float T = static_cast<float>(a[13] * kHbarC);
    r[12] = E;
    r[13] = T;
    r[14] = a[17] * T - E;
    r[15] = a[29];
    r[16] = static_cast<float>(a[14] * kHbarC);
    r[17] = static_cast<float>(a[15] * kHbarC);
    r[18] = static_cast<float>(a[16] * kHbarC);
    for (int k = 0; k < 10; k++) r[19 + k] = static_cast<float>(a[18 + k] * kHbarC);
    r[29] = static_cast<float>(a[28] * kHbarC);
    r[30] = a[30];
    r[31] = a[31];
    r[32] = a[32];
    r[33] = a[33];
}

void push_if_warm(const float* r, std::vector<float>* out) {
    if (r[13] > 0.01) out->insert(out->end(), r, r + kFoSurfFloats);
}

}  // namespace

bool read_music_surface(const std::string& filename, int hydro_mode, const MusicSettings& s,
                        std::vector<float>* fo34, std::string* err) {
    fo34->clear();
    if (hydro_mode != 1 && hydro_mode != 2) {
        *err = "unsupported hydro_mode for MUSIC surfaces";
        return false;
    }
    if (s.binary) {
        std::FILE* f = std::fopen(filename.c_str(), "rb");
        if (!f) {
            *err = "surface file is not found: " + filename;
            return false;
        }
        std::fseek(f, 0, SEEK_END);
        const long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        const size_t n = static_cast<size_t>(bytes) / (sizeof(float) * kFoSurfFloats);
        std::vector<float> raw(n * kFoSurfFloats);
        const size_t got = raw.empty() ? 0 : std::fread(raw.data(), sizeof(float) * kFoSurfFloats, n, f);
        std::fclose(f);
        fo34->reserve(got * kFoSurfFloats);
        float r[kFoSurfFloats];
        for (size_t i = 0; i < got; i++) {
            fill_record(&raw[i * kFoSurfFloats], hydro_mode, r);
            push_if_warm(r, fo34);
        }
        return true;
    }
    std::ifstream f(filename);
    if (!f) {
        *err = "surface file is not found: " + filename;
        return false;
    }
    // Text columns: tau x y eta, da0..da3, u0..u3, e T muB muS muQ (e+P)/T,
    // ten shear components, then the optional bulk, n_B and q^mu columns.
    // The reference extracts some columns as float and others as double
    // before scaling by hbar c; the same conversions are used here.
    const int ncols = 28 + (s.turn_on_bulk == 1) + (s.turn_on_rhob == 1) +
                      4 * (s.turn_on_diff == 1);
    std::vector<std::string> tok(static_cast<size_t>(ncols));
    auto fl = [](const std::string& t) { return std::strtof(t.c_str(), nullptr); };
    auto db = [](const std::string& t) { return std::strtod(t.c_str(), nullptr); };
    auto convert = [&](float* r) {
        for (int k = 0; k < kFoSurfFloats; k++) r[k] = 0.0f;
        if (hydro_mode == 2) {
            for (int k = 0; k < 4; k++) r[k] = fl(tok[k]);
        } else {
            for (int k = 0; k < 3; k++) r[k] = static_cast<float>(db(tok[k]));
        }
        for (int k = 4; k < 12; k++) r[k] = fl(tok[k]);
        if (hydro_mode != 2) {
            r[3] = 0.0f;
            r[7] = 0.0f;
        }
        r[12] = static_cast<float>(db(tok[12]) * kHbarC);
        r[13] = static_cast<float>(db(tok[13]) * kHbarC);
        r[16] = static_cast<float>(db(tok[14]) * kHbarC);
        r[17] = static_cast<float>(db(tok[15]) * kHbarC);
        r[18] = static_cast<float>(db(tok[16]) * kHbarC);
        r[14] = static_cast<float>(db(tok[17]) * r[13] - r[12]);
        for (int k = 0; k < 10; k++) r[19 + k] = static_cast<float>(db(tok[18 + k]) * kHbarC);
        int c = 28;
        if (s.turn_on_bulk == 1) r[29] = static_cast<float>(db(tok[c++]) * kHbarC);
        if (s.turn_on_rhob == 1) r[15] = static_cast<float>(db(tok[c++]));
        if (s.turn_on_diff == 1) {
            for (int k = 0; k < 4; k++) r[30 + k] = fl(tok[c++]);
        }
    };
    float r[kFoSurfFloats];
    if (hydro_mode == 2) {
        // whitespace-separated stream; like the reference, a record whose
        // reading reaches the end of the file is not kept
        for (;;) {
            int got = 0;
            for (; got < ncols; got++) {
                if (!(f >> tok[static_cast<size_t>(got)])) break;
            }
            if (got < ncols) break;
            if (f.peek() == std::char_traits<char>::eof()) break;
            convert(r);
            push_if_warm(r, fo34);
        }
    } else {
        std::string line;
        while (std::getline(f, line)) {
            if (f.eof()) break;
            std::istringstream ss(line);
            int got = 0;
            while (got < ncols && (ss >> tok[static_cast<size_t>(got)])) got++;
            for (int k = got; k < ncols; k++) tok[static_cast<size_t>(k)] = "0";
            convert(r);
            push_if_warm(r, fo34);
        }
    }
    return true;
}

void regulate_temperature(const HrgEos& eos, std::vector<float>* fo34) {
    const size_t n = fo34->size() / kFoSurfFloats;
    for (size_t i = 0; i < n; i++) {
        float* r = fo34->data() + i * kFoSurfFloats;
        double v[5];
        if (hrg_eos_values(eos, r[12], r[15], v)) {
            r[13] = static_cast<float>(v[1]);
            r[16] = static_cast<float>(v[2]);
            r[17] = static_cast<float>(v[3]);
            r[18] = static_cast<float>(v[4]);
            r[14] = static_cast<float>(v[0]);
        }
    }
}

}  // namespace iss
