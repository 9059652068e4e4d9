#include "shim/iSS.h"

#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>

static_assert(sizeof(iSS_Hadron) == sizeof(iss_hadron_t), "iSS_Hadron layout");

// ---------------------------------------------------------------------------
// ParameterReader

void ParameterReader::readFromFile(std::string filename, std::string) {
    std::ifstream f(filename);
    if (!f) throw std::runtime_error("ParameterReader::readFromFile: file " + filename +
                                     " does not exist");
    std::string line;
    while (std::getline(f, line)) iss_gpu_parse_param_line(h_, line.c_str());
}

void ParameterReader::readFromArguments(long argc, char* argv[], std::string, long start_from) {
    for (long i = start_from; i < argc; i++) iss_gpu_parse_param_line(h_, argv[i]);
}

void ParameterReader::phraseOneLine(std::string str, std::string) {
    iss_gpu_parse_param_line(h_, str.c_str());
}

bool ParameterReader::exist(std::string name) {
    double v;
    return iss_gpu_get_param(h_, name.c_str(), &v) == ISS_OK;
}

void ParameterReader::setVal(std::string name, double value) {
    iss_gpu_set_param(h_, name.c_str(), value);
}

double ParameterReader::getVal(std::string name) {
    double v;
    if (iss_gpu_get_param(h_, name.c_str(), &v) != ISS_OK)
        throw std::out_of_range("ParameterReader::getVal: parameter with name " + name +
                                " not found");
    return v;
}

double ParameterReader::getVal(std::string name, double defaultValue) {
    double v;
    return iss_gpu_get_param(h_, name.c_str(), &v) == ISS_OK ? v : defaultValue;
}

void ParameterReader::echo() {}

// ---------------------------------------------------------------------------
// iSS

iSS::iSS(std::string path, std::string table_path, std::string particle_table_path,
         std::string inputfile, std::string surface_filename) {
    status_ = iss_gpu_create(path.c_str(), table_path.c_str(), particle_table_path.c_str(),
                             inputfile.c_str(), surface_filename.c_str(), &h_);
    if (status_ != ISS_OK) {
        // an unreadable parameter file still yields a usable (empty) handle
        iss_gpu_create(path.c_str(), table_path.c_str(), particle_table_path.c_str(), "",
                       surface_filename.c_str(), &h_);
    }
    paraRdr_ptr = new ParameterReader(h_);
}

iSS::~iSS() {
    delete paraRdr_ptr;
    iss_gpu_destroy(h_);
}

void iSS::set_random_seed() { iss_gpu_set_seed_from_params(h_); }
void iSS::set_random_seed(int randomSeed_in) { iss_gpu_set_seed(h_, randomSeed_in); }

int iSS::read_in_FO_surface() { return iss_gpu_read_surface(h_); }

int iSS::generate_samples() {
    events_.clear();
    return iss_gpu_generate(h_);
}

int iSS::shell() {
    int st = read_in_FO_surface();
    if (st != ISS_OK) return st;
    set_random_seed();
    return generate_samples();
}

int iSS::get_number_of_sampled_events() {
    int32_t n = 0;
    return iss_gpu_num_events(h_, &n) == ISS_OK ? n : 0;
}

int iSS::get_number_of_particles(int iev) {
    int64_t n = 0;
    return iss_gpu_num_particles(h_, iev, &n) == ISS_OK ? static_cast<int>(n) : 0;
}

iSS_Hadron iSS::get_hadron(int iev, int ipart) {
    iSS_Hadron out{};
    iss_gpu_get_hadron(h_, iev, ipart, reinterpret_cast<iss_hadron_t*>(&out));
    return out;
}

std::vector<iSS_Hadron>* iSS::get_hadron_list_iev(const int iev) {
    const int nev = get_number_of_sampled_events();
    if (iev < 0 || iev >= nev) throw std::out_of_range("get_hadron_list_iev: event out of range");
    if (events_.size() != static_cast<size_t>(nev)) events_.resize(static_cast<size_t>(nev));
    auto& slot = events_[static_cast<size_t>(iev)];
    if (!slot) {
        int64_t n = 0;
        iss_gpu_copy_event(h_, iev, nullptr, 0, &n);
        slot.reset(new std::vector<iSS_Hadron>(static_cast<size_t>(n)));
        if (n > 0)
            iss_gpu_copy_event(h_, iev, reinterpret_cast<iss_hadron_t*>(slot->data()), n, &n);
    }
    return slot.get();
}

void iSS::clear() {
    events_.clear();
    iss_gpu_clear(h_);
}

// T^{mu nu} rebuilt from the samples against the first cell's fluid T^{mu nu}
// (iSS::construct_Tmunu_from_particle_samples, src/iSS.cpp:296-363; valid
// for one-cell surfaces like the reference's own check).
void iSS::construct_Tmunu_from_particle_samples() {
    int64_t ncell = 0;
    iss_gpu_num_cells(h_, &ncell);
    if (ncell <= 0) return;
    std::vector<float> lrf(static_cast<size_t>(ncell) * 28);
    if (iss_gpu_copy_lrf_cells(h_, lrf.data(), ncell) != ISS_OK) return;
    const float* c = lrf.data();
    const double volume = c[4] / c[8];
    // fluid T^{mu nu} in the t-z frame: boost the LRF tensor
    const double u[4] = {c[8], c[9], c[10], c[11]};
    const double e = c[12], P = c[14], Pi = c[19];
    double TL[4][4] = {{e, 0, 0, 0}, {0, P + Pi, 0, 0}, {0, 0, P + Pi, 0}, {0, 0, 0, P + Pi}};
    TL[1][1] += c[20];
    TL[1][2] = TL[2][1] = c[21];
    TL[1][3] = TL[3][1] = c[22];
    TL[2][2] += c[23];
    TL[2][3] = TL[3][2] = c[24];
    TL[3][3] += -c[20] - c[23];
    double L[4][4];
    L[0][0] = u[0];
    for (int i = 1; i < 4; i++) {
        L[0][i] = L[i][0] = u[i];
        for (int j = 1; j < 4; j++) L[i][j] = (i == j) + u[i] * u[j] / (1.0 + u[0]);
    }
    double Tf[4][4] = {};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) Tf[i][j] += L[i][a] * TL[a][b] * L[j][b];
    double T[4][4] = {};
    const int nev = get_number_of_sampled_events();
    for (int iev = 0; iev < nev; iev++) {
        std::vector<iSS_Hadron>* ev = get_hadron_list_iev(iev);
        for (const iSS_Hadron& hd : *ev) {
            const double p[4] = {hd.E, hd.px, hd.py, hd.pz};
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) T[i][j] += p[i] * p[j] / p[0];
        }
    }
    std::ofstream out("checkReconstructedTmunu.dat");
    out << "# Tmunu_FOcell[GeV/fm^3]  Tmunu_Particles[GeV/fm^3]  diff" << std::endl;
    for (int i = 0; i < 4; i++) {
        for (int j = 0; j < 4; j++) {
            const double tp = (nev > 0 && volume > 0) ? T[i][j] / (nev * volume) : 0.0;
            out << std::scientific << std::setprecision(8) << Tf[i][j] << "  " << tp << "  "
                << Tf[i][j] - tp << std::endl;
        }
    }
}

// iSS::perform_checks (src/iSS.cpp:59-83): T^{mu nu} check and pT spectra
// of pi+ and protons (100 bins in [0, 5] GeV, per event).
void iSS::perform_checks() {
    construct_Tmunu_from_particle_samples();
    const int nev = get_number_of_sampled_events();
    std::vector<double> hp(100, 0.0), hn(100, 0.0);
    for (int iev = 0; iev < nev; iev++) {
        for (const iSS_Hadron& hd : *get_hadron_list_iev(iev)) {
            const double pT = std::sqrt(static_cast<double>(hd.px) * hd.px +
                                        static_cast<double>(hd.py) * hd.py);
            const int b = static_cast<int>(pT / 0.05);
            if (b < 0 || b >= 100) continue;
            if (hd.pid == 211) hp[b] += 1.0;
            if (hd.pid == 2212) hn[b] += 1.0;
        }
    }
    const char* names[2] = {"check_211_spectra.dat", "check_2212_spectra.dat"};
    const std::vector<double>* hs[2] = {&hp, &hn};
    for (int k = 0; k < 2; k++) {
        std::ofstream out(names[k]);
        for (int b = 0; b < 100; b++) {
            const double x = (b + 0.5) * 0.05;
            out << std::scientific << std::setprecision(8) << x << "  "
                << (*hs[k])[b] / std::max(nev, 1) / 0.05 << std::endl;
        }
    }
}
