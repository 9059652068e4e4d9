// Test infrastructure only: a small driver that links the UNMODIFIED reference
// sources (compiled by oracle/Makefile `ref`) and dumps, at full FP64
// precision, what the reference computes on the sampling path, so that the C
// restatement in oracle/ and the CUDA path can be pinned against it.
//
//   ref_driver yields <param_file> <work_dir> <surface_file> <table_path> <out.bin> [key=val ...]
//     Runs iSS::read_in_FO_surface (src/iSS.cpp:86-113), builds the FSSW
//     sampler exactly as iSS::generate_samples does (src/iSS.cpp:130-150) and
//     calls FSSW::calculate_dN_dxtdy_for_one_particle_species
//     (src/FSSW.cpp:565-715) for every chosen species in the sampler's
//     mass-sorted order (src/FSSW.cpp:151-162).  Writes the species table, the
//     local-rest-frame cells and the per-cell yields dN/(dx_t dy).
//
//   ref_driver sample <param_file> <work_dir> <surface_file> <table_path> <out.bin> [key=val ...]
//     Runs iSS::shell() (src/iSS.cpp:41-56) and writes every sampled hadron
//     (iSS_Hadron records, src/data_struct.h:79-84) event by event.
//
//   ref_driver write <param_file> <work_dir> <surface_file> <table_path> <in.bin> [key=val ...]
//     Builds the FSSW sampler as in `yields`, replaces its in-memory hadron
//     list by the events of <in.bin> (the format `sample` writes) and calls
//     the reference's three writers on it: FSSW::combine_samples_to_OSCAR,
//     combine_samples_to_gzip_file and combine_samples_to_binary_file
//     (src/FSSW.cpp:365-561), which write OSCAR.DAT, particle_samples.gz and
//     particle_samples.bin into the current directory.
//
// The reference keeps the data it computes in private members; this driver
// reads them by compiling the reference headers with `private` mapped to
// `public` (the reference sources themselves are compiled unchanged).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>
#include <array>
#include <random>
#include <map>
#include <zlib.h>

#define private public
#define protected public
#include "iSS.h"
#include "FSSW.h"
#include "Table.h"
#undef private
#undef protected

namespace {

void write_raw(std::FILE* f, const void* p, size_t n) {
    if (n && std::fwrite(p, 1, n, f) != n) {
        std::fprintf(stderr, "ref_driver: short write\n");
        std::exit(3);
    }
}

template <typename T> void put(std::FILE* f, T v) { write_raw(f, &v, sizeof(T)); }

int run_yields(iSS& iss, const std::string& work_dir, const std::string& table_path,
               const char* out_name) {
    iss.read_in_FO_surface();
    iss.set_random_seed();
    Table chosen;
    if (iss.afterburner_type_ == AfterburnerType::SMASH) {
        chosen.loadTableFromFile(table_path + "/chosen_particles_SMASH.dat");
    } else if (iss.afterburner_type_ == AfterburnerType::UrQMD) {
        chosen.loadTableFromFile(table_path + "/chosen_particles_urqmd_v3.3+.dat");
    } else {
        chosen.loadTableFromFile(table_path + "/chosen_particles_s95p-v1.dat");
    }
    FSSW sampler(iss.ran_gen_ptr_, &chosen, iss.particle_, iss.FOsurf_LRF_array_,
                 iss.flag_PCE_, iss.paraRdr_ptr, work_dir, table_path,
                 iss.afterburner_type_);
    const std::vector<FO_surf_LRF>& cells = iss.FOsurf_LRF_array_;
    const int n_species = sampler.number_of_chosen_particles;
    const int64_t n_cells = static_cast<int64_t>(cells.size());

    std::FILE* f = std::fopen(out_name, "wb");
    if (!f) { std::perror(out_name); return 2; }
    put<int32_t>(f, 0x59494c44);  // 'YILD'
    put<int32_t>(f, n_species);
    put<int64_t>(f, n_cells);
    for (int n = 0; n < n_species; n++) {
        const int idx = sampler.chosen_particles_sampling_table[n];
        const particle_info& p = sampler.particles[idx];
        put<int32_t>(f, p.monval);
        put<int32_t>(f, idx);
        put<double>(f, p.mass);
        put<int32_t>(f, p.gspin);
        put<int32_t>(f, p.baryon);
        put<int32_t>(f, p.strange);
        put<int32_t>(f, p.charge);
        put<int32_t>(f, p.sign);
    }
    for (const FO_surf_LRF& c : cells) {
        float rec[28] = {c.tau, c.xpt, c.ypt, c.eta,
                         c.da_mu_LRF[0], c.da_mu_LRF[1], c.da_mu_LRF[2], c.da_mu_LRF[3],
                         c.u_tz[0], c.u_tz[1], c.u_tz[2], c.u_tz[3],
                         c.Edec, c.Tdec, c.Pdec, c.Bn, c.muB, c.muS, c.muQ, c.bulkPi,
                         c.piLRF_xx, c.piLRF_xy, c.piLRF_xz, c.piLRF_yy, c.piLRF_yz,
                         c.qmuLRF_x, c.qmuLRF_y, c.qmuLRF_z};
        write_raw(f, rec, sizeof(rec));
    }
    for (int n = 0; n < n_species; n++) {
        const int idx = sampler.chosen_particles_sampling_table[n];
        sampler.calculate_dN_dxtdy_for_one_particle_species(idx);
        write_raw(f, sampler.dN_dxtdy_for_one_particle_species.data(),
                  sizeof(double) * static_cast<size_t>(n_cells));
    }
    std::fclose(f);
    return 0;
}

int run_write(iSS& iss, const std::string& work_dir, const std::string& table_path,
              const char* in_name) {
    iss.read_in_FO_surface();
    iss.set_random_seed();
    Table chosen;
    chosen.loadTableFromFile(table_path + "/chosen_particles_s95p-v1.dat");
    FSSW sampler(iss.ran_gen_ptr_, &chosen, iss.particle_, iss.FOsurf_LRF_array_,
                 iss.flag_PCE_, iss.paraRdr_ptr, work_dir, table_path,
                 iss.afterburner_type_);
    std::FILE* f = std::fopen(in_name, "rb");
    if (!f) { std::perror(in_name); return 2; }
    int32_t magic = 0, nev = 0;
    if (std::fread(&magic, 4, 1, f) != 1 || magic != 0x48414452 || std::fread(&nev, 4, 1, f) != 1) {
        std::fprintf(stderr, "ref_driver: %s is not a hadron list\n", in_name);
        return 2;
    }
    for (auto* ev : *sampler.Hadron_list) delete ev;
    sampler.Hadron_list->clear();
    for (int iev = 0; iev < nev; iev++) {
        int32_t n = 0;
        if (std::fread(&n, 4, 1, f) != 1) return 2;
        auto* ev = new std::vector<iSS_Hadron>(static_cast<size_t>(n));
        if (n > 0 && std::fread(ev->data(), sizeof(iSS_Hadron), static_cast<size_t>(n), f) !=
                         static_cast<size_t>(n))
            return 2;
        sampler.Hadron_list->push_back(ev);
    }
    std::fclose(f);
    sampler.flag_store_samples_in_memory = 1;
    sampler.combine_samples_to_OSCAR();
    sampler.combine_samples_to_gzip_file();
    sampler.combine_samples_to_binary_file();
    return 0;
}

int run_sample(iSS& iss, const char* out_name) {
    iss.shell();
    std::FILE* f = std::fopen(out_name, "wb");
    if (!f) { std::perror(out_name); return 2; }
    const int nev = iss.get_number_of_sampled_events();
    put<int32_t>(f, 0x48414452);  // 'HADR'
    put<int32_t>(f, nev);
    for (int iev = 0; iev < nev; iev++) {
        std::vector<iSS_Hadron>* ev = iss.get_hadron_list_iev(iev);
        put<int32_t>(f, static_cast<int32_t>(ev->size()));
        if (!ev->empty()) write_raw(f, ev->data(), sizeof(iSS_Hadron) * ev->size());
    }
    std::fclose(f);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr,
                     "usage: %s yields|sample|write <param_file> <work_dir> <surface_file> "
                     "<table_path> <out.bin | in.bin> [key=val ...]\n", argv[0]);
        return 1;
    }
    const std::string mode = argv[1];
    const std::string param_file = argv[2];
    const std::string work_dir = argv[3];
    const std::string surface_file = argv[4];
    const std::string table_path = argv[5];
    const char* out_name = argv[6];
    iSS iss(work_dir, table_path, table_path, param_file, surface_file);
    iss.paraRdr_ptr->readFromArguments(argc, argv, "#", 7);
    if (mode == "yields") return run_yields(iss, work_dir, table_path, out_name);
    if (mode == "sample") return run_sample(iss, out_name);
    if (mode == "write") return run_write(iss, work_dir, table_path, out_name);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 1;
}
