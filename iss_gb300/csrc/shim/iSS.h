// C++ compatibility class with the public surface of the reference's driver
// class `iSS` (src/iSS.h:16-102) and its ParameterReader
// (src/ParameterReader.h), implemented on the C ABI of include/iss_gpu.h.
// Code written against the reference's libiSS recompiles against this header
// unchanged; sampling runs on the GPU.  Errors that make the reference call
// exit() are reported through the int return codes (an iss_status) or, for
// getVal of an unknown key, a std::out_of_range exception.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "iss_gpu.h"

struct iSS_Hadron {
    int pid;
    float mass;
    float E, px, py, pz;
    float t, x, y, z;
};

class ParameterReader {
 public:
    explicit ParameterReader(iss_handle* h) : h_(h) {}
    void readFromFile(std::string filename, std::string commentSymbol = "#");
    void readFromArguments(long argc, char* argv[], std::string commentSymbol = "#",
                           long start_from = 1);
    void phraseOneLine(std::string str, std::string commentSymbol = "#");
    bool exist(std::string name);
    void setVal(std::string name, double value);
    double getVal(std::string name);
    double getVal(std::string name, double defaultValue);
    void echo();

 private:
    iss_handle* h_;
};

class iSS {
 public:
    iSS(std::string path, std::string table_path = "iSS_tables",
        std::string particle_table_path = "iSS_tables",
        std::string inputfile = "iSS_parameters.dat", std::string surface_filename = "surface.dat");
    ~iSS();

    ParameterReader* paraRdr_ptr;

    void set_random_seed();
    void set_random_seed(int randomSeed_in);

    void perform_checks();
    void construct_Tmunu_from_particle_samples();

    int shell();
    int read_in_FO_surface();
    int generate_samples();

    int get_number_of_sampled_events();
    int get_number_of_particles(int iev);
    iSS_Hadron get_hadron(int iev, int ipart);
    std::vector<iSS_Hadron>* get_hadron_list_iev(const int iev);

    void clear();

    // the underlying C handle (for the C ABI's inspection calls)
    iss_handle* handle() { return h_; }
    int status() const { return status_; }

 private:
    iss_handle* h_ = nullptr;
    int status_ = 0;
    std::vector<std::unique_ptr<std::vector<iSS_Hadron>>> events_;
};
