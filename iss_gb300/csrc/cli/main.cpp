// iSS.e: command-line driver with the reference's argument conventions
// (src/main.cpp:22-74): iSS.e [parameter_file] [work_dir] [surface_file]
// [key=value ...]; tables are read from ./iSS_tables.  Output files follow
// use_OSCAR_format / use_gzip_format / use_binary_format (src/FSSW.cpp:354-360).
#include <cstdio>
#include <string>

#include "shim/iSS.h"

int main(int argc, char** argv) {
    std::string input_file = "iSS_parameters.dat";
    std::string path = "results";
    std::string surface = "surface.dat";
    if (argc > 1 && std::string(argv[1]).find('=') == std::string::npos) input_file = argv[1];
    if (argc > 2 && std::string(argv[2]).find('=') == std::string::npos) path = argv[2];
    if (argc > 3 && std::string(argv[3]).find('=') == std::string::npos) surface = argv[3];
    std::printf("input file : %s\nwork folder path : %s\nsurface filename : %s\n",
                input_file.c_str(), path.c_str(), surface.c_str());
    iSS sampler(path, "iSS_tables", "iSS_tables", input_file, surface);
    sampler.paraRdr_ptr->readFromArguments(argc, argv);
    const int status = sampler.shell();
    if (status != 0) {
        std::fprintf(stderr, "[Error] %s: %s\n", iss_gpu_status_string(status),
                     iss_gpu_last_error(sampler.handle()));
        return status;
    }
    iss_handle* h = sampler.handle();
    int fmt = 0;
    if (sampler.paraRdr_ptr->getVal("use_OSCAR_format", 0) == 1) fmt = ISS_OUTPUT_OSCAR;
    else if (sampler.paraRdr_ptr->getVal("use_gzip_format", 0) == 1) fmt = ISS_OUTPUT_GZIP;
    else if (sampler.paraRdr_ptr->getVal("use_binary_format", 0) == 1) fmt = ISS_OUTPUT_BINARY;
    if (fmt != 0) {
        const int st = iss_gpu_write_output(h, fmt, nullptr);
        if (st != 0) {
            std::fprintf(stderr, "[Error] %s\n", iss_gpu_last_error(h));
            return st;
        }
    }
    iss_timings_t t;
    iss_gpu_get_timings(h, &t);
    std::printf("sampled %lld hadrons in %d events; device time %.3f ms\n",
                static_cast<long long>(t.n_hadrons), sampler.get_number_of_sampled_events(),
                t.ms_total);
    if (static_cast<int>(sampler.paraRdr_ptr->getVal("perform_checks", 0)) == 1)
        sampler.perform_checks();
    std::printf("Program executed normally.\n");
    return 0;
}
