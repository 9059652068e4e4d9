// Test infrastructure: a caller written against the reference's driver class
// `iSS` (src/iSS.h:16-102) the way the reference's own main program uses it
// (src/main.cpp:22-74), extended to every other public member of the class.
// It compiles against the library's compatibility header shim/iSS.h without
// change, which is the drop-in claim tests/test_shim.py checks; run, it prints
// one line per check and returns the first failing status.
//
//   caller <parameter_file> <work_dir> <surface_file> [key=value ...]
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "shim/iSS.h"

int main(int argc, char** argv) {
    const std::string table_path = "iSS_tables";
    const std::string particle_table_path = "iSS_tables";
    std::string path = "results";
    std::string input_file = "iSS_parameters.dat";
    std::string surface_filename = "surface.dat";
    if (argc > 1 && std::string(argv[1]).find('=') == std::string::npos) input_file = argv[1];
    if (argc > 2 && std::string(argv[2]).find('=') == std::string::npos) path = argv[2];
    if (argc > 3 && std::string(argv[3]).find('=') == std::string::npos) surface_filename = argv[3];

    iSS iSsampler(path, table_path, particle_table_path, input_file, surface_filename);
    iSsampler.paraRdr_ptr->readFromArguments(argc, argv);
    iSsampler.paraRdr_ptr->echo();
    std::printf("MC_sampling %g\n", iSsampler.paraRdr_ptr->getVal("MC_sampling"));

    int status = iSsampler.shell();
    std::printf("shell %d\n", status);
    if (status != 0) return status;

    const int testFlag = static_cast<int>(iSsampler.paraRdr_ptr->getVal("perform_checks", 0));
    if (testFlag == 1) iSsampler.perform_checks();

    // the hadron-list accessors agree with one another
    const int nev = iSsampler.get_number_of_sampled_events();
    long total = 0;
    for (int iev = 0; iev < nev; iev++) {
        const int n = iSsampler.get_number_of_particles(iev);
        std::vector<iSS_Hadron>* list = iSsampler.get_hadron_list_iev(iev);
        if (static_cast<int>(list->size()) != n) return 100;
        for (int i = 0; i < n; i++) {
            const iSS_Hadron a = iSsampler.get_hadron(iev, i);
            const iSS_Hadron& b = (*list)[i];
            if (a.pid != b.pid || a.E != b.E || a.px != b.px || a.z != b.z) return 101;
            const double m2 = static_cast<double>(a.E) * a.E - static_cast<double>(a.px) * a.px -
                              static_cast<double>(a.py) * a.py - static_cast<double>(a.pz) * a.pz;
            if (std::fabs(m2 - static_cast<double>(a.mass) * a.mass) > 1e-3 * (1.0 + a.E * a.E))
                return 102;
        }
        total += n;
    }
    std::printf("events %d hadrons %ld\n", nev, total);

    // a second generate with an explicit seed, then clear
    iSsampler.set_random_seed(4321);
    status = iSsampler.generate_samples();
    std::printf("generate %d events %d\n", status, iSsampler.get_number_of_sampled_events());
    if (status != 0) return status;
    iSsampler.clear();
    std::printf("Program executed normally.\n");
    return 0;
}
