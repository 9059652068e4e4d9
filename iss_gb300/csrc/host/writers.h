// Output writers in the reference's formats (src/FSSW.cpp:365-561).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "iss_gpu.h"

namespace iss {

// FSSW::combine_samples_to_OSCAR, in-memory branch (src/FSSW.cpp:459-486):
// header copied from <table_path>/OSCAR_header.txt, events with at least one
// hadron, event index from 0, particle lines in %24.16e.
bool write_oscar(const std::string& filename, const std::string& header_file,
                 const iss_hadron_t* h, const int64_t* event_offsets, int n_events,
                 std::string* err);

// FSSW::combine_samples_to_gzip_file (src/FSSW.cpp:497-526): gzip stream of
// "count" lines and "pid mass t x y z E px py pz" lines (%.7e).  Uses zlib
// when the shared library is present, otherwise writes the same bytes as an
// uncompressed (stored-block) gzip member.
bool write_gzip(const std::string& filename, const iss_hadron_t* h,
                const int64_t* event_offsets, int n_events, std::string* err);

// FSSW::combine_samples_to_binary_file (src/FSSW.cpp:529-561): per event an
// int count, then per hadron int pid + float mass, t, x, y, z, E, px, py, pz.
bool write_binary(const std::string& filename, const iss_hadron_t* h,
                  const int64_t* event_offsets, int n_events, std::string* err);

}  // namespace iss
