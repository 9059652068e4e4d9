#include "writers.h"

#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <fstream>

namespace iss {

namespace {

// %24.16e of a float promoted to double, as sprintf does in the reference
int fmt_line_oscar(char* buf, size_t cap, int64_t ipart, const iss_hadron_t& p) {
    return std::snprintf(buf, cap,
                         "%10lld  %10d  %24.16e  %24.16e  %24.16e  %24.16e  %24.16e  %24.16e  "
                         "%24.16e  %24.16e  %24.16e\n",
                         static_cast<long long>(ipart), p.pid, static_cast<double>(p.px),
                         static_cast<double>(p.py), static_cast<double>(p.pz),
                         static_cast<double>(p.E), static_cast<double>(p.mass),
                         static_cast<double>(p.x), static_cast<double>(p.y),
                         static_cast<double>(p.z), static_cast<double>(p.t));
}

// ---------------------------------------------------------------------------
// gzip: zlib through dlopen, or stored deflate blocks with our own CRC-32

struct ZlibApi {
    void* lib = nullptr;
    void* (*gzopen)(const char*, const char*) = nullptr;
    int (*gzwrite)(void*, const void*, unsigned) = nullptr;
    int (*gzclose)(void*) = nullptr;
};

bool load_zlib(ZlibApi* z) {
    const char* names[] = {"libz.so.1", "libz.so"};
    for (const char* n : names) {
        z->lib = dlopen(n, RTLD_NOW | RTLD_LOCAL);
        if (z->lib) break;
    }
    if (!z->lib) return false;
    z->gzopen = reinterpret_cast<void* (*)(const char*, const char*)>(dlsym(z->lib, "gzopen"));
    z->gzwrite = reinterpret_cast<int (*)(void*, const void*, unsigned)>(dlsym(z->lib, "gzwrite"));
    z->gzclose = reinterpret_cast<int (*)(void*)>(dlsym(z->lib, "gzclose"));
    return z->gzopen && z->gzwrite && z->gzclose;
}

struct Crc32Table {
    uint32_t v[256];
    Crc32Table() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            v[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
    // built once; the initialisation of a function-local static is thread-safe,
    // so handles on several threads may write gzip output at the same time
    static const Crc32Table tab;
    const uint32_t* table = tab.v;
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

class GzipSink {
 public:
    bool open(const std::string& fn) {
        if (load_zlib(&z_)) {
            gz_ = z_.gzopen(fn.c_str(), "wb");
            if (gz_) return true;
        }
        f_ = std::fopen(fn.c_str(), "wb");
        if (!f_) return false;
        const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 255};
        std::fwrite(hdr, 1, 10, f_);
        return true;
    }
    void write(const char* p, size_t n) {
        if (gz_) {
            z_.gzwrite(gz_, p, static_cast<unsigned>(n));
            return;
        }
        buf_.insert(buf_.end(), p, p + n);
        if (buf_.size() >= 60000) flush_block(false);
    }
    void close() {
        if (gz_) {
            z_.gzclose(gz_);
            gz_ = nullptr;
            return;
        }
        if (!f_) return;
        flush_block(true);
        unsigned char trailer[8];
        for (int i = 0; i < 4; i++) trailer[i] = static_cast<unsigned char>(crc_ >> (8 * i));
        for (int i = 0; i < 4; i++) trailer[4 + i] = static_cast<unsigned char>(size_ >> (8 * i));
        std::fwrite(trailer, 1, 8, f_);
        std::fclose(f_);
        f_ = nullptr;
    }

 private:
    void flush_block(bool final) {
        size_t off = 0;
        do {
            const size_t len = std::min<size_t>(65535, buf_.size() - off);
            const bool last = final && (off + len == buf_.size());
            const unsigned char h[5] = {static_cast<unsigned char>(last ? 1 : 0),
                                        static_cast<unsigned char>(len & 0xFF),
                                        static_cast<unsigned char>(len >> 8),
                                        static_cast<unsigned char>(~len & 0xFF),
                                        static_cast<unsigned char>((~len >> 8) & 0xFF)};
            std::fwrite(h, 1, 5, f_);
            const unsigned char* p = reinterpret_cast<const unsigned char*>(buf_.data()) + off;
            std::fwrite(p, 1, len, f_);
            crc_ = crc32_update(crc_, p, len);
            size_ += static_cast<uint32_t>(len);
            off += len;
        } while (off < buf_.size());
        buf_.clear();
    }
    ZlibApi z_;
    void* gz_ = nullptr;
    std::FILE* f_ = nullptr;
    std::vector<char> buf_;
    uint32_t crc_ = 0;
    uint32_t size_ = 0;
};

}  // namespace

bool write_oscar(const std::string& filename, const std::string& header_file,
                 const iss_hadron_t* h, const int64_t* off, int n_events, std::string* err) {
    std::ifstream header(header_file);
    if (!header) {
        *err = "OSCAR header file " + header_file + " not found";
        return false;
    }
    std::remove(filename.c_str());
    std::FILE* f = std::fopen(filename.c_str(), "w");
    if (!f) {
        *err = "can not open " + filename;
        return false;
    }
    std::string line;
    while (std::getline(header, line)) std::fprintf(f, "%s\n", line.c_str());
    std::vector<char> buf(1 << 20);
    char lb[512];
    for (int e = 0; e < n_events; e++) {
        const int64_t n = off[e + 1] - off[e];
        if (n <= 0) continue;
        // event header: setw(10) iev, setw(10) n, setw(8) 0.0 (printed "0")
        std::fprintf(f, "%10d  %10lld  %8s  %8s\n", e, static_cast<long long>(n), "0", "0");
        size_t used = 0;
        for (int64_t i = 0; i < n; i++) {
            const int len = fmt_line_oscar(lb, sizeof(lb), i + 1, h[off[e] + i]);
            if (used + static_cast<size_t>(len) > buf.size()) {
                std::fwrite(buf.data(), 1, used, f);
                used = 0;
            }
            std::memcpy(buf.data() + used, lb, static_cast<size_t>(len));
            used += static_cast<size_t>(len);
        }
        std::fwrite(buf.data(), 1, used, f);
    }
    std::fclose(f);
    return true;
}

bool write_gzip(const std::string& filename, const iss_hadron_t* h, const int64_t* off,
                int n_events, std::string* err) {
    std::remove(filename.c_str());
    GzipSink sink;
    if (!sink.open(filename)) {
        *err = "can not open " + filename;
        return false;
    }
    char lb[512];
    for (int e = 0; e < n_events; e++) {
        const int64_t n = off[e + 1] - off[e];
        int len = std::snprintf(lb, sizeof(lb), "%lld \n", static_cast<long long>(n));
        sink.write(lb, static_cast<size_t>(len));
        for (int64_t i = 0; i < n; i++) {
            const iss_hadron_t& p = h[off[e] + i];
            len = std::snprintf(lb, sizeof(lb), "%d %.7e %.7e %.7e %.7e %.7e %.7e %.7e %.7e %.7e\n",
                                p.pid, static_cast<double>(p.mass), static_cast<double>(p.t),
                                static_cast<double>(p.x), static_cast<double>(p.y),
                                static_cast<double>(p.z), static_cast<double>(p.E),
                                static_cast<double>(p.px), static_cast<double>(p.py),
                                static_cast<double>(p.pz));
            sink.write(lb, static_cast<size_t>(len));
        }
    }
    sink.close();
    return true;
}

bool write_binary(const std::string& filename, const iss_hadron_t* h, const int64_t* off,
                  int n_events, std::string* err) {
    std::remove(filename.c_str());
    std::FILE* f = std::fopen(filename.c_str(), "wb");
    if (!f) {
        *err = "can not open " + filename;
        return false;
    }
    std::vector<char> buf;
    for (int e = 0; e < n_events; e++) {
        const int n = static_cast<int>(off[e + 1] - off[e]);
        buf.resize(sizeof(int) + static_cast<size_t>(n) * 40);
        std::memcpy(buf.data(), &n, sizeof(int));
        char* q = buf.data() + sizeof(int);
        for (int i = 0; i < n; i++) {
            const iss_hadron_t& p = h[off[e] + i];
            const float a[9] = {p.mass, p.t, p.x, p.y, p.z, p.E, p.px, p.py, p.pz};
            std::memcpy(q, &p.pid, 4);
            std::memcpy(q + 4, a, 36);
            q += 40;
        }
        std::fwrite(buf.data(), 1, buf.size(), f);
    }
    std::fclose(f);
    return true;
}

}  // namespace iss
