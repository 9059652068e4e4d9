// OSCAR text of the hadron records on the GPU (FSSW::combine_samples_to_OSCAR,
// src/FSSW.cpp:365-494): every record becomes one fixed-width line
//   setw(10) ipart+1, "  ", setw(10) pid, then nine "%24.16e" fields
//   (px py pz E mass x y z t) separated by two spaces, and "\n",
// and every event with hadrons gets the sub-header
//   setw(10) iev, "  ", setw(10) n, "  ", setw(8) 0.0, "  ", setw(8) 0.0, "\n".
// The fields are formatted exactly (format_e.h), so the bytes equal those of
// the C library's printf.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "format_e.h"
#include "kernels.h"

namespace iss {

namespace {

constexpr int kOscarThreads = 128;

__device__ __forceinline__ void put(char* dst, const char* src, int n) {
    for (int i = 0; i < n; i++) dst[i] = src[i];
}

__global__ void __launch_bounds__(kOscarThreads)
oscar_lines_kernel(const HadronRec* __restrict__ had, int64_t h0, int64_t h1,
                   const int64_t* __restrict__ ev_off, const int64_t* __restrict__ ev_byte,
                   int e_lo, int e_hi, int64_t byte0, char* __restrict__ out) {
    for (int64_t h = h0 + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; h < h1;
         h += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        // event of hadron h: the last e in [e_lo, e_hi) with ev_off[e] <= h
        int lo = e_lo, hi = e_hi - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ev_off[mid] <= h) lo = mid; else hi = mid - 1;
        }
        const int64_t ipart = h - ev_off[lo];
        char* base = out + (ev_byte[lo] - byte0);
        if (ipart == 0) {
            char sh[kOscarSubHeader];
            fmt::format_int(lo, 10, sh);
            sh[10] = ' ';
            sh[11] = ' ';
            fmt::format_int(ev_off[lo + 1] - ev_off[lo], 10, sh + 12);
            const char tail[] = "         0         0\n";   // "  " + setw(8) "0", twice
            for (int i = 0; i < 21; i++) sh[22 + i] = tail[i];
            put(base, sh, kOscarSubHeader);
        }
        char* line = base + kOscarSubHeader + ipart * kOscarLine;
        const HadronRec r = had[h];
        char buf[kOscarLine];
        fmt::format_int(ipart + 1, 10, buf);
        buf[10] = ' ';
        buf[11] = ' ';
        fmt::format_int(r.pid, 10, buf + 12);
        const float v[9] = {r.px, r.py, r.pz, r.E, r.mass, r.x, r.y, r.z, r.t};
        int pos = 22;
#pragma unroll 1
        for (int k = 0; k < 9; k++) {
            buf[pos++] = ' ';
            buf[pos++] = ' ';
            fmt::format_e24_16(v[k], buf + pos);
            pos += 24;
        }
        buf[pos] = '\n';
        put(line, buf, kOscarLine);
    }
}

}  // namespace

cudaError_t launch_oscar_lines(const HadronRec* had, int64_t h0, int64_t h1, const int64_t* ev_off,
                               const int64_t* ev_byte, int e_lo, int e_hi, int64_t byte0,
                               char* out, int num_sms, cudaStream_t stream) {
    if (h1 <= h0) return cudaSuccess;
    int64_t blocks = (h1 - h0 + kOscarThreads - 1) / kOscarThreads;
    const int64_t cap = static_cast<int64_t>(num_sms) * 16;
    if (blocks > cap) blocks = cap;
    oscar_lines_kernel<<<static_cast<unsigned>(blocks), kOscarThreads, 0, stream>>>(
        had, h0, h1, ev_off, ev_byte, e_lo, e_hi, byte0, out);
    return cudaGetLastError();
}

}  // namespace iss
