// Cell prologue: regulate_surface_cells (src/readindata.cpp:802-841, with
// regulate_Wmunu :1216-1246), iSS::transform_to_local_rest_frame
// (src/iSS.cpp:170-293) and the per-cell delta-f coefficient lookups
// (src/FSSW.cpp:598-637, 1379-1430, 1433-1487, 1571-1606), one thread per cell.
//
// This translation unit is compiled with --fmad=false and keeps the
// reference's mix of float members and double temporaries operation by
// operation.  That matters: at large space-time rapidity the transform goes
// through the (t, z) frame, where terms of size cosh(eta)^2 u^t cancel down
// to O(1), so the result is only reproducible by rounding at the same points
// as the reference (float storage of u^t, dsigma^mu, pi^{mu nu}_{tz}; double
// boost matrix and products).  The double temporaries are float-float pairs
// (ffloat.cuh, about 48 bits): each rounds to the same float as the
// reference's double unless it lies within about 2^-46 of a float rounding
// boundary, and the FP64 pipe, a small fraction of the FP32 rate on GB300,
// is left to cosh/sinh of eta and the delta-f coefficient lookups.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "ffloat.cuh"
#include "kernels.h"

namespace iss {

namespace {

constexpr int kPrologueThreads = 128;

__device__ void bulk14_coeff(const DevTables& t, double T, double muB, double* out) {
    const int idx_T = static_cast<int>((T - t.b14_T0) / t.b14_dT);
    const int idx_mu = static_cast<int>((muB - t.b14_mu0) / t.b14_dmu);
    const double xf = (T - t.b14_T0) / t.b14_dT - idx_T;
    const double yf = (muB - t.b14_mu0) / t.b14_dmu - idx_mu;
    const int nT = t.b14_nT, nmu = t.b14_nmu;
    const int iT1 = min(max(idx_T, 0), nT - 1), iT2 = min(max(idx_T + 1, 0), nT - 1);
    const int im1 = min(max(idx_mu, 0), nmu - 1), im2 = min(max(idx_mu + 1, 0), nmu - 1);
    const double* tabs[3] = {t.b14c0, t.b14c1, t.b14c2};
    double v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double* tb = tabs[k];
        const double f1 = tb[iT1 * nmu + im1], f2 = tb[iT1 * nmu + im2];
        const double f3 = tb[iT2 * nmu + im2], f4 = tb[iT2 * nmu + im1];
        v[k] = f1 * (1. - xf) * (1. - yf) + f2 * (1. - xf) * yf + f3 * xf * yf +
               f4 * xf * (1. - yf);
    }
    const double T3 = T * T * T;
    const double T4 = T3 * T;
    out[0] = (v[0] - v[2]) / T4;
    out[1] = v[1] / T3;
    out[2] = (4. * v[2] - v[0]) / T4;
}

// polynomial fits of FSSW::getbulkvisCoefficients(T), bulk_deltaf_kind 1
// (src/FSSW.cpp:1109-1136), T in 1/fm
__device__ void bulk_rta_coeff(double T, double* out) {
    const double a[11] = {642096.624265727, -8163329.49562861, 47162768.4292073,
                          -162590040.002683, 369637951.096896, -578181331.809836,
                          629434830.225675, -470493661.096657, 230936465.421,
                          -67175218.4629078, 8789472.32652964};
    const double b[11] = {1.18171174036192, -17.6740645873717, 136.298469057177,
                          -635.999435106846, 1918.77100633321, -3836.32258307711,
                          5136.35746882372, -4566.22991441914, 2593.45375240886,
                          -853.908199724349, 124.260460450113};
    const double x = T / 0.197327053;
    double p = 1.0, s0 = a[0], s1 = b[0];
    for (int k = 1; k < 11; k++) {
        p *= x;
        s0 += a[k] * p;
        s1 += b[k] * p;
    }
    out[0] = s0;
    out[1] = s1;
    out[2] = 0.0;
}

__device__ void ce_neos_coeff(const double* tb, double Edec, double nB, double* out) {
    const double de = tb[5 * 200] - tb[0];
    int idx_e = static_cast<int>((Edec - tb[0]) / de);
    idx_e = max(0, min(198, idx_e));
    const int Ne1 = idx_e * 200, Ne2 = (idx_e + 1) * 200;
    const double e_frac = (Edec - tb[5 * Ne1]) / de;
    const double dnB1 = tb[5 * (Ne1 + 1) + 1], dnB2 = tb[5 * (Ne2 + 1) + 1];
    // the reference clamps these indices from above only
    const int i1 = min(198, static_cast<int>(nB / dnB1));
    const int i2 = min(198, static_cast<int>(nB / dnB2));
    const double f1 = fmin(1., (nB - tb[5 * (Ne1 + i1) + 1]) / dnB1);
    const double f2 = fmin(1., (nB - tb[5 * (Ne2 + i2) + 1]) / dnB2);
    double c[3];
#pragma unroll
    for (int i = 2; i < 5; i++) {
        const double t1 = tb[5 * (Ne1 + i1) + i] * (1 - f1) + tb[5 * (Ne1 + i1 + 1) + i] * f1;
        const double t2 = tb[5 * (Ne2 + i2) + i] * (1 - f2) + tb[5 * (Ne2 + i2 + 1) + i] * f2;
        c[i - 2] = t1 * (1. - e_frac) + t2 * e_frac;
    }
    out[0] = 1. / c[1];
    out[1] = 1. / 3. - c[0];
    out[2] = c[2];
}

__device__ double qmu_coeff(const double* tb, double T, double muB) {
    const int idx_T = static_cast<int>((T - 0.05) / 0.001);
    const int idx_mu = static_cast<int>((muB - 0.0) / 0.007892);
    const double xf = (T - 0.05) / 0.001 - idx_T;
    const double yf = (muB - 0.0) / 0.007892 - idx_mu;
    if (idx_mu > 98 || idx_T > 148 || idx_mu < 0 || idx_T < 0) return 1e30;
    const double f1 = tb[idx_T * 100 + idx_mu], f2 = tb[idx_T * 100 + idx_mu + 1];
    const double f3 = tb[(idx_T + 1) * 100 + idx_mu + 1], f4 = tb[(idx_T + 1) * 100 + idx_mu];
    return f1 * (1. - xf) * (1. - yf) + f2 * (1. - xf) * yf + f3 * xf * yf + f4 * xf * (1. - yf);
}

__global__ void __launch_bounds__(kPrologueThreads)
cell_prologue_kernel(DevConfig cfg, const float* __restrict__ fo34, int64_t n, CellArrays cells) {
    __shared__ float s_rec[kPrologueThreads * 34];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kPrologueThreads;
    const int64_t nrec = min(static_cast<int64_t>(kPrologueThreads), n - base);
    for (int k = threadIdx.x; k < nrec * 34; k += kPrologueThreads) s_rec[k] = fo34[base * 34 + k];
    __syncthreads();
    if (threadIdx.x >= nrec) return;
    const int64_t l = base + threadIdx.x;
    const float* s = s_rec + threadIdx.x * 34;
    const float tau = s[0], xpt = s[1], ypt = s[2], eta = s[3];
    const float da0 = s[4], da1 = s[5], da2 = s[6], da3 = s[7];
    const float u1 = s[9], u2 = s[10], u3 = s[11];
    const float Edec = s[12], Tdec = s[13], Pdec = s[14], Bn = s[15];
    const float q1 = s[31], q2 = s[32], q3 = s[33];
    float pi[10];
    for (int k = 0; k < 10; k++) pi[k] = s[19 + k];

    // regulate_surface_cells.  Each double temporary of the reference is a
    // float-float value here; float operations stay float, in the
    // reference's order (C++ promotes a float product to double only after
    // rounding it to float).
    const float u0 = ff_to_float(ff_sqrt(
        ff_add(ff_add(ff_two_sum(1.0f, u1 * u1), ff_of(u2 * u2)), ff_of(u3 * u3))));
    const float q0 = ((u1 * q1 + u2 * q2 + u3 * q3) / u0);
    {
        const float g[4] = {-1.f, 1.f, 1.f, 1.f};
        const float u[4] = {u0, u1, u2, u3};
        const float W[4][4] = {{pi[0], pi[1], pi[2], pi[3]},
                               {pi[1], pi[4], pi[5], pi[6]},
                               {pi[2], pi[5], pi[7], pi[8]},
                               {pi[3], pi[6], pi[8], pi[9]}};
        ff udp[4];
        for (int i = 0; i < 4; i++) {
            ff t = ff_two_prod(-u[0], W[0][i]);
            t = ff_add(t, ff_two_prod(u[1], W[1][i]));
            t = ff_add(t, ff_two_prod(u[2], W[2][i]));
            udp[i] = ff_add(t, ff_two_prod(u[3], W[3][i]));
        }
        const ff tr = ff_add(ff_add(ff_two_sum(-W[0][0], W[1][1]), ff_of(W[2][2])), ff_of(W[3][3]));
        ff udpdu = ff_of(0.0f);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                udpdu = ff_add(udpdu, ff_mul_f(ff_two_prod(g[i] * u[i], W[i][j]), g[j] * u[j]));
        const ff third = ff{0.333333343f, -9.93410746e-9f};   // 1/3 as a float pair
        const ff trsum = ff_add(tr, udpdu);
        const int ii[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
        const int jj[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
        for (int k = 0; k < 10; k++) {
            const int i = ii[k], j = jj[k];
            const float gij = (i == j) ? g[i] : 0.0f;
            const ff uu = ff_two_prod(u[i], u[j]);
            ff v = ff_add(ff_of(W[i][j]), ff_mul_f(udp[j], u[i]));
            v = ff_add(v, ff_mul_f(udp[i], u[j]));
            v = ff_add(v, ff_mul(uu, udpdu));
            v = ff_sub(v, ff_mul(ff_mul(third, ff_add(ff_of(gij), uu)), trsum));
            pi[k] = ff_to_float(v);
        }
    }

    // transform_to_local_rest_frame (cosh and sinh of the double eta, rounded
    // to float, stay in FP64: every later rounding point depends on them)
    const float ch = static_cast<float>(cosh(static_cast<double>(eta)));
    const float sh = static_cast<float>(sinh(static_cast<double>(eta)));
    const float ut = u0 * ch + u3 * sh;
    const float uz = u3 * ch + u0 * sh;
    const float ux = u1, uy = u2;
    const ff den = ff_two_sum(ut, 1.0f);
    const ff Lxx = ff_add(ff_of(1.0f), ff_div(ff_of(ux * ux), den));
    const ff Lyy = ff_add(ff_of(1.0f), ff_div(ff_of(uy * uy), den));
    const ff Lzz = ff_add(ff_of(1.0f), ff_div(ff_of(uz * uz), den));
    const ff Lxy = ff_div(ff_of(ux * uy), den);
    const ff Lxz = ff_div(ff_of(ux * uz), den);
    const ff Lyz = ff_div(ff_of(uy * uz), den);
    const ff L[4][4] = {{ff_of(ut), ff_of(-ux), ff_of(-uy), ff_of(-uz)},
                        {ff_of(-ux), Lxx, Lxy, Lxz},
                        {ff_of(-uy), Lxy, Lyy, Lyz},
                        {ff_of(-uz), Lxz, Lyz, Lzz}};
    const float da_up[4] = {tau * da0 * ch - da3 * sh, -tau * da1, -tau * da2,
                            -da3 * ch + tau * da0 * sh};
    float dl[4] = {0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) dl[i] = ff_to_float(ff_add(ff_of(dl[i]), ff_mul_f(L[i][j], da_up[j])));
    const float qt[4] = {q0 * ch + q3 * sh, q1, q2, q3 * ch + q0 * sh};
    float ql[4] = {0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) ql[i] = ff_to_float(ff_add(ff_of(ql[i]), ff_mul_f(L[i][j], qt[j])));
    float pt[4][4];
    // 2. * pi * ch * sh is a double product in the reference; the float terms
    // around it are rounded to float first
    pt[0][0] = ff_to_float(ff_add(ff_add(ff_of(pi[0] * ch * ch),
                                         ff_mul_f(ff_two_prod(2.0f * pi[3], ch), sh)),
                                  ff_of(pi[9] * sh * sh)));
    pt[0][1] = pi[1] * ch + pi[6] * sh;
    pt[0][2] = pi[2] * ch + pi[8] * sh;
    pt[0][3] = (pi[0] * ch * sh + pi[3] * (ch * ch + sh * sh) + pi[9] * sh * ch);
    pt[1][0] = pt[0][1];
    pt[1][1] = pi[4];
    pt[1][2] = pi[5];
    pt[1][3] = pi[1] * sh + pi[6] * ch;
    pt[2][0] = pt[0][2];
    pt[2][1] = pi[5];
    pt[2][2] = pi[7];
    pt[2][3] = pi[2] * sh + pi[8] * ch;
    pt[3][0] = pt[0][3];
    pt[3][1] = pt[1][3];
    pt[3][2] = pt[2][3];
    pt[3][3] = ff_to_float(ff_add(ff_add(ff_of(pi[0] * sh * sh),
                                         ff_mul_f(ff_two_prod(2.0f * pi[3], sh), ch)),
                                  ff_of(pi[9] * ch * ch)));
    const int pi_i[5] = {1, 1, 1, 2, 2};
    const int pi_j[5] = {1, 2, 3, 2, 3};
    float pl[5];
    for (int k = 0; k < 5; k++) {
        const int i = pi_i[k], j = pi_j[k];
        float acc = 0.f;
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                acc = ff_to_float(ff_add(ff_of(acc), ff_mul(ff_mul_f(L[i][a], pt[a][b]), L[b][j])));
        pl[k] = acc;
    }

    if (cells.milne) {
        // the regulated surface cell in the Milne frame, as the reference's
        // EmissionFunctionArray reads it (src/iSS.cpp:105-109)
        float4* m = cells.milne + 6 * l;
        m[0] = make_float4(da0, da1, da2, da3);
        m[1] = make_float4(u0, u1, u2, u3);
        m[2] = make_float4(pi[0], pi[1], pi[2], pi[3]);
        m[3] = make_float4(pi[4], pi[5], pi[6], pi[7]);
        m[4] = make_float4(pi[8], pi[9], q0, q1);
        m[5] = make_float4(q2, q3, s[29], 0.0f);
    }
    float4* rec = cells.rec + 8 * l;
    rec[0] = cells.pos[l] = make_float4(tau, xpt, ypt, eta);
    rec[1] = cells.da[l] = make_float4(dl[0], -dl[1], -dl[2], -dl[3]);
    rec[2] = cells.u[l] = make_float4(ut, ux, uy, uz);
    rec[3] = cells.th[l] = make_float4(Tdec, s[16], s[17], s[18]);
    rec[4] = cells.th2[l] = make_float4(Edec, Pdec, Bn, s[29]);
    rec[5] = cells.pi1[l] = make_float4(pl[0], pl[1], pl[2], pl[3]);
    rec[6] = cells.pi2[l] = make_float4(pl[4], ql[1], ql[2], ql[3]);

    double c[3] = {0.0, 0.0, 0.0};
    double kappa = 1.0;
    if (cfg.neos_kind == 1) {
        ce_neos_coeff(cfg.tab.ce, Edec, Bn, c);
    } else if (cfg.include_bulk) {
        if (cfg.bulk_kind == 11) bulk14_coeff(cfg.tab, Tdec, s[16], c);
        else if (cfg.bulk_kind == 1) bulk_rta_coeff(Tdec, c);
    }
    if (cfg.include_diff) kappa = qmu_coeff(cfg.tab.qmu, Tdec, s[16]);
    rec[7] = cells.coef[l] = make_float4(static_cast<float>(c[0]), static_cast<float>(c[1]),
                                         static_cast<float>(c[2]), static_cast<float>(kappa));
    if (cells.srec) {
        // the lean sampler's per-cell constants, from the record's floats
        const float4 da = make_float4(dl[0], -dl[1], -dl[2], -dl[3]);
        const float4 th = make_float4(Tdec, s[16], s[17], s[18]);
        const float4 th2 = make_float4(Edec, Pdec, Bn, s[29]);
        const float4 p1 = make_float4(pl[0], pl[1], pl[2], pl[3]);
        const float4 p2 = make_float4(pl[4], ql[1], ql[2], ql[3]);
        const float4 cf = make_float4(static_cast<float>(c[0]), static_cast<float>(c[1]),
                                      static_cast<float>(c[2]), static_cast<float>(kappa));
        const float T = th.x;
        const float d0 = fabsf(da.x);
        float D = sqrtf(da.y * da.y + da.z * da.z + da.w * da.w);
        float nx = 0.0f, ny = 0.0f, nz = 1.0f;
        if (D > 1e-30f) {
            const float inv = 1.0f / D;
            nx = da.y * inv;
            ny = da.z * inv;
            nz = da.w * inv;
        } else {
            D = 0.0f;
        }
        const float einv = fabsf(nz) < 0.9f ? 1.0f / sqrtf(ny * ny + nx * nx)
                                            : 1.0f / sqrtf(nz * nz + ny * ny);
        // shear prefactor (the sampler divides by p0 for the CE form, neos_kind 1)
        float sc = 0.0f;
        if (cfg.include_shear) {
            if (cfg.neos_kind == 1) sc = 1.0f / (2.0f * cf.z * T);
            else if (cfg.neos_kind == 0) sc = cf.x;
            else sc = 1.0f / (2.0f * T * T * (th2.x + th2.y));
        }
        float cb0 = 0.0f, cb1 = 0.0f, cb2 = 0.0f, cbi0 = 0.0f;
        if (cfg.include_bulk) {
            if (cfg.bulk_kind == 11) {
                const float Pi = th2.w;
                cb0 = Pi * cf.x;
                cb1 = Pi * cf.y;
                cb2 = Pi * cf.z;
            } else if (cfg.bulk_kind == 21 || cfg.bulk_kind == 1) {
                const float Pi = (cfg.bulk_kind == 1) ? th2.w / 0.197327053f : th2.w;
                cbi0 = -cf.x * Pi / (3.0f * T);
                cb1 = cf.x * Pi * cf.y / T;
            }
        }
        float4* sr = cells.srec + 8 * l;
        sr[0] = cfg.hydro_mode == 2 ? make_float4(tau * coshf(eta), xpt, ypt, tau * sinhf(eta))
                                    : make_float4(tau, xpt, ypt, eta);
        sr[1] = make_float4(ut, ux, uy, uz);
        sr[2] = make_float4(d0, D, einv, T);
        sr[3] = make_float4(nx, ny, nz, 1.0f / T);
        // diffusion: n_B / (e + P) and q^mu / kappa_B (the sampler's pq and q)
        float pq = 0.0f, qkx = 0.0f, qky = 0.0f, qkz = 0.0f;
        if (cfg.include_diff) {
            const float ik = 1.0f / cf.w;
            qkx = p2.y * ik;
            qky = p2.z * ik;
            qkz = p2.w * ik;
            pq = th2.z / (th2.x + th2.y);
        }
        sr[4] = make_float4(th.y, th.z, th.w, pq);
        sr[5] = make_float4(p1.x * sc, p1.y * sc, p1.z * sc, p1.w * sc);
        sr[6] = make_float4(p2.x * sc, cb0, cb1, cb2);
        sr[7] = make_float4(cbi0, qkx, qky, qkz);
    }
}

}  // namespace

cudaError_t launch_cell_prologue(const DevConfig& cfg, const float* fo34, int64_t n,
                                 const CellArrays& cells, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((n + kPrologueThreads - 1) / kPrologueThreads);
    cell_prologue_kernel<<<blocks, kPrologueThreads, 0, stream>>>(cfg, fo34, n, cells);
    return cudaGetLastError();
}

}  // namespace iss
