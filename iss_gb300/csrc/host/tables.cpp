#include "tables.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <sstream>

namespace iss {

namespace {

std::string pdg_file(int afterburner) {
    if (afterburner == 2) return "pdg-SMASH.dat";
    if (afterburner == 1) return "pdg-urqmd_v3.3+.dat";
    return "pdg-s95pv1.dat";
}

std::string chosen_file(int afterburner) {
    if (afterburner == 2) return "chosen_particles_SMASH.dat";
    if (afterburner == 1) return "chosen_particles_urqmd_v3.3+.dat";
    return "chosen_particles_s95p-v1.dat";
}

}  // namespace

bool load_resonances(const std::string& particle_table_path, int afterburner,
                     bool quantum_statistics, std::vector<Species>* out, std::string* err) {
    const std::string fn = particle_table_path + "/" + pdg_file(afterburner);
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find pdg file " + fn;
        return false;
    }
    out->clear();
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        Species s{};
        std::string name;
        double width;
        int charm, bottom, giso, ndecays;
        if (!(ss >> s.pid >> name >> s.mass >> width >> s.gspin >> s.baryon >> s.strange >> charm
                 >> bottom >> giso >> s.charge >> ndecays)) {
            continue;
        }
        for (int j = 0; j < ndecays && std::getline(f, line); j++) {
        }
        s.real_idx = static_cast<int32_t>(out->size());
        out->push_back(s);
        if (s.baryon > 0) {
            Species a = s;
            a.pid = -s.pid;
            a.baryon = -s.baryon;
            a.strange = -s.strange;
            a.charge = -s.charge;
            a.real_idx = static_cast<int32_t>(out->size());
            out->push_back(a);
        }
    }
    for (Species& s : *out) {
        s.sign = quantum_statistics ? (s.baryon == 0 ? -1 : 1) : 0;
    }
    return true;
}

bool load_decay_table(const std::string& particle_table_path, int afterburner, DecayTable* out,
                      std::string* err) {
    const std::string fn = particle_table_path + "/" + pdg_file(afterburner);
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find pdg file " + fn;
        return false;
    }
    struct Raw {
        int32_t pid, baryon, strange, charge;
        double mass, width;
        std::vector<DecayChannel> ch;
    };
    std::vector<Raw> raw;
    auto find = [&](int32_t pid) -> int {
        for (size_t i = 0; i < raw.size(); i++)
            if (raw[i].pid == pid) return static_cast<int>(i);
        return -1;
    };
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        Raw r;
        std::string name;
        int gspin, charm, bottom, giso, ndecays;
        if (!(ss >> r.pid >> name >> r.mass >> r.width >> gspin >> r.baryon >> r.strange >> charm >>
              bottom >> giso >> r.charge >> ndecays)) {
            continue;
        }
        for (int j = 0; j < ndecays && std::getline(f, line); j++) {
            std::istringstream cs(line);
            int dummy;
            DecayChannel c{};
            if (!(cs >> dummy >> c.n_daughters >> c.branching_ratio >> c.daughter[0] >> c.daughter[1] >>
                  c.daughter[2] >> c.daughter[3] >> c.daughter[4])) {
                *err = "bad decay channel line in " + fn;
                return false;
            }
            r.ch.push_back(c);
        }
        raw.push_back(r);
        if (r.baryon == 1) {
            Raw a = r;
            a.pid = -r.pid;
            a.baryon = -r.baryon;
            a.strange = -r.strange;
            a.charge = -r.charge;
            for (DecayChannel& c : a.ch) {
                for (int k = 0; k < 5; k++) {
                    const int32_t d = c.daughter[k];
                    if (d == 0) continue;
                    const int idx = find(d);
                    // neutral, non-strange mesons are their own antiparticles
                    // (src/particle_decay.cpp:139-147); unknown daughters are
                    // negated like the others and stay unknown (no product
                    // record of theirs carries the sign)
                    if (idx >= 0 && raw[idx].baryon == 0 && raw[idx].charge == 0 &&
                        raw[idx].strange == 0)
                        c.daughter[k] = d;
                    else
                        c.daughter[k] = -d;
                }
            }
            raw.push_back(a);
        }
    }
    out->particles.clear();
    out->channels.clear();
    for (const Raw& r : raw) {
        DecayParticle p{};
        p.pid = r.pid;
        p.mass = static_cast<float>(r.mass);
        p.width = static_cast<float>(r.width);
        p.stable = (!r.ch.empty() && r.ch[0].n_daughters == 1) ? 1 : 0;
        p.first_channel = static_cast<int32_t>(out->channels.size());
        p.n_channels = static_cast<int32_t>(r.ch.size());
        out->particles.push_back(p);
        double cum = 0.0;
        for (DecayChannel c : r.ch) {
            cum += c.branching_ratio;
            const double x = std::ceil(std::ldexp(cum, 53));
            c.cum53 = x <= 0.0 ? 0 : (x >= 18446744073709551615.0 ? ~0ull : static_cast<uint64_t>(x));
            out->channels.push_back(c);
        }
    }
    // daughters as indices (the first entry with that pid, as
    // particle_decay::get_particle_mass looks it up)
    for (DecayChannel& c : out->channels) {
        for (int k = 0; k < 5; k++) {
            const int32_t d = c.daughter[k];
            c.daughter[k] = (k < c.n_daughters && d != 0) ? find(d) : -1;
        }
    }
    return true;
}

bool load_chosen_species(const std::string& particle_table_path, int afterburner,
                         bool quantum_statistics, std::vector<Species>* out,
                         std::vector<int32_t>* unidentified, std::string* err) {
    std::vector<Species> all;
    if (!load_resonances(particle_table_path, afterburner, quantum_statistics, &all, err)) {
        return false;
    }
    const std::string fn = particle_table_path + "/" + chosen_file(afterburner);
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find chosen particle table " + fn;
        return false;
    }
    std::vector<int> table;
    double v;
    while (f >> v) {
        const int mon = static_cast<int>(v);
        bool found = false;
        for (size_t n = 0; n < all.size(); n++) {
            if (all[n].pid == mon) {
                table.push_back(static_cast<int>(n));
                found = true;
                break;
            }
        }
        if (!found && unidentified) unidentified->push_back(mon);
    }
    // stable sort by mass, as the reference's bubble sort
    std::stable_sort(table.begin(), table.end(),
                     [&](int a, int b) { return all[a].mass < all[b].mass; });
    out->clear();
    for (int n : table) out->push_back(all[n]);
    return true;
}

// ---------------------------------------------------------------------------
// special functions

double bessel_k(int n, double x) {
    // K_n(x) = int_0^inf exp(-x cosh t) cosh(n t) dt.  Trapezoidal rule on the
    // half line; the integrand is entire and decays double-exponentially, so
    // the rule converges geometrically (error ~ exp(-2 pi^2 / (h^2 x))).
    if (!(x > 0.0)) return HUGE_VAL;
    const double h = std::min(0.02, 0.5 / std::sqrt(x));
    const double nu = std::abs(n);
    double acc = 0.5;
    for (int k = 1; k < 400000; k++) {
        const double t = k * h;
        const double lg = nu * t - x * (std::cosh(t) - 1.0);
        const double v = 0.5 * std::exp(lg) * (1.0 + std::exp(-2.0 * nu * t));
        acc += v;
        if (lg < -70.0) break;
    }
    return acc * h * std::exp(-x);
}

double expint_en(int n, double x) {
    // E_n(x) = int_1^inf exp(-x t) t^-n dt: power series (Abramowitz &
    // Stegun 5.1.12) for x <= 1, continued fraction (A&S 5.1.22) by the
    // modified Lentz method above.
    if (n == 0) return std::exp(-x) / x;
    if (x <= 0.0) return n > 1 ? 1.0 / (n - 1) : HUGE_VAL;
    if (x > 1.0) {
        double b = x + n, c = 1e300, d = 1.0 / b, h = d;
        for (int i = 1; i < 100000; i++) {
            const double a = -static_cast<double>(i) * (n - 1 + i);
            b += 2.0;
            d = 1.0 / (a * d + b);
            c = b + a / c;
            const double del = c * d;
            h *= del;
            if (std::abs(del - 1.0) < 1e-16) break;
        }
        return h * std::exp(-x);
    }
    const double gamma_e = 0.57721566490153286061;
    double psi = -gamma_e;
    for (int k = 1; k < n; k++) psi += 1.0 / k;
    double sum = (n == 1) ? (-std::log(x) - gamma_e) : 1.0 / (n - 1);
    double term = 1.0;
    for (int m = 1; m < 500; m++) {
        term *= -x / m;
        const double del = (m != n - 1) ? -term / (m - n + 1) : term * (psi - std::log(x));
        sum += del;
        if (std::abs(del) < 1e-17 * std::abs(sum)) break;
    }
    return sum;
}

void special_function_tables(bool with_bulk, bool with_diffusion, std::vector<double>* K,
                             std::vector<double>* E) {
    K->assign(static_cast<size_t>(kSfLen) * 3, 0.0);
    if (with_diffusion) E->assign(static_cast<size_t>(kSfLen) * kNumExpint, 0.0);
    for (int i = 0; i < kSfLen; i++) {
        const double x = kSfX0 + i * kSfDx;
        if (with_bulk) {
            (*K)[3 * i + 0] = bessel_k(1, x);
            (*K)[3 * i + 2] = bessel_k(3, x);
        }
        (*K)[3 * i + 1] = bessel_k(2, x);
        if (with_diffusion) {
            (*E)[kNumExpint * i + 0] = expint_en(2, x);
            for (int k = 1; k < kNumExpint; k++) (*E)[kNumExpint * i + k] = expint_en(2 * k + 2, x);
        }
    }
}

// ---------------------------------------------------------------------------
// delta-f tables

bool load_bulk14(const std::string& table_path, int afterburner, bool fix_c0,
                 Bulk14Table* out, std::string* err) {
    const std::string dir =
        table_path + "/deltaf_tables/" + (afterburner == 2 ? "smash_box" : "urqmd");
    auto read = [&](const std::string& name, int* nT, int* nmu,
                    std::vector<double>* rows) -> bool {
        std::ifstream f(dir + "/" + name);
        if (!f) {
            *err = "can not find file " + dir + "/" + name;
            return false;
        }
        std::string line;
        std::getline(f, line);
        *nT = std::atoi(line.c_str());
        std::getline(f, line);
        *nmu = std::atoi(line.c_str());
        std::getline(f, line);  // column titles
        double a, b, c;
        rows->clear();
        while (f >> a >> b >> c) {
            rows->push_back(a);
            rows->push_back(b);
            rows->push_back(c);
        }
        return true;
    };
    int nT = 0, nmu = 0, t1, t2;
    std::vector<double> r0, r1, r2;
    if (!read("c1.dat", &nT, &nmu, &r1) || !read("c2.dat", &t1, &t2, &r2) ||
        !read("c0.dat", &t1, &t2, &r0)) {
        return false;
    }
    const size_t n = static_cast<size_t>(nT) * nmu;
    if (r1.size() < 3 * n || r2.size() < 3 * n || (fix_c0 && r0.size() < 3 * n) || nT < 2 ||
        nmu < 2) {
        *err = "malformed 14-moment table in " + dir;
        return false;
    }
    out->nT = nT;
    out->nmu = nmu;
    out->c0.assign(n, 0.0);
    out->c1.assign(n, 0.0);
    out->c2.assign(n, 0.0);
    // file order: mu outer, T inner; stored [iT * nmu + imu]
    for (int j = 0; j < nmu; j++) {
        for (int i = 0; i < nT; i++) {
            const size_t row = static_cast<size_t>(j) * nT + i;
            out->c1[static_cast<size_t>(i) * nmu + j] = r1[3 * row + 2];
            out->c2[static_cast<size_t>(i) * nmu + j] = r2[3 * row + 2];
            if (fix_c0) out->c0[static_cast<size_t>(i) * nmu + j] = r0[3 * row + 2];
        }
    }
    out->T0 = r2[0];
    out->mu0 = r2[1];
    out->dT = r2[3] - r2[0];
    out->dmu = r2[3 * static_cast<size_t>(nT) + 1] - r2[1];
    return true;
}

bool load_ce_neos(const std::string& table_path, int afterburner, std::vector<double>* out,
                  std::string* err) {
    const std::string fn = table_path + "/deltaf_tables/" +
                           (afterburner == 2 ? "smash" : "urqmd") + "/NEoSBQS_CE_deltafCoeff.dat";
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find file " + fn;
        return false;
    }
    std::string header;
    std::getline(f, header);
    out->assign(200 * 200 * 5, 0.0);
    for (size_t k = 0; k < out->size(); k++) {
        if (!(f >> (*out)[k])) {
            *err = "truncated table " + fn;
            return false;
        }
    }
    return true;
}

bool load_qmu_coeff(const std::string& table_path, std::vector<double>* out, std::string* err) {
    const std::string fn = table_path + "/deltaf_tables/Coefficients_RTA_diffusion.dat";
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find file " + fn;
        return false;
    }
    out->assign(150 * 100, 0.0);
    double a, b;
    for (int j = 0; j < 100; j++) {
        for (int i = 0; i < 150; i++) {
            if (!(f >> a >> b >> (*out)[static_cast<size_t>(i) * 100 + j])) {
                *err = "truncated table " + fn;
                return false;
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// HRG EoS regulation

bool load_hrg_eos(const std::string& table_path, int iEOS, int afterburner, HrgEos* out,
                  std::string* err) {
    std::string fn = table_path + "/EOS_tables/";
    if (iEOS == 9 || iEOS == 91) fn += "HRGEOS_PST-";
    else if (iEOS == 12) fn += "HRGNEOS_B-";
    else if (iEOS == 14) fn += "HRGNEOS_BQS-";
    fn += (afterburner == 2) ? "SMASH.dat" : "urqmd_v3.3+.dat";
    std::ifstream f(fn);
    if (!f) {
        *err = "can not find EOS file " + fn;
        return false;
    }
    out->iEOS = iEOS;
    out->rows.clear();
    std::string line;
    std::getline(f, line);
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::vector<double> item(7, 0.0);
        if (iEOS == 9 || iEOS == 91) {
            double ed, P, s, T;
            if (!(ss >> ed >> P >> s >> T)) continue;
            item[0] = ed;
            item[2] = P;
            item[3] = T;
        } else {
            const int ncol = (iEOS == 12) ? 5 : 7;
            bool ok = true;
            for (int i = 0; i < ncol; i++) ok = ok && static_cast<bool>(ss >> item[i]);
            if (!ok) continue;
        }
        out->rows.push_back(item);
    }
    return true;
}

bool hrg_eos_values(const HrgEos& eos, double ed, double nB, double* v) {
    const auto& H = eos.rows;
    const int nBlen = (eos.iEOS == 12 || eos.iEOS == 14) ? 200 : 1;
    if (static_cast<int>(H.size()) <= nBlen) return false;
    const double de = H[nBlen][0] - H[0][0];
    const double e0 = H[0][0];
    const int e_idx = static_cast<int>((ed - e0) / de);
    if (e_idx < 0 || e_idx >= static_cast<int>(H.size() / nBlen) - 2) return false;
    const int i1 = e_idx * nBlen, i2 = (e_idx + 1) * nBlen;
    const double e_frac = (ed - H[i1][0]) / de;
    double f1 = 0, f2 = 0;
    int n1 = 0, n2 = 0;
    if (nBlen > 1) {
        const double d1 = H[i1 + 1][1], d2 = H[i2 + 1][1];
        n1 = std::min(nBlen - 2, static_cast<int>(nB / d1));
        n2 = std::min(nBlen - 2, static_cast<int>(nB / d2));
        f1 = std::min(1., (nB - H[i1 + n1][1]) / d1);
        f2 = std::min(1., (nB - H[i2 + n2][1]) / d2);
    }
    auto col = [&](int c) {
        const double a = H[i1 + n1][c] * (1. - f1) + H[i1 + n1 + 1][c] * f1;
        const double b = H[i2 + n2][c] * (1. - f2) + H[i2 + n2 + 1][c] * f2;
        return a * (1 - e_frac) + b * e_frac;
    };
    v[0] = col(2);
    v[1] = col(3);
    v[2] = v[3] = v[4] = 0.0;
    if (nBlen > 1) {
        for (int c = 4; c < 7; c++) v[c - 2] = col(c);
    }
    return true;
}

}  // namespace iss
