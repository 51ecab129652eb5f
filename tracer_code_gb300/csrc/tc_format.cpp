// tc_format.cpp -- the reference's text outputs, formatted on the host as
// gfortran's formatted WRITE lays them out:
//
//   stats.dat               basics.f90:283-314 (local_time = 0 branches)
//   viscosity_smoother.dat  basics.f90:316-322
//   T1xxxx snapshots        snapshots, main.f90:237-270
//   equalize.dat            equalize_tracers, composition.f90:568-574
//
// Fortran edit descriptors used there: Gw.d and Gw.dEe for reals, Iw for
// integers; list-directed WRITE(u,*) " " for the blank line after each
// column of a snapshot.
//
// Gw.d[Ee] output (Fortran 2008 10.7.5.2.2, 10.7.2.3): the value rounded to
// d significant digits is 0.d1...dd x 10^s; when 0 <= s <= d it is written
// as F(w-n).(d-s) followed by n blanks (n = 4, or e + 2 with Ee), otherwise
// as Ew.d[Ee] = [-]0.d1...ddE+xx (exponents above 99 without Ee drop the E:
// +xxx).  Zero is F(w-n).(d-1).  A field that does not fit is w asterisks.
// Rounding is to nearest on the exact binary value (the C library's %e and
// %f conversions give exactly that).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tracer_gpu.h"

namespace {

void stars(std::string& out, int w) { out.append((size_t)w, '*'); }

void right(std::string& out, const std::string& s, int w) {
    if ((int)s.size() > w) return stars(out, w);
    out.append((size_t)(w - (int)s.size()), ' ');
    out += s;
}

void fmt_i(std::string& out, long long v, int w) { right(out, std::to_string(v), w); }

void fmt_g(std::string& out, double x, int w, int d, int e) {
    const int n = (e > 0) ? e + 2 : 4;
    char b[512];
    if (std::isnan(x)) return right(out, "NaN", w);
    if (std::isinf(x)) return right(out, x < 0 ? "-Infinity" : "Infinity", w);
    if (x == 0.0) {
        // F(w-n).(d-1), n blanks; a negative zero keeps its sign
        std::snprintf(b, sizeof b, "%#.*f", d - 1 > 0 ? d - 1 : 0, 0.0);
        std::string s = std::signbit(x) ? std::string("-") + b : std::string(b);
        right(out, s, w - n);
        out.append((size_t)n, ' ');
        return;
    }
    // d significant digits of |x|, correctly rounded: m.mmm e X, value = 0.mmmm x 10^(X+1)
    std::snprintf(b, sizeof b, "%.*e", d - 1, std::fabs(x));
    const char* ep = std::strchr(b, 'e');
    const int s = std::atoi(ep + 1) + 1;
    if (s >= 0 && s <= d) {
        std::snprintf(b, sizeof b, "%#.*f", d - s, x);
        right(out, b, w - n);
        out.append((size_t)n, ' ');
        return;
    }
    std::string digits;
    for (const char* c = b; c < ep; c++)
        if (*c >= '0' && *c <= '9') digits += *c;
    char ex[32];
    const int as = s < 0 ? -s : s;
    if (e > 0) {
        std::snprintf(ex, sizeof ex, "E%c%0*d", s < 0 ? '-' : '+', e, as);
        if ((int)std::strlen(ex) > e + 2) return stars(out, w);
    } else if (as <= 99) {
        std::snprintf(ex, sizeof ex, "E%c%02d", s < 0 ? '-' : '+', as);
    } else if (as <= 999) {
        std::snprintf(ex, sizeof ex, "%c%03d", s < 0 ? '-' : '+', as);
    } else {
        return stars(out, w);
    }
    const std::string sign = (x < 0) ? "-" : "";
    std::string body = sign + "0." + digits + ex;
    if ((int)body.size() > w) body = sign + "." + digits + ex;  // the leading zero is optional
    right(out, body, w);
}

tc_status finish(const std::string& s, char* buf, int32_t cap) {
    if (!buf || cap < 1) return TC_ERR_ARG;
    if ((int64_t)s.size() + 1 > cap) return TC_ERR_TOO_LARGE;
    std::memcpy(buf, s.data(), s.size());
    buf[s.size()] = '\0';
    return TC_OK;
}

constexpr int kSpan = 2;

}  // namespace

extern "C" {

int32_t tc_format_g(double x, int32_t w, int32_t d, int32_t e, char* out) {
    if (!out || w < 1 || w > 200 || d < 1 || d > 60 || e < 0 || e > 9) return -1;
    std::string s;
    fmt_g(s, x, w, d, e);
    std::memcpy(out, s.data(), s.size());
    out[s.size()] = '\0';
    return (int32_t)s.size();
}

tc_status tc_format_stats_line(const tc_stats_row* r, int32_t comp, int32_t tracer, int32_t ntype, double RaT,
                               char* buf, int32_t cap) {
    if (!r || ntype < 0 || ntype > TC_MAX_TYPES) return TC_ERR_ARG;
    std::string s;
    auto g = [&](double v) { fmt_g(s, v, 20, 8, 0); };
    const bool counts = (comp == 1) || (RaT != 0.0 && tracer == 1);
    if (RaT != 0.0) {
        for (double v : {r->time, r->Tavg, r->vrms, r->Nu, r->Nu_bot, r->RaT_avg, r->mobility, r->strain_max, r->q1,
                         r->q2, r->q3, r->q4})
            g(v);
    } else {
        for (double v : {r->time, r->vrms, r->mobility, r->strain_max}) g(v);
    }
    if (counts) {
        fmt_i(s, r->empty_cells, 6);
        fmt_i(s, r->tracer_min, 6);
        fmt_i(s, r->tracer_max, 6);
    }
    if (comp == 1) {
        for (int t = 0; t < ntype; t++) g(r->Cavg[t]);
        for (int t = 0; t < ntype; t++) g(r->ent[t]);
    }
    return finish(s, buf, cap);
}

tc_status tc_format_vis_line(const tc_stats_row* r, int32_t comp, int32_t ntype, double RaT, char* buf,
                             int32_t cap) {
    if (!r || ntype < 0 || ntype > TC_MAX_TYPES) return TC_ERR_ARG;
    std::string s;
    if (RaT == 0.0 && comp != 1) return finish(s, buf, cap);  // the reference writes no row
    fmt_g(s, r->time, 20, 8, 0);
    fmt_i(s, r->n_eta, 5);
    fmt_g(s, r->eig_fine, 20, 8, 0);
    if (RaT != 0.0) fmt_i(s, r->n_temp, 5);
    if (comp == 1)
        for (int t = 0; t < ntype; t++) fmt_i(s, r->n_comp[t], 5);
    return finish(s, buf, cap);
}

tc_status tc_format_equalize_line(double time, const int64_t* row, int32_t len, char* buf, int32_t cap) {
    if (!row || len < 1) return TC_ERR_ARG;
    const int n = (int)row[0];
    if (n < 1 || len != 4 + 3 * n) return TC_ERR_ARG;
    std::string s;
    fmt_g(s, time, 20, 8, 0);
    for (int q = 1; q < len; q++) fmt_i(s, row[q], 10);
    return finish(s, buf, cap);
}

tc_status tc_write_snapshot(tc_handle* h, const char* path) {
    if (!h || !path) return TC_ERR_ARG;
    tc_info info;
    tc_status st = tc_get_info(h, &info);
    if (st != TC_OK) return st;
    tc_params p;
    st = tc_get_params(h, &p);
    if (st != TC_OK) return st;
    const int nx = info.nx, nz = info.nz, ntype = (p.comp == 1) ? p.ntype : 0;
    const size_t fi = (size_t)nx + 1 + 2 * kSpan, nf = fi * ((size_t)nz + 1 + 2 * kSpan);
    const size_t vi = (size_t)nx + 3, nv = vi * ((size_t)nz + 3);
    std::vector<double> T(nf), SF(nf), C((size_t)(ntype ? ntype : 1) * nf), u(nv), w(nv), strain(nf), vis(nf),
        Tvis(nf), Cvis((size_t)(ntype ? ntype : 1) * nf), tmp(nf);
    std::vector<int32_t> cnt(nf * (size_t)(ntype + 1));
    st = tc_download_state(h, T.data(), ntype ? C.data() : nullptr, SF.data(), nullptr, nullptr, nullptr);
    if (st == TC_OK) st = tc_download_velocities(h, u.data(), w.data());
    if (st == TC_OK) st = tc_debug_field(h, "strain", 1, 0, strain.data());
    if (st == TC_OK) st = tc_debug_field(h, "vis_grid", 1, 0, vis.data());
    if (st == TC_OK) st = tc_debug_field(h, "Tvis", 1, 0, Tvis.data());
    for (int t = 0; st == TC_OK && t < ntype; t++) {
        st = tc_debug_field(h, "Cvis", 1, t + 1, tmp.data());
        for (size_t q = 0; q < nf; q++) Cvis[q * ntype + t] = tmp[q];
    }
    const bool counted = (p.comp == 1 || p.tracer == 1);
    if (st == TC_OK && counted) st = tc_download_counts(h, cnt.data());
    if (st != TC_OK) return st;
    std::vector<double> xg(nx + 7), zg(nz + 7);
    st = tc_grid_coordinates(h, xg.data(), zg.data());
    if (st != TC_OK) return st;
    FILE* f = std::fopen(path, "w");
    if (!f) return TC_ERR_ARG;
    std::string line;
    bool ok = true;
    auto g = [&](double v) { fmt_g(line, v, 14, 5, 3); };
    for (int i = 0; i <= nx && ok; i++) {
        for (int k = 0; k <= nz; k++) {
            const size_t q = (size_t)(i + kSpan) + (size_t)(k + kSpan) * fi;
            const size_t qv = (size_t)(i + 1) + (size_t)(k + 1) * vi;
            int nempty = 0;
            const int nct = ntype + 1;  // count_type(0:ntype)
            if (counted)
                for (int t = 0; t < nct; t++) nempty += cnt[q * nct + t];
            line.clear();
            g(xg[i + 3]);
            g(zg[k + 3]);
            if (p.RaT != 0.0) {
                g(T[q]);
                g(SF[q]);
                g(u[qv]);
                g(w[qv]);
                if (p.comp == 0 && p.tracer == 0) {
                    g(vis[q]);
                    g(Tvis[q]);
                } else if (p.comp == 0) {
                    g(strain[q]);
                    g(vis[q]);
                    g(Tvis[q]);
                    fmt_i(line, nempty, 6);
                } else {
                    g(strain[q]);
                    g(vis[q]);
                    g(Tvis[q]);
                    fmt_i(line, nempty, 6);
                    for (int t = 0; t < ntype; t++) g(C[q * ntype + t]);
                    for (int t = 0; t < ntype; t++) g(Cvis[q * ntype + t]);
                }
            } else {
                g(SF[q]);
                g(u[qv]);
                g(w[qv]);
                g(strain[q]);
                g(vis[q]);
                fmt_i(line, nempty, 6);
                for (int t = 0; t < ntype; t++) g(C[q * ntype + t]);
                for (int t = 0; t < ntype; t++) g(Cvis[q * ntype + t]);
            }
            line += '\n';
            ok = ok && std::fwrite(line.data(), 1, line.size(), f) == line.size();
        }
        // list-directed WRITE(101,*) " ": a leading blank, then the one-blank string
        ok = ok && std::fputs("  \n", f) >= 0;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TC_OK : TC_ERR_ARG;
}

}  // extern "C"
