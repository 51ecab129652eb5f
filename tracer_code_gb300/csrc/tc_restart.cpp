// tc_restart.cpp -- the reference's restart files, read and written on the
// host (no reference counterpart in the GPU path itself; the formats are the
// reference's).
//
//   Trestart         print_restart (main.f90:301-320) / build_grid
//                    (grid.f90:55-66): one unformatted record
//                    xg(-3:nx+3), zg(-3:nz+3), [T], [Cnew(1:ntype,:,:)], SF
//                    (T when RaT /= 0, Cnew when comp = 1; T, SF and Cnew on
//                    the (-span:nx+span, -span:nz+span) box, i fastest)
//   restart_tracers  print_restart (main.f90:321-330) / grid.f90:74-84: one
//                    record rtr(ntr), str(ntr), then Ttype(ntr) (comp = 1)
//                    and/or Ttr(ntr) (temperature tracers, tracer = 1)
//
// A gfortran unformatted sequential record is a 4-byte little-endian length,
// the payload, and the same length again.  Records of 2^31 bytes or more
// (which gfortran splits into subrecords) are refused.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "tracer_gpu.h"

namespace {

constexpr int kSpan = 2, kSpanX = 3;  // field ghost width; coordinate ghost width (span + span_interp)

struct Part {
    const void* src;
    void* dst;
    size_t bytes;
};

tc_status write_record(const char* path, const std::vector<Part>& parts) {
    size_t total = 0;
    for (const Part& p : parts) total += p.bytes;
    if (total >= (size_t)INT32_MAX) return TC_ERR_TOO_LARGE;
    FILE* f = std::fopen(path, "wb");
    if (!f) return TC_ERR_ARG;
    const int32_t n = (int32_t)total;
    bool ok = std::fwrite(&n, 4, 1, f) == 1;
    for (const Part& p : parts) ok = ok && std::fwrite(p.src, 1, p.bytes, f) == p.bytes;
    ok = ok && std::fwrite(&n, 4, 1, f) == 1;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TC_OK : TC_ERR_ARG;
}

// reads the file's one record, whose length must equal the parts' total
tc_status read_record(const char* path, const std::vector<Part>& parts) {
    size_t total = 0;
    for (const Part& p : parts) total += p.bytes;
    if (total >= (size_t)INT32_MAX) return TC_ERR_TOO_LARGE;
    FILE* f = std::fopen(path, "rb");
    if (!f) return TC_ERR_ARG;
    int32_t n0 = -1, n1 = -2;
    bool ok = std::fread(&n0, 4, 1, f) == 1 && n0 >= 0 && (size_t)n0 == total;
    for (const Part& p : parts) ok = ok && std::fread(p.dst, 1, p.bytes, f) == p.bytes;
    ok = ok && std::fread(&n1, 4, 1, f) == 1 && n1 == n0;
    ok = ok && std::fgetc(f) == EOF;  // the file is this one record
    std::fclose(f);
    return ok ? TC_OK : TC_ERR_ARG;
}

size_t field_count(int nx, int nz) { return (size_t)(nx + 1 + 2 * kSpan) * (size_t)(nz + 1 + 2 * kSpan); }

std::vector<Part> trestart_parts(int nx, int nz, int ntype, int thermal, const double* xg, const double* zg,
                                 const double* T, const double* Cnew, const double* SF, bool reading) {
    const size_t nf = field_count(nx, nz) * sizeof(double);
    auto part = [&](const double* p, size_t bytes) {
        return reading ? Part{nullptr, const_cast<double*>(p), bytes} : Part{p, nullptr, bytes};
    };
    std::vector<Part> v;
    v.push_back(part(xg, sizeof(double) * (size_t)(nx + 1 + 2 * kSpanX)));
    v.push_back(part(zg, sizeof(double) * (size_t)(nz + 1 + 2 * kSpanX)));
    if (thermal) v.push_back(part(T, nf));
    if (ntype > 0) v.push_back(part(Cnew, nf * (size_t)ntype));
    v.push_back(part(SF, nf));
    return v;
}

}  // namespace

extern "C" {

tc_status tc_restart_write(const char* path, int32_t nx, int32_t nz, int32_t ntype, int32_t thermal,
                           const double* xg, const double* zg, const double* T, const double* Cnew,
                           const double* SF) {
    if (!path || nx < 1 || nz < 1 || ntype < 0 || ntype > TC_MAX_TYPES || !xg || !zg || !SF) return TC_ERR_ARG;
    if ((thermal && !T) || (ntype > 0 && !Cnew)) return TC_ERR_ARG;
    return write_record(path, trestart_parts(nx, nz, ntype, thermal, xg, zg, T, Cnew, SF, false));
}

tc_status tc_restart_read(const char* path, int32_t nx, int32_t nz, int32_t ntype, int32_t thermal, double* xg,
                          double* zg, double* T, double* Cnew, double* SF) {
    if (!path || nx < 1 || nz < 1 || ntype < 0 || ntype > TC_MAX_TYPES || !xg || !zg || !SF) return TC_ERR_ARG;
    if ((thermal && !T) || (ntype > 0 && !Cnew)) return TC_ERR_ARG;
    return read_record(path, trestart_parts(nx, nz, ntype, thermal, xg, zg, T, Cnew, SF, true));
}

tc_status tc_restart_tracers_write(const char* path, int64_t ntr, const double* rtr, const double* str,
                                   const int32_t* Ttype, const double* Ttr) {
    if (!path || ntr < 1 || !rtr || !str || (!Ttype && !Ttr)) return TC_ERR_ARG;
    const size_t n = (size_t)ntr;
    std::vector<Part> v = {{rtr, nullptr, 8 * n}, {str, nullptr, 8 * n}};
    if (Ttype) v.push_back({Ttype, nullptr, 4 * n});
    if (Ttr) v.push_back({Ttr, nullptr, 8 * n});
    return write_record(path, v);
}

tc_status tc_restart_tracers_read(const char* path, int64_t ntr, double* rtr, double* str, int32_t* Ttype,
                                  double* Ttr) {
    if (!path || ntr < 1 || !rtr || !str || (!Ttype && !Ttr)) return TC_ERR_ARG;
    const size_t n = (size_t)ntr;
    std::vector<Part> v = {{nullptr, rtr, 8 * n}, {nullptr, str, 8 * n}};
    if (Ttype) v.push_back({nullptr, Ttype, 4 * n});
    if (Ttr) v.push_back({nullptr, Ttr, 8 * n});
    return read_record(path, v);
}

void tc_restart_grid(int32_t nx, int32_t nz, double aspect, double* xg, double* zg) {
    // build_grid's uniform coordinates (grid.f90:46-54, 97-108): x = dr*i,
    // ghosts mirrored about both walls, the end nodes set exactly
    const double dr = aspect / (double)nx, ds = 1.0 / (double)nz;
    double* x = xg + kSpanX;
    double* z = zg + kSpanX;
    for (int i = 0; i <= nx; i++) x[i] = dr * (double)i;
    for (int k = 0; k <= nz; k++) z[k] = ds * (double)k;
    for (int i = 1; i <= kSpanX; i++) {
        x[-i] = -x[i];
        x[nx + i] = aspect - x[nx - i] + aspect;
    }
    for (int k = 1; k <= kSpanX; k++) {
        z[-k] = -z[k];
        z[nz + k] = 1.0 - z[nz - k] + 1.0;
    }
    x[0] = 0.0;
    z[0] = 0.0;
    x[nx] = aspect;
    z[nz] = 1.0;
}

tc_status tc_write_restart(tc_handle* h, const char* trestart, const char* tracers) {
    if (!h || !trestart) return TC_ERR_ARG;
    tc_info info;
    tc_status s = tc_get_info(h, &info);
    if (s != TC_OK) return s;
    tc_params p;
    s = tc_get_params(h, &p);
    if (s != TC_OK) return s;
    const int nx = info.nx, nz = info.nz, ntype = (p.comp == 1) ? p.ntype : 0;
    const size_t nf = field_count(nx, nz);
    std::vector<double> xg(nx + 1 + 2 * kSpanX), zg(nz + 1 + 2 * kSpanX), T(nf), SF(nf), C(nf * (ntype ? ntype : 1));
    std::vector<double> r, st, Tt;
    std::vector<int32_t> tt;
    const bool trc = ((p.comp == 1 || p.tracer == 1) && info.ntr > 0);
    if (trc) {
        r.resize((size_t)info.ntr);
        st.resize((size_t)info.ntr);
        if (p.comp == 1) tt.resize((size_t)info.ntr);
        if (p.tracer == 1) Tt.resize((size_t)info.ntr);
    }
    s = tc_download_state(h, T.data(), ntype ? C.data() : nullptr, SF.data(), trc ? r.data() : nullptr,
                          trc ? st.data() : nullptr, tt.empty() ? nullptr : tt.data());
    if (s == TC_OK && !Tt.empty()) s = tc_download_tracer_temperature(h, Tt.data());
    if (s != TC_OK) return s;
    s = tc_grid_coordinates(h, xg.data(), zg.data());
    if (s != TC_OK) return s;
    s = tc_restart_write(trestart, nx, nz, ntype, p.RaT != 0.0, xg.data(), zg.data(), T.data(), C.data(), SF.data());
    if (s != TC_OK || !trc || !tracers) return s;
    return tc_restart_tracers_write(tracers, info.ntr, r.data(), st.data(), tt.empty() ? nullptr : tt.data(),
                                    Tt.empty() ? nullptr : Tt.data());
}

tc_status tc_read_restart(tc_handle* h, const char* trestart, const char* tracers) {
    if (!h || !trestart) return TC_ERR_ARG;
    tc_info info;
    tc_status s = tc_get_info(h, &info);
    if (s != TC_OK) return s;
    tc_params p;
    s = tc_get_params(h, &p);
    if (s != TC_OK) return s;
    const int nx = info.nx, nz = info.nz, ntype = (p.comp == 1) ? p.ntype : 0;
    const size_t nf = field_count(nx, nz);
    std::vector<double> xg(nx + 1 + 2 * kSpanX), zg(nz + 1 + 2 * kSpanX), T(nf, 0.0), SF(nf), C(nf * (ntype ? ntype : 1));
    s = tc_restart_read(trestart, nx, nz, ntype, p.RaT != 0.0, xg.data(), zg.data(), T.data(), C.data(), SF.data());
    if (s != TC_OK) return s;
    const bool trc = ((p.comp == 1 || p.tracer == 1) && info.ntr > 0);
    std::vector<double> r, st, Tt;
    std::vector<int32_t> tt;
    if (trc) {
        if (!tracers) return TC_ERR_ARG;
        r.resize((size_t)info.ntr);
        st.resize((size_t)info.ntr);
        if (p.comp == 1) tt.resize((size_t)info.ntr);
        if (p.tracer == 1) Tt.resize((size_t)info.ntr);
        s = tc_restart_tracers_read(tracers, info.ntr, r.data(), st.data(), tt.empty() ? nullptr : tt.data(),
                                    Tt.empty() ? nullptr : Tt.data());
        if (s != TC_OK) return s;
    }
    return tc_upload_state_ex(h, T.data(), ntype ? C.data() : nullptr, SF.data(), trc ? r.data() : nullptr,
                              trc ? st.data() : nullptr, tt.empty() ? nullptr : tt.data(),
                              Tt.empty() ? nullptr : Tt.data(), trc ? info.ntr : 0);
}

}  // extern "C"
