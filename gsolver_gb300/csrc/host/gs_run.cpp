// gs_run.cpp -- the reference's z-loop with its .udf dumps, driving the GPU core.
//
// Mirrors main() (solver_main.cpp:151-251): set-up from the config (process_input),
// dump files created with the UDF1.0 header (dumps.cpp, dump_types.cpp:25-52), then
//   while: if CURRENT_Z >= ZNET[n_Z]: dump all, stop after the last ZNET point, n_Z++
//          propagator(); STEP_N++; CURRENT_Z += ZSTEP
// Supported dump types (FILTER_TYPE NO): flux, maxI, field_axis, plasma_max,
// average_spectrum, full (with NZ_DENOM).  DUMP_FILENAMEi may hold one %s, replaced by
// DUMP_FILENAME_MOD (default empty) as the reference does.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gs_abi.h"
#include "gs_setup.h"

namespace {

std::string g_run_err;

struct Dump {
    std::string type, path;
    int iscomplex = 0, tN = 1, xN = 1, yN = 1, zN = 1, nz_denom = 1;
    long long piece = 0;
};

bool write_header(const Dump& d) {
    FILE* f = std::fopen(d.path.c_str(), "wb");
    if (!f) return false;
    const char name[] = "UDF1.0";
    std::fwrite(name, 1, sizeof(name), f);   // including the terminating zero
    const int hdr[6] = {8, d.iscomplex, d.tN, d.xN, d.yN, d.zN};
    std::fwrite(hdr, sizeof(int), 6, f);
    std::fclose(f);
    return true;
}

bool write_slab(const Dump& d, long long ofs_elems, const double* data, long long n_elems) {
    FILE* f = std::fopen(d.path.c_str(), "r+b");
    if (!f) return false;
    const long long esz = d.iscomplex ? 16 : 8;
    const long long ofs = 7 + 6 * 4 + ofs_elems * esz;
    bool ok = fseeko(f, (off_t)ofs, SEEK_SET) == 0 &&
              std::fwrite(data, (size_t)esz, (size_t)n_elems, f) == (size_t)n_elems;
    std::fclose(f);
    return ok;
}

struct Cfg {
    std::vector<std::pair<std::string, std::string>> pairs, over;
    const std::string* raw(const std::string& k) const {
        for (auto& p : over) if (p.first == k) return &p.second;
        for (auto& p : pairs) if (p.first == k) return &p.second;
        return nullptr;
    }
    // load_namednum*: NAMEi first, then NAME
    const std::string* num(const char* k, int i) const {
        const std::string* v = raw(std::string(k) + std::to_string(i));
        return v ? v : raw(k);
    }
};

}  // namespace

extern "C" const char* gs_run_last_error(void) { return g_run_err.c_str(); }

extern "C" int gs_run_config(const char* config_path, const char* out_dir, int n_overrides, const char* const* keys,
                             const char* const* values, int precision, int device, unsigned long long noise_seed,
                             double noise_sigma, long long max_calls, gs_run_stats* stats) {
    g_run_err.clear();
    gs_setup* S = nullptr;
    int rc = gs_setup_from_config(config_path, n_overrides, keys, values, noise_seed, noise_sigma, &S);
    if (rc) { g_run_err = gs_setup_last_error(); return rc; }
    Cfg cfg;
    {
        FILE* f = std::fopen(config_path, "r");
        char a[512], b[512];
        while (f && std::fscanf(f, "%511s %511s", a, b) == 2) cfg.pairs.emplace_back(a, b);
        if (f) std::fclose(f);
        for (int i = 0; i < n_overrides; i++) cfg.over.emplace_back(keys[i], values[i]);
    }
    int nr, nt, nz;
    gs_setup_grid(S, &nr, &nt, &nz);
    std::vector<double> znet(nz), x(nr);
    double dz = 0, r_max = 0;
    gs_setup_znet(S, znet.data(), &dz, &r_max, x.data());
    gs_params p;
    gs_setup_params(S, &p);
    p.precision = precision;
    p.nonlinear = 1;
    p.device = device;
    gs_tables t;
    gs_setup_tables(S, &t);
    std::vector<double> field(2 * (size_t)nr * nt);
    gs_setup_field(S, field.data());

    // dump_manager_class (dumps.cpp:15-45)
    std::vector<Dump> dumps;
    const std::string* dn = cfg.raw("DUMPS_N");
    const int ndumps = dn ? std::atoi(dn->c_str()) : 0;
    const std::string* modp = cfg.raw("DUMP_FILENAME_MOD");
    const std::string mod = modp ? *modp : "";
    for (int i = 0; i < ndumps; i++) {
        Dump d;
        const std::string* ty = cfg.raw("DUMPTYPE" + std::to_string(i));
        const std::string* fn = cfg.raw("DUMP_FILENAME" + std::to_string(i));
        if (!ty || !fn) { g_run_err = "dump_manager_class: DUMPTYPE/DUMP_FILENAME missing"; gs_setup_destroy(S); return GS_ERR_ARG; }
        const std::string* filt = cfg.num("FILTER_TYPE", i);
        if (filt && filt->compare(0, 2, "NO") != 0) {
            g_run_err = "only FILTER_TYPE NO is supported";
            gs_setup_destroy(S);
            return GS_ERR_UNSUPPORTED;
        }
        char name[1024];
        std::snprintf(name, sizeof(name), fn->c_str(), mod.c_str());
        d.type = *ty;
        d.path = std::string(out_dir && *out_dir ? out_dir : ".") + "/" + name;
        if (d.type == "flux" || d.type == "maxI" || d.type == "plasma_max") {
            d.xN = nr; d.zN = nz; d.piece = nr;
        } else if (d.type == "field_axis") {
            d.iscomplex = 1; d.tN = nt; d.zN = nz; d.piece = nt;
        } else if (d.type == "average_spectrum") {
            d.tN = nt; d.zN = nz; d.piece = nt;
        } else if (d.type == "full") {
            const std::string* zd = cfg.num("NZ_DENOM", i);
            d.nz_denom = zd ? std::atoi(zd->c_str()) : 1;
            d.iscomplex = 1; d.tN = nt; d.xN = nr; d.zN = nz / d.nz_denom; d.piece = (long long)nr * nt;
        } else {
            g_run_err = "dump type " + d.type + " is not supported by this driver";
            gs_setup_destroy(S);
            return GS_ERR_UNSUPPORTED;
        }
        if (!write_header(d)) { g_run_err = "Unable to open file " + d.path; gs_setup_destroy(S); return GS_ERR_ARG; }
        dumps.push_back(d);
    }

    gs_handle* h = nullptr;
    rc = gs_create(&p, &h);
    if (!rc) rc = gs_upload_tables(h, &t);
    if (!rc) rc = gs_set_field(h, field.data(), nullptr);
    if (!rc) {
        int nap = 0;
        gs_setup_apertures(S, &nap, nullptr, nullptr);
        std::vector<double> apz(nap), apr(nap);
        gs_setup_apertures(S, &nap, apz.data(), apr.data());
        rc = gs_set_apertures(h, nap, apz.data(), apr.data(), x.data(), r_max);
    }
    if (rc) {
        g_run_err = gs_last_error(h);
        if (h) gs_destroy(h);
        gs_setup_destroy(S);
        return rc;
    }
    std::vector<double> mI(nr), fl(nr), pm(nr), fa(2 * (size_t)nt), sp(nt), full;
    auto t0 = std::chrono::steady_clock::now();
    double cz = znet[0];
    int n_z = 0;
    unsigned step_n = 0;
    long long calls = 0;
    while (true) {
        if (cz >= znet[n_z]) {
            bool need_mI = false, need_f = false, need_pm = false, need_fa = false, need_s = false, need_full = false;
            for (auto& d : dumps) {
                need_mI |= d.type == "maxI";
                need_f |= d.type == "flux";
                need_pm |= d.type == "plasma_max";
                need_fa |= d.type == "field_axis";
                need_s |= d.type == "average_spectrum";
                need_full |= d.type == "full" && (n_z % d.nz_denom) == 0;
            }
            rc = gs_dump_reductions(h, x.data(), r_max, need_mI ? mI.data() : nullptr, need_f ? fl.data() : nullptr,
                                    need_pm ? pm.data() : nullptr, need_fa ? fa.data() : nullptr,
                                    need_s ? sp.data() : nullptr);
            if (!rc && need_full) {
                full.resize(2 * (size_t)nr * nt);
                rc = gs_get_time_field(h, full.data());
            }
            if (rc) { g_run_err = gs_last_error(h); break; }
            for (auto& d : dumps) {
                bool ok = true;
                if (d.type == "maxI") ok = write_slab(d, (long long)nr * n_z, mI.data(), nr);
                else if (d.type == "flux") ok = write_slab(d, (long long)nr * n_z, fl.data(), nr);
                else if (d.type == "plasma_max") ok = write_slab(d, (long long)nr * n_z, pm.data(), nr);
                else if (d.type == "field_axis") ok = write_slab(d, (long long)nt * n_z, fa.data(), nt);
                else if (d.type == "average_spectrum") ok = write_slab(d, (long long)nt * n_z, sp.data(), nt);
                else if (d.type == "full" && (n_z % d.nz_denom) == 0)
                    ok = write_slab(d, (long long)nt * nr * (n_z / d.nz_denom), full.data(), (long long)nr * nt);
                if (!ok) { g_run_err = "write failed: " + d.path; rc = GS_ERR_ARG; break; }
            }
            if (rc) break;
            if (n_z == nz - 1) break;
            n_z++;
        }
        if (max_calls >= 0 && calls >= max_calls) break;
        // the calls up to the next ZNET point (or the call budget), the step controller on the
        // device where the grid allows (gs_advance; else gs_step per call, the same results)
        const long long left = max_calls >= 0 ? max_calls - calls : (1LL << 30);
        int done = 0, reached = 0;
        rc = gs_advance(h, znet.data(), nz, n_z, &cz, &dz, &step_n, (int)std::min<long long>(left, 1 << 30), &done,
                        &reached);
        calls += done;
        if (rc) { g_run_err = gs_last_error(h); break; }
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) {
        stats->calls = calls;
        stats->step_n = step_n;
        stats->n_z = n_z;
        stats->z = cz;
        stats->zstep = dz;
        stats->seconds = secs;
    }
    gs_destroy(h);
    gs_setup_destroy(S);
    return rc;
}
