// ref_harness.cpp -- command-line driver around the reference solver's own functions (TEST
// INFRASTRUCTURE: built into oracle/_ref/ with the reference's unmodified sources and the
// stand-ins of oracle/ref_shim; used only by tests and by tests/golden/make_ref_golden.py).
//
//   gsref_<build> CONFIG [KEY VALUE ...] -- MODE [IN] OUT [ARG]
//
// CONFIG and the KEY VALUE overrides are what the reference's own command line takes
// (process_input(argc, argv), process_input.cpp:33-95); the harness runs that start-up in the
// current directory, then one mode:
//   tables OUT            the start-up's tables, scalars, start field and BIGBUFFER2
//   run IN OUT STEPS [DZ0]  FIELD = IN; BIGBUFFER2 = ht_run(FIELD) and the Kerr-limited first
//                         step as process_input.cpp:62-73 does (or DZ0 when given); then the
//                         z-loop of solver_main.cpp:202-225 (computationcycle() ->
//                         propagator()) for STEPS calls or to the last ZNET point (STEPS < 0)
//   nlstep IN OUT DZ      FIELD = IN, ZSTEP = DZ, calculate_NLstep (propagator.cu:268-426)
//   nlresponse IN OUT     calculate_NLresponse of one spectral row (propagator.cu:629-783)
//   plasma IN OUT         calculate_plasmadensity_losses_small of one time row
//                         (ionization.cpp:9-95)
//   qdht IN OUT           ht_run of an [N_R][N_T] array (solver.h:337-346)
// IN is raw complex128 [rows][N_T] (the reference's FIELD layout); OUT is a sequence of
// records: int32 name length, name, int32 kind (0 float64, 1 complex128), int64 count, data.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "solver.h"
#include "ionization.h"

void calculate_NLresponse(f_complex* input, f_complex* output);
void calculate_NLstep(float_type* maxI, float_type* maxNL2);
void init_zstep_kerr();

namespace {

struct Out {
    FILE* f;
    explicit Out(const char* path) : f(fopen(path, "wb")) {
        if (!f) {
            fprintf(stderr, "cannot write %s\n", path);
            exit(4);
        }
    }
    ~Out() { fclose(f); }
    void put(const char* name, int kind, const void* data, long long count) {
        const int nl = (int)strlen(name);
        fwrite(&nl, 4, 1, f);
        fwrite(name, 1, nl, f);
        fwrite(&kind, 4, 1, f);
        fwrite(&count, 8, 1, f);
        fwrite(data, kind ? 16 : 8, (size_t)count, f);
    }
    void real(const char* name, const double* d, long long n) { put(name, 0, d, n); }
    void cplx(const char* name, const f_complex* d, long long n) { put(name, 1, d, n); }
    void scalar(const char* name, double v) { put(name, 0, &v, 1); }
};

std::vector<f_complex> read_c128(const char* path, size_t n) {
    std::vector<f_complex> v(n);
    FILE* f = fopen(path, "rb");
    if (!f || fread(v.data(), 16, n, f) != n) {
        fprintf(stderr, "cannot read %zu complex values from %s\n", n, path);
        exit(4);
    }
    fclose(f);
    return v;
}

// process_input.cpp:62-73 with FIELD given: time-domain copy, Kerr-limited first step,
// BIGBUFFER2 = ht_run(FIELD)
void restart_from_field(const std::vector<f_complex>& field) {
    const size_t n = (size_t)N_T * MY_NX * MY_NY;
    memcpy(FIELD, field.data(), n * sizeof(f_complex));
    fftwt_execute(FFT_ALLBWPLAN_T);
    fftwt_Nnormalize(MY_NX * MY_NY, BIGBUFFER1);
    init_zstep_kerr();
    memcpy(BIGBUFFER2, FIELD, n * sizeof(f_complex));
    ht_run(BIGBUFFER2, BIGBUFFER1);
    CURRENT_Z = ZNET[0];
    n_Z = 0;
    STEP_N = 0;
}

int run_mode(const std::string& mode, int na, char** a) {
    const size_t nfield = (size_t)N_T * MY_NX * MY_NY;
    if (mode == "tables" && na == 1) {
        Out o(a[0]);
        o.scalar("n_t", N_T);
        o.scalar("n_r", N_X);
        o.scalar("tstep", TSTEP);
        o.scalar("tmin", TMIN);
        o.scalar("tmax", TMAX);
        o.scalar("omega0", OMEGA0);
        o.scalar("omega_min", OMEGA_MIN);
        o.scalar("omega_max", OMEGA_MAX);
        o.scalar("max_tolerance", MAX_TOLERANCE);
        o.scalar("group_velocity", GROUP_VELOCITY);
        o.scalar("ionization_potential", IONIZATION_POTENTIAL);
        o.scalar("ponderomotive", PONDEROMOTIVE_COEFFICIENT);
        o.scalar("avalanche_cs", AVALANCHE_CROSSSECTION);
        o.scalar("recombination_tau", RECOMBINATION_TAU);
        o.scalar("raman_fraction", RAMAN_FRACTION);
        o.scalar("n2", NONLIN_REFRINDEX);
        o.scalar("neutral_density", NEUTRAL_DENSITY);
        o.scalar("init_zstep", ZSTEP);
        o.scalar("r_max", XMAX);
        o.real("omega", OMEGA, N_T);
        o.cplx("wavenum", WAVENUMBER, N_T);
        o.real("ho_disp", HO_DISPERSION, N_T);
        o.real("kerr", KERR_PROFILE, N_T);
        o.cplx("plasma_func", PLASMA_FUNC, N_T);
        o.cplx("raman_func", RAMAN_FUNCTION, N_T);
#ifdef MULTI_LEVEL_IONIZATION
        o.real("rate_ln", IONIZATION_RATE_LN, (long long)IONIZATION_N * IONIZATION_LEVEL_N);
        o.real("ion_potentials", IONIZATION_POTENTIALS, IONIZATION_LEVEL_N);
        o.scalar("th_kerr_ratio", KERR_PROFILE[0] != 0 ? KERR_TH_PROFILE[0] / KERR_PROFILE[0] : 0.0);
#else
        o.real("rate_ln", IONIZATION_RATE_LN, IONIZATION_N);
#endif
        o.real("znet", ZNET, N_Z);
        std::vector<double> x(N_X);
        for (int i = 0; i < N_X; i++) x[i] = HT_PLAN->x_n(i);
        o.real("qdht_x", x.data(), N_X);
        o.cplx("field", FIELD, (long long)nfield);
        o.cplx("bb2", BIGBUFFER2, (long long)nfield);
        return 0;
    }
    if (mode == "run" && (na == 3 || na == 4)) {
        restart_from_field(read_c128(a[0], nfield));
        const double init_zstep = ZSTEP;
        if (na == 4) ZSTEP = atof(a[3]);
        const long long steps = atoll(a[2]);
        long long calls = 0;
        while (true) {   // solver_main.cpp:202-225 without the dumps
            if (CURRENT_Z >= ZNET[n_Z]) {
                if (n_Z == N_Z - 1) break;
                n_Z++;
            }
            if (steps >= 0 && calls >= steps) break;
            computationcycle();
            CURRENT_Z += ZSTEP;
            calls++;
        }
        Out o(a[1]);
        o.scalar("init_zstep", init_zstep);
        o.scalar("z", CURRENT_Z);
        o.scalar("zstep", ZSTEP);
        o.scalar("step_n", STEP_N);
        o.scalar("n_z", n_Z);
        o.scalar("calls", (double)calls);
        o.cplx("field", FIELD, (long long)nfield);
        o.cplx("bb2", BIGBUFFER2, (long long)nfield);
        return 0;
    }
    if (mode == "nlstep" && na == 3) {
        std::vector<f_complex> f = read_c128(a[0], nfield);
        memcpy(FIELD, f.data(), nfield * sizeof(f_complex));
        ZSTEP = atof(a[2]);
        float_type a2 = 0, n2 = 0;
        calculate_NLstep(&a2, &n2);
        Out o(a[1]);
        o.scalar("max_a2", a2);
        o.scalar("max_nl2", n2);
        o.cplx("bb1", BIGBUFFER1, (long long)nfield);
        return 0;
    }
    if (mode == "nlresponse" && na == 2) {
        std::vector<f_complex> in = read_c128(a[0], N_T), out(N_T);
        calculate_NLresponse(in.data(), out.data());
        Out o(a[1]);
        o.cplx("nl", out.data(), N_T);
        return 0;
    }
    if (mode == "plasma" && na == 2) {
        std::vector<f_complex> e = read_c128(a[0], N_T), loss(N_T), n2f(N_T);
        std::vector<double> pro(N_T);
        calculate_plasmadensity_losses_small(e.data(), pro.data(), 1, loss.data(), n2f.data());
        Out o(a[1]);
        o.real("rho", pro.data(), N_T);
        o.cplx("loss", loss.data(), N_T);
        return 0;
    }
    if (mode == "qdht" && na == 2) {
        std::vector<f_complex> d = read_c128(a[0], nfield);
        ht_run(d.data(), BIGBUFFER1);
        Out o(a[1]);
        o.cplx("y", d.data(), (long long)nfield);
        return 0;
    }
    fprintf(stderr, "bad mode or arguments: %s\n", mode.c_str());
    return 5;
}

}  // namespace

int main(int argc, char** argv) {
    int sep = -1;
    for (int i = 1; i < argc; i++)
        if (strcmp(argv[i], "--") == 0) {
            sep = i;
            break;
        }
    if (sep < 2 || sep + 1 >= argc) {
        fprintf(stderr, "usage: %s CONFIG [KEY VALUE ...] -- MODE [IN] OUT [ARG]\n", argv[0]);
        return 2;
    }
    int rc = 0;
    try {
        MPI_Init(&argc, &argv);
        MPI_Comm_size(MPI_COMM_WORLD, &PROCESS_N);
        MPI_Comm_rank(MPI_COMM_WORLD, &PROCESS_RANK);
        _ARGC = sep;   // the reference's own command line: program, CONFIG, overrides
        _ARGV = argv;
        fftwt_mpi_init();
        srand48(12345);
        STEP_N = 0;
        process_input(sep, argv);
        rc = run_mode(argv[sep + 1], argc - sep - 2, argv + sep + 2);
    } catch (const char* msg) {
        fprintf(stderr, "\nreference error: %s\n", msg);
        rc = 6;
    } catch (char* msg) {
        fprintf(stderr, "\nreference error: %s\n", msg);
        rc = 6;
    }
    fflush(stdout);
    return rc;
}
