// gs_nl_row16k.cu -- calculate_NLstep (propagator.cu:375-425) for rows of 16384 complex FP32
// samples: one CTA of 1024 threads runs a radial row's four RK4 stages in turn (the
// 1024 x 16384 fused-silica workload's NL kernel).
//
// Thread t owns the 16 consecutive samples 16t .. 16t+15 in time and the 16 consecutive
// spectral positions 16t .. 16t+15, so:
//   * the radix-4 pass of each FFT (the last pass of the forward transform, the first of the
//     inverse) runs in registers: the forward one inside the spectral combination, the inverse
//     one where the next stage's input (A + c dz k) / N is formed, both on the thread's own
//     positions; the remaining radix-16 passes depend on the thread's quad (pass 2), its
//     4-warp group (pass 1) or the whole row (pass 0), and synchronise only that far;
//   * the per-sample recurrences (rates, Raman sums, carrier density, sources) run on the
//     thread's own samples, as in the general fused kernel (gs_nl_fused.cu).
// The RK4 sum k1 + 2 k2 + 2 k3 and the row's A (FIELD at the step's start) live in tensor
// memory (tcgen05.st / ld), 32 columns each per thread: k of stages 0-2 never leaves the SM.
// The FFT arithmetic (radix-16 butterflies, radix-4 butterflies) is that of the shared-memory
// FFT in gs_internal.cuh; the twiddles of pass 0 come from its per-stage base rows, those of
// passes 1 and 2 (w_1024^{q r}, w_64^{q r}: 960 and 45 values) from tables in shared memory,
// each value rounded once from FP64.
//
// The Raman response (solver_main.cpp:401-413, propagator.cu:694-705) is the one-pole
// recurrence z_t = a z_{t-1} + I_t; the Kerr factor needs Im(v_t) for
// v_t = (1 - a^N) z_t + a^{t+1} z_{N-1}, which obeys v_t = a v_{t-1} + (1 - a^N) I_t with
// v_{t0-1} = (1 - a^N) z_{t0-1} + a^{t0} z_{N-1} at a chunk start: one complex multiply-add
// per sample.  Chunk starts z_{16c-1} come from a scan whose multiplier a^16 is the same for
// every chunk, so the scan needs only the powers a^{16 j} (a table in shared memory).
#include <type_traits>

#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_plasma.cuh"

namespace gs {
namespace r16k {

constexpr int N = 16384;   // samples per row
constexpr int NT = 1024;   // threads per row
constexpr int L = 16;      // samples / positions per thread
constexpr int LOGN = 14;
static_assert(N == NT * L, "one chunk of 16 per thread");

// shared memory (bytes): E row (padded), rates W_t (padded), chunk starts of the density,
// a^{16 j} (j < 1024), Raman warp totals and prefixes, density scan scratch, warp maxima, the
// twiddles of radix-16 passes 2 and 1, flag
constexpr int OFF_E = 0;
constexpr int OFF_W = OFF_E + (N + N / 16) * 8;
constexpr int OFF_S = OFF_W + ((N + N / 32 + 1 + 3) & ~3) * 4;
constexpr int OFF_APW = OFF_S + NT * 4;
constexpr int OFF_WTOT = OFF_APW + NT * 8;
constexpr int OFF_WPRE = OFF_WTOT + 32 * 8;
constexpr int OFF_RA = OFF_WPRE + 32 * 8;
constexpr int OFF_RB = OFF_RA + 32 * 4;
constexpr int OFF_MX = OFF_RB + 32 * 4;
constexpr int OFF_TW2 = OFF_MX + 32 * 4;   // w_64^{q r}, q = 1..3, r = 1..15 (45 complex)
constexpr int OFF_TW1 = OFF_TW2 + 48 * 8;  // w_1024^{q r}, r = 1..15, q = 0..63 ([r - 1][q])
constexpr int OFF_FLAG = OFF_TW1 + 15 * 64 * 8;
constexpr int SMEM = OFF_FLAG + 16;
static_assert(SMEM + 16 <= 227 * 1024, "fits one CTA");

// ---- tensor memory: 8 columns (4 complex) per access, the wait separate so that two loads
// overlap; the wait names the registers so that nothing reads them before it
__device__ __forceinline__ void tld8(uint32_t ta, float* v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "r"(ta)
                 : "memory");
}
__device__ __forceinline__ void tld_wait(float* v) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7])
                 :
                 : "memory");
}
__device__ __forceinline__ void tld_wait2(float* v, float* w) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                   "+f"(w[0]), "+f"(w[1]), "+f"(w[2]), "+f"(w[3]), "+f"(w[4]), "+f"(w[5]), "+f"(w[6]), "+f"(w[7])
                 :
                 : "memory");
}
__device__ __forceinline__ void tst8(uint32_t ta, const float* v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(ta),
                 "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tst_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// the threads of one 4-warp group (128 threads: named barriers 1..8)
__device__ __forceinline__ void bar_group(int t) {
    asm volatile("bar.sync %0, 128;" ::"r"(1 + (t >> 7)) : "memory");
}

// x[r] *= w_64^{SIGN-sign q r}, r = 1..15, from the shared table of pass 2 (q = 1..3: a warp
// reads four addresses, broadcast; forward values, conjugated for the inverse)
template <int SIGN>
__device__ __forceinline__ void tw64(float2* x, const float2* tw2, int q) {
#pragma unroll
    for (int r = 1; r < 16; r++) {
        float2 w = tw2[(q - 1) * 15 + r - 1];
        if (SIGN > 0) w.y = -w.y;
        x[r] = cmul(x[r], w);
    }
}

// x[r] *= w_1024^{SIGN-sign q r}, r = 1..15, from the shared table of pass 1 (a warp reads 32
// consecutive entries per r)
template <int SIGN>
__device__ __forceinline__ void tw1024(float2* x, const float2* tw1, int q) {
#pragma unroll
    for (int r = 1; r < 16; r++) {
        float2 w = tw1[(r - 1) * 64 + q];
        if (SIGN > 0) w.y = -w.y;
        x[r] = cmul(x[r], w);
    }
}

// One radix-16 pass of the 16384-point FFT, butterfly t of sub-problems of size S (the
// fft_stage_ct butterfly: the same loads, twiddles from the stage's base rows, DFT and stores);
// the sub-problems of 64 (q < 4) and of 1024 (q < 64) take their twiddles from the shared
// tables tws (tw2, tw1).
template <int SIGN, int S>
__device__ __forceinline__ void pass16(float2* E, const float2* __restrict__ stb, int t, const float2* tws = nullptr) {
    constexpr int sub = S / 16;
    const int q = t & (sub - 1);
    float2* p = E + pad16((t / sub) * S + q);
    float2 x[16];
#pragma unroll
    for (int r = 0; r < 16; r++) x[r] = p[pad16(sub * r)];
    if (SIGN > 0 && q != 0) {
        if constexpr (S == 64) tw64<SIGN>(x, tws, q);
        else if constexpr (S == 1024) tw1024<SIGN>(x, tws, q);
        else apply_tw16<SIGN, float>(x, stb, sub, q);
    }
    RegDFT<16, SIGN, float, float2>::run(x);
    if (SIGN < 0 && q != 0) {
        if constexpr (S == 64) tw64<SIGN>(x, tws, q);
        else if constexpr (S == 1024) tw1024<SIGN>(x, tws, q);
        else apply_tw16<SIGN, float>(x, stb, sub, q);
    }
#pragma unroll
    for (int r = 0; r < 16; r++) p[pad16(sub * r)] = x[r];
}

// the twiddle base rows of radix-16 pass j (sub-problems of 16384 / 16^j)
__device__ __forceinline__ const float2* stage_base(const float2* twb, int j) { return twb + tw_base_offset(LOGN, j); }

// inverse transform after the radix-4 pass: every thread has written its 16 positions
__device__ __forceinline__ void inverse_rest(float2* E, const float2* __restrict__ twb, int t, const float2* tw2,
                                             const float2* tw1) {
    __syncwarp();                                  // pass 2 reads the quad's positions
    pass16<+1, 64>(E, nullptr, t, tw2);
    bar_group(t);                                  // pass 1 reads the 4-warp group's
    pass16<+1, 1024>(E, nullptr, t, tw1);
    __syncthreads();                               // pass 0 reads the whole row
    pass16<+1, 16384>(E, stage_base(twb, 0), t);
    __syncthreads();
}

// forward transform up to the radix-4 pass (the caller synchronised the row before)
__device__ __forceinline__ void forward_head(float2* E, const float2* __restrict__ twb, int t, const float2* tw2,
                                             const float2* tw1) {
    pass16<-1, 16384>(E, stage_base(twb, 0), t);
    __syncthreads();
    pass16<-1, 1024>(E, nullptr, t, tw1);
    bar_group(t);
    pass16<-1, 64>(E, nullptr, t, tw2);
    __syncwarp();                                  // the radix-4 pass reads the quad's positions
}

// the radix-4 pass on positions 16t + 4g .. + 3 (sub-problems of 4: no twiddles)
template <int SIGN>
__device__ __forceinline__ void radix4(float2* x) {
    RegDFT<4, SIGN, float, float2>::run(x);
}


// The row's four RK4 stages (step f.dzs): stage s's input is (A + c_s dz k_{s-1}) / N with
// c = 0, 1/2, 1/2, 1, its k feeds the RK4 sum (k1 + 2 k2 + 2 k3 + k4) / 6 written to sp.nb
// (when set) and, when sp.nbc is set, its spectral-window positions compactly; max |A|^2 and max |nb|^2
// go to f.max_out and sp.max_out.  FIELD is read from sp.ac (compact window columns) when set,
// else from A.
__global__ void __launch_bounds__(NT, 1) nl_row16k_kernel(FftArgs<float> f, PlasmaArgs<float> a,
                                                         const float2* __restrict__ A, SpecArgs<float> sp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t tslot;
    float2* const E = reinterpret_cast<float2*>(smem_raw + OFF_E);
    float* const Wb = reinterpret_cast<float*>(smem_raw + OFF_W);
    float* const s_start = reinterpret_cast<float*>(smem_raw + OFF_S);
    float2* const apw = reinterpret_cast<float2*>(smem_raw + OFF_APW);
    float2* const wtot = reinterpret_cast<float2*>(smem_raw + OFF_WTOT);
    float2* const wpre = reinterpret_cast<float2*>(smem_raw + OFF_WPRE);
    float* const rA = reinterpret_cast<float*>(smem_raw + OFF_RA);
    float* const rB = reinterpret_cast<float*>(smem_raw + OFF_RB);
    float* const wmx = reinterpret_cast<float*>(smem_raw + OFF_MX);
    float2* const tw2 = reinterpret_cast<float2*>(smem_raw + OFF_TW2);
    float2* const tw1 = reinterpret_cast<float2*>(smem_raw + OFF_TW1);
    int* const flag = reinterpret_cast<int*>(smem_raw + OFF_FLAG);
    if (f.halt && *f.halt) return;   // gs_advance: the z-loop stopped (the whole CTA returns)
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int row = blockIdx.x;
    const size_t base = (size_t)row * N;
    const int t0 = t * L;
    float2* const Ec = E + pad16(t0);   // the thread's samples / positions (pad16(t0 + i) = pad16(t0) + i)
    float* const Wc = Wb + pad32(t0);
    const float2* const twb = f.twb;

    // ---- stage 0's input: FIELD (compact window columns or the full row); the loads are issued
    // before the set-up below so that their latency overlaps it
    float2 x[L];
    const float* acr = (sp.ac && !(f.ac_on && *f.ac_on == 0)) ? sp.ac + (size_t)row * sp.ncw : nullptr;
    if (acr) {   // the thread's positions from their window column pairs (zero outside)
        int cc[L];
#pragma unroll
        for (int h = 0; h < L / 4; h++) {
            const int4 v = __ldg(reinterpret_cast<const int4*>(sp.cinv + t0) + h);
            cc[4 * h] = v.x;
            cc[4 * h + 1] = v.y;
            cc[4 * h + 2] = v.z;
            cc[4 * h + 3] = v.w;
        }
#pragma unroll
        for (int i = 0; i < L; i++)
            x[i] = (cc[i] >= 0 && in_bounds(cc[i] + 2 <= sp.ncw, a.err)) ? *reinterpret_cast<const float2*>(acr + cc[i])
                                                                       : make_float2(0.f, 0.f);
    } else {
        const float4* a4 = reinterpret_cast<const float4*>(A + base + t0);
#pragma unroll
        for (int h = 0; h < L / 2; h++) {
            const float4 v = a4[h];
            x[2 * h] = make_float2(v.x, v.y);
            x[2 * h + 1] = make_float2(v.z, v.w);
        }
    }

    // tensor memory: per thread 32 columns of the RK4 sum, then 32 of A, in its warp's lanes
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tslot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // a^{16 j}: the Raman scan's multipliers and each chunk's a^{t0}
    const bool rscan = a.raman_scan != 0;
    const float2 ra = make_float2(a.k.a_re, a.k.a_im);
    if (rscan) {
        float2 a16 = ra;
#pragma unroll
        for (int i = 0; i < 4; i++) a16 = cmul(a16, a16);
        float2 b = a16, pr = make_float2(1.f, 0.f);
        for (int e = t; e > 0; e >>= 1) {
            if (e & 1) pr = cmul(pr, b);
            b = cmul(b, b);
        }
        apw[t] = pr;
    }
    if (t < 45) {   // w_64^{q r} = w_16384^{256 q r} from the row's table (256 q r < 16384)
        const int q = 1 + t / 15, r = 1 + t % 15;
        tw2[t] = __ldg(f.tw + 256 * q * r);
    }
    if (t < 15 * 64) {   // w_1024^{q r} = w_16384^{16 q r} from the row's table (16 q r < 16384)
        const int q = t & 63, r = 1 + (t >> 6);
        tw1[t] = __ldg(f.tw + 16 * q * r);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tslot + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(64 * (w >> 2));

    const float sc = 1.0f / (float)N;   // the inverse transform's 1/N, exact on 2^14 points
    const double dzs = f.dz_dev ? *f.dz_dev : f.dzs;
    const float c_half = (float)(dzs * 0.5), c_full = (float)dzs;

    // ---- stage 0's input into tensor memory (loaded above)
    {
#pragma unroll
        for (int g = 0; g < 4; g++) tst8(tm + 32 + 8 * g, reinterpret_cast<const float*>(&x[4 * g]));
        float amax = 0.f;
#pragma unroll
        for (int i = 0; i < L; i++) amax = fmaxf(amax, x[i].x * x[i].x + x[i].y * x[i].y);
        for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        if (lane == 0) wmx[w] = amax;   // one atomic per row, after the next barrier
        // the row that takes this SM's next slot: its input travels to L2 meanwhile
        if (t < 32 && f.ahead > 0 && row + f.ahead < f.rows) {
            if (acr) prefetch_row_l2(acr + (size_t)f.ahead * sp.ncw, (size_t)sp.ncw * sizeof(float), t);
            else prefetch_row_l2(A + base + (size_t)f.ahead * N, (size_t)N * sizeof(float2), t);
        }
#pragma unroll
        for (int g = 0; g < 4; g++) {
            float2* y = &x[4 * g];
#pragma unroll
            for (int i = 0; i < 4; i++) y[i] = make_float2(y[i].x * sc, y[i].y * sc);
            radix4<+1>(y);
#pragma unroll
            for (int i = 0; i < 4; i++) Ec[4 * g + i] = y[i];
        }
        tst_wait();
    }

    const bool gas = a.gas != 0;
    const bool kerr = sp.kerr_on != 0;
    const float ND = a.k.ND, tstep = a.k.tstep, U = a.k.U, Pc = a.k.Pc, AV = a.k.AV;
    const float invND = a.k.invND, invTAU = a.k.invTAU;
    const float2 oma = make_float2(a.k.oma_re, a.k.oma_im);
    const float fRM = a.k.fRM, omf = a.k.omf;
    float nmax = 0.f;
#pragma unroll 1
    for (int s = 0; s < 4; s++) {
        // ---- E = IFFT(stage input) / N (propagator.cu:386-396, 640-641)
        inverse_rest(E, twb, t, tw2, tw1);

        // ---- one pass over the thread's samples: rates W_t (the first sample is taken as
        // E_0 = 0: W_0 = 0) and the Raman chunk sum; groups of 8 samples, whose table reads are
        // issued together when a sample of the warp is at or above the table threshold
        bool anyw = false;
        float2 zl = make_float2(0.f, 0.f);
#pragma unroll
        for (int g = 0; g < L; g += 8) {
            float Iv[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const float2 e = Ec[g + u];
                Iv[u] = e.x * e.x + e.y * e.y;
                if (rscan) {
                    zl = cmul(ra, zl);
                    zl.x += Iv[u];
                }
            }
            bool above = false;
#pragma unroll
            for (int u = 0; u < 8; u++) above = above || (t0 + g + u > 0 && !(Iv[u] < (float)(1e13 / 1e16)));
            float W[8];
            if (__any_sync(0xffffffffu, above)) {
                int n[8];
                float dl[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    dl[u] = 0.f;
                    n[u] = (t0 + g + u > 0) ? photo_index<float>(Iv[u], &dl[u], a.err) : -1;
                    if (n[u] >= 0 && !in_bounds(n[u] + 1 < 8192, a.err)) n[u] = -1;
                }
                float w0[8], w1[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    w0[u] = n[u] >= 0 ? __ldg(&a.rate[n[u]]) : 0.f;
                    w1[u] = n[u] >= 0 ? __ldg(&a.rate[n[u] + 1]) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    W[u] = n[u] >= 0 ? photo_rate_from<float>(w0[u], w1[u], dl[u]) : 0.f;
                    anyw = anyw || n[u] >= 0;
                }
            } else {
#pragma unroll
                for (int u = 0; u < 8; u++) W[u] = 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) Wc[g + u] = gas ? gas_rate_slot<float>(t0 + g + u, Iv[u], W[u]) : W[u];
        }
        // Raman: chunk sums scanned within the warp (multiplier a^{16 o} at offset o)
        float2 B = zl;
        if (rscan) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float2 pb = shfl_up<float2>(B, o);
                if (lane >= o) B = cadd(cmul(apw[o], pb), B);
            }
            if (lane == 31) wtot[w] = B;
        }
        // W > 0 somewhere (exp of the table is positive above its threshold) or rho starting
        // above 0: otherwise every Heun / gas step adds exactly 0 and the density stays 0
        const bool ion = __syncthreads_or(anyw ? 1 : 0) != 0 || a.k.rho0 != 0.f;
        if (s == 0 && w == 0) {   // max |A|^2 of the row (the warps' maxima are in wmx since stage 0's input)
            float m = wmx[lane];
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) atomic_max_nonneg(f.max_out, (double)m);
        }
        float2 zs = make_float2(0.f, 0.f), zN = zs;
        if (rscan) {   // warp totals scanned by warp 0 (multiplier a^{512 o}); chunk starts
            if (w == 0) {
                float2 X = wtot[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const float2 px = shfl_up<float2>(X, o);
                    if (lane >= o) X = cadd(cmul(apw[32 * o], px), X);
                }
                wpre[lane] = X;
            }
            __syncthreads();
            const float2 Bx = shfl_up<float2>(B, 1);
            zs = (w > 0) ? cmul(apw[lane], wpre[w - 1]) : make_float2(0.f, 0.f);
            if (lane > 0) zs = cadd(zs, Bx);
            zN = wpre[31];
        }
        if (t == 0 && a.row_ion) a.row_ion[row] = ion ? 1 : 0;

        // ---- carrier density by multiple shooting (Newton on the chunk starts); rows that do
        // not ionize keep rho = 0 and skip it.  Newton on a forward recurrence is exact after
        // chunks + 1 iterations (each makes one more chunk start the sequential one), so the
        // loop is bounded by that; typical rows stop after a few
        auto g_of = [&](int tt) -> float {
            if (tt == 0) return 0.f;
            const float2 e = E[pad16(tt)];
            const float I = e.x * e.x + e.y * e.y;
            return __fdividef(AV, U + Pc * I) * I;
        };
        auto run_chunk = [&](float st0, float* dout) -> float {
            float ro = st0, d = 1.f;
            if (gas) {   // ionization.cpp:45-60, one level
                float W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : -1.f;
#pragma unroll 4
                for (int i = 0; i < L; i++) {
                    const float W1 = Wc[i];
                    if (t0 + i > 0) ro = gas_step<float>(ro, W0, W1, tstep, ND, &d);
                    W0 = W1;
                }
                *dout = d;
                return ro;
            }
            float W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : 0.f, g0 = (t0 > 0) ? g_of(t0 - 1) : 0.f;
#pragma unroll 4
            for (int i = 0; i < L; i++) {
                const float W1 = Wc[i];
                const float2 e = Ec[i];
                const float I = e.x * e.x + e.y * e.y;
                const float g1 = (t0 + i == 0) ? 0.f : __fdividef(AV, U + Pc * I) * I;
                if (t0 + i > 0) ro = heun_step<float>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
                W0 = W1;
                g0 = g1;
            }
            *dout = d;
            return ro;
        };
        if (ion) {
            s_start[t] = (t == 0) ? a.k.rho0 : 0.f;
            if (t == 0) *flag = 0;
            __syncthreads();
            const float tol = 1e-5f;
            for (int it = 0; it < NT + 1; it++) {
                const float st0 = s_start[t];
                float D;
                const float e = run_chunk(st0, &D);
                float Am = D, Bm = e - D * st0;
                block_affine_scan<float>(Am, Bm, 1.f, 0.f, rA, rB);
                const float next = Am * s_start[0] + Bm;   // start of chunk t + 1
                float change = 0.f, mag = 0.f;
                __syncthreads();
                if (t + 1 < NT) {
                    change = fabsf(next - s_start[t + 1]);
                    mag = fabsf(next);
                    s_start[t + 1] = next;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    change = fmaxf(change, __shfl_xor_sync(0xffffffffu, change, o));
                    mag = fmaxf(mag, __shfl_xor_sync(0xffffffffu, mag, o));
                }
                if (lane == 0) { rA[w] = change; rB[w] = mag; }
                __syncthreads();
                if (t == 0) {
                    float cm = 0.f, mm = 0.f;
                    for (int k = 0; k < NT / 32; k++) { cm = fmaxf(cm, rA[k]); mm = fmaxf(mm, rB[k]); }
                    *flag = (cm <= tol * mm && !a.shoot_exhaust) ? 1 : 0;
                }
                __syncthreads();
                if (*flag) break;
                __syncthreads();
            }
        }

        // ---- final pass: density, Raman factor Q, the sources Q E (over E), loss and rho E
        {
            float2 v = make_float2(0.f, 0.f);   // (1 - a^N) z_{t-1} + a^t z_{N-1}
            if (rscan) v = cadd(cmul(oma, zs), cmul(apw[t], zN));
            if (!ion && !gas && !a.th) {   // the common row: the Kerr source only
#pragma unroll 4
                for (int i = 0; i < L; i++) {
                    const float2 e = Ec[i];
                    const float I = e.x * e.x + e.y * e.y;
                    float Q = I;
                    if (rscan) {
                        v = cmul(ra, v);
                        v.x += oma.x * I;
                        v.y += oma.y * I;
                        Q = omf * I + fRM * v.y;
                    }
                    Ec[i] = make_float2(Q * e.x, Q * e.y);
                }
            } else {
                float ro = ion ? s_start[t] : 0.f, d = 1.f;
                float W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : 0.f, g0 = (t0 > 0) ? g_of(t0 - 1) : 0.f;
                if (gas && t0 == 0) W0 = -1.f;
                __syncthreads();   // every chunk has read its left neighbour's last sample
#pragma unroll 2
                for (int i = 0; i < L; i++) {
                    const int tt = t0 + i;
                    const float2 e = Ec[i];
                    const float I = e.x * e.x + e.y * e.y;
                    const float W1 = Wc[i];
                    float2 loss = make_float2(0.f, 0.f);
                    if (!ion) {
                        // the density stays 0 and there is no loss
                    } else if (gas) {
                        if (tt > 0) ro = gas_step<float>(ro, W0, W1, tstep, ND, &d);
                        W0 = W1;
                        if (tt < N - 1 && W1 >= 0.f) {   // loss = tl E (ionization.cpp:60-81)
                            const float sl = gas_loss_factor<float>(W1, ro, I, tstep, ND, U, Pc);
                            loss = make_float2(sl * e.x, sl * e.y);
                        }
                    } else {
                        const float g1 = (tt == 0) ? 0.f : __fdividef(AV, U + Pc * I) * I;
                        if (tt > 0) ro = heun_step<float>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
                        W0 = W1;
                        g0 = g1;
                        // loss (ionization.cpp:43): W at (E_t, rho_t), the reference's log-threshold test
                        if (tt > 0 && tt < N - 1 && I > (float)GS_ION_MIN_LN) {
                            const float W01 = (ro > ND) ? 0.f : W1;
                            const float sl = __fdividef(-0.5f * W01 * (U + Pc * I), I);
                            loss = make_float2(sl * e.x, sl * e.y);
                        }
                    }
                    float Q = I;
                    if (rscan) {
                        v = cmul(ra, v);
                        v.x += oma.x * I;
                        v.y += oma.y * I;
                        Q = omf * I + fRM * v.y;
                    }
                    float2 src3 = make_float2(Q * e.x, Q * e.y);
                    if (a.th) {   // third harmonic (propagator.cu:712-720): + th_t E^3
                        const float2 h = cmul(a.th[tt], cmul(cmul(e, e), e));
                        src3.x += h.x;
                        src3.y += h.y;
                    }
                    if (ion) {   // chunk-interleaved (sample 16 t + i at i NT + t): coalesced
                        const size_t q = base + (size_t)i * NT + t;
                        a.u1[q] = loss;
                        a.u2[q] = make_float2(ro * e.x, ro * e.y);
                    }
                    Ec[i] = src3;
                }
            }
        }
        __syncthreads();   // the Kerr source is complete in E

        // ---- spectra of the sources: j = 0 Q E (Kerr), 1 loss, 2 rho E (rows that ionize).
        // All but the last go through their radix-4 pass to U3 / U1 at the thread's own slots
        // (4 positions as two 16-byte words per group, coalesced across the warp); the last
        // stays in E for the combination
        const int lastj = ion ? 2 : (kerr ? 0 : -1);
#pragma unroll 1
        for (int j = 0; j < 3; j++) {
            if (!(j == 0 ? kerr : ion)) continue;
            if (j > 0) {   // the source's samples (written by this thread, chunk-interleaved)
                const float2* src = (j == 1 ? sp.u1 : sp.u2) + base;
                float2 y[L];
#pragma unroll
                for (int i = 0; i < L; i++) y[i] = src[(size_t)i * NT + t];
#pragma unroll
                for (int i = 0; i < L; i++) Ec[i] = y[i];
                __syncthreads();
            }
            forward_head(E, twb, t, tw2, tw1);
            if (j != lastj) {
                float4* keep = reinterpret_cast<float4*>((j == 0 ? sp.u3 : sp.u1) + base);
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    float2 x[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) x[i] = Ec[4 * g + i];
                    radix4<-1>(x);
                    keep[2 * (g * NT + t)] = make_float4(x[0].x, x[0].y, x[1].x, x[1].y);
                    keep[2 * (g * NT + t) + 1] = make_float4(x[2].x, x[2].y, x[3].x, x[3].y);
                }
            }
        }

        // ---- N = FFT(loss) + PLASMA_FUNC FFT(rho E) - j KERR_PROFILE FFT(Q E) on the thread's
        // positions, 4 at a time (the last source's radix-4 pass first); stages 0-2 add k to
        // the RK4 sum and leave the next stage's input, through its radix-4 pass, in E; stage 3
        // writes (k1 + 2 k2 + 2 k3 + k4) / 6, accumulated in that order (propagator.cu:412)
        const float cnext = (s < 2) ? c_half : c_full;
        float4 kq[4];   // KERR_PROFILE at the thread's positions, its reads issued first
#pragma unroll
        for (int g = 0; g < 4; g++)
            kq[g] = kerr ? __ldg(reinterpret_cast<const float4*>(sp.kerr + t0) + g) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const int p0 = t0 + 4 * g;
            float2 v[4];
            if (lastj >= 0) {
#pragma unroll
                for (int i = 0; i < 4; i++) v[i] = Ec[4 * g + i];
                radix4<-1>(v);
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) v[i] = make_float2(0.f, 0.f);
            }
            const float kc[4] = {-kq[g].x, -kq[g].y, -kq[g].z, -kq[g].w};
            float2 k[4], qs[4];
            if (ion) {
                const float4* u1q = reinterpret_cast<const float4*>(sp.u1 + base) + 2 * (g * NT + t);
                const float4* pfq = reinterpret_cast<const float4*>(sp.pf + p0);
                const float4 a0 = u1q[0], a1 = u1q[1], f0 = __ldg(pfq), f1 = __ldg(pfq + 1);
                float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
                if (kerr) {
                    const float4* u3q = reinterpret_cast<const float4*>(sp.u3 + base) + 2 * (g * NT + t);
                    q0 = u3q[0];
                    q1 = u3q[1];
                }
                const float2 ac[4] = {make_float2(a0.x, a0.y), make_float2(a0.z, a0.w), make_float2(a1.x, a1.y),
                                      make_float2(a1.z, a1.w)};
                const float2 pf[4] = {make_float2(f0.x, f0.y), make_float2(f0.z, f0.w), make_float2(f1.x, f1.y),
                                      make_float2(f1.z, f1.w)};
                qs[0] = make_float2(q0.x, q0.y);
                qs[1] = make_float2(q0.z, q0.w);
                qs[2] = make_float2(q1.x, q1.y);
                qs[3] = make_float2(q1.z, q1.w);
#pragma unroll
                for (int i = 0; i < 4; i++) k[i] = cadd(ac[i], cmul(v[i], pf[i]));   // FFT(loss) + FFT(rho E) PF
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    k[i] = make_float2(0.f, 0.f);
                    qs[i] = v[i];
                }
            }
            if (kerr) {   // += -j KERR_PROFILE FFT(Q E)
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    k[i].x += -kc[i] * qs[i].y;
                    k[i].y += kc[i] * qs[i].x;
                }
            }
            float sum[8];
            if (s < 3) {
                float av[8];
                tld8(tm + 32 + 8 * g, av);
                if (s > 0) {
                    tld8(tm + 8 * g, sum);
                    tld_wait2(sum, av);
                } else {
                    tld_wait(av);
                }
                float tv[8];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    tv[2 * i] = k[i].x;
                    tv[2 * i + 1] = k[i].y;
                }
                if (s > 0) {   // k1, then + 2 k2, + 2 k3 in that order (2 tv exact: one rounding)
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float2 r = __ffma2_rn(make_float2(2.0f, 2.0f), make_float2(tv[2 * i], tv[2 * i + 1]),
                                                    make_float2(sum[2 * i], sum[2 * i + 1]));
                        tv[2 * i] = r.x;
                        tv[2 * i + 1] = r.y;
                    }
                }
                tst8(tm + 8 * g, tv);
                float2 x[4];   // the next stage's input (A + c dz k) / N, as a stage load forms it
#pragma unroll
                for (int i = 0; i < 4; i++)
                    x[i] = __fmul2_rn(__ffma2_rn(make_float2(cnext, cnext), k[i], make_float2(av[2 * i], av[2 * i + 1])),
                                      make_float2(sc, sc));
                radix4<+1>(x);
#pragma unroll
                for (int i = 0; i < 4; i++) Ec[4 * g + i] = x[i];
            } else {
                tld8(tm + 8 * g, sum);
                tld_wait(sum);
#pragma unroll
                for (int i = 0; i < 4; i++) {   // to E: the warp stores its 512 positions below
                    const float2 nb = make_float2((sum[2 * i] + k[i].x) / 6.0f, (sum[2 * i + 1] + k[i].y) / 6.0f);
                    nmax = fmaxf(nmax, nb.x * nb.x + nb.y * nb.y);
                    Ec[4 * g + i] = nb;
                }
            }
        }
        if (s < 3) tst_wait();
    }
    // ---- BIGBUFFER1 and (sp.nbc) its spectral-window positions compactly, the linear step's
    // input: each warp's 512 consecutive positions, two per lane per 16-byte store
    __syncwarp();
    {
        float* const nbr = sp.nbc ? sp.nbc + (size_t)row * sp.ncw : nullptr;
#pragma unroll 4
        for (int r = 0; r < 8; r++) {
            const int p = 512 * w + 64 * r + 2 * lane;
            const float2 y0 = E[pad16(p)], y1 = E[pad16(p) + 1];
            if (sp.nb) *reinterpret_cast<float4*>(sp.nb + base + p) = make_float4(y0.x, y0.y, y1.x, y1.y);
            if (nbr) {
                const int2 c2 = __ldg(reinterpret_cast<const int2*>(sp.cinv + p));
                if (c2.x >= 0 && in_bounds(c2.x + 2 <= sp.ncw, a.err)) *reinterpret_cast<float2*>(nbr + c2.x) = y0;
                if (c2.y >= 0 && in_bounds(c2.y + 2 <= sp.ncw, a.err)) *reinterpret_cast<float2*>(nbr + c2.y) = y1;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) nmax = fmaxf(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
    if (lane == 0) wmx[w] = nmax;

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (w == 0) {
        float m = wmx[lane];
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) atomic_max_nonneg(sp.max_out, (double)m);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tslot), "r"(512));
    }
}

}  // namespace r16k

bool nl_row16k_applies(int N, int threads) { return N == r16k::N && (threads == 0 || threads == r16k::NT); }

cudaError_t nl_row16k_setup() {
    return cudaFuncSetAttribute(r16k::nl_row16k_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, r16k::SMEM);
}

cudaError_t launch_nl_row16k(FftArgs<float> f, PlasmaArgs<float> a, const float2* A, SpecArgs<float> s, int rows,
                             int ahead, cudaStream_t st, long long* nl) {
    if (f.N != r16k::N || !f.twb || !f.tw || a.tape_e || (s.ac && !s.cinv) || (s.nbc && !s.cinv) || (!s.nb && !s.nbc))
        return cudaErrorInvalidValue;
    f.rows = rows;
    f.ahead = ahead;
    r16k::nl_row16k_kernel<<<rows, r16k::NT, r16k::SMEM, st>>>(f, a, A, s);
    (*nl)++;
    return cudaGetLastError();
}

int nl_row16k_resident(int* out) {
    int per = 0, dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, r16k::nl_row16k_kernel, r16k::NT, r16k::SMEM);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *out = per * sms;
    return (int)e;
}
}  // namespace gs
