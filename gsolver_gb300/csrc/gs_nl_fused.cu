// gs_nl_fused.cu -- one RK4 stage of calculate_NLstep in one kernel, one CTA per row, for rows
// that fit one CTA's shared memory (N_t <= 16384 complex float / 8192 complex double).
//
//   nl_stage_kernel  first half: stage input X = A + c dz k_prev, E = IFFT(X)/N_t (shared
//                    memory), then with E resident: photoionization rates, the Heun
//                    carrier-density recurrence by multiple shooting (ionization.cpp:9-95), the
//                    Raman response as an exact one-pole recurrence (solver_main.cpp:401-413,
//                    propagator.cu:697-705), and the sources loss(t), rho(t) E(t), Q(t) E(t);
//                    second half: N = FFT(loss) + PLASMA_FUNC FFT(rho E) - j KERR_PROFILE
//                    FFT(Q E) (propagator.cu:679-710) and the RK4 accumulation of
//                    calculate_NLstep (propagator.cu:386-421) with max |N|^2.
// The Kerr source replaces E in shared memory and is transformed there; the loss and plasma
// sources exist only on rows that ionize, which store them and read them back.  Per stage a
// row without ionization reads A, k_prev and the RK4 sum and writes k and the RK4 sum.
#include <type_traits>

#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_plasma.cuh"

namespace gs {


template <typename Rl> struct FrontSmem {
    static __host__ __device__ size_t bytes(int N, int nthr) {
        using T2 = typename Vec2<Rl>::T;
        return (size_t)padded_len(N) * sizeof(T2)       // E row
               + (size_t)(N / 64 + 64) * sizeof(T2)     // twiddle tables
               + (size_t)wb_count(N) * sizeof(Rl)       // photoionization rates W_t
               + (size_t)nthr * sizeof(Rl)              // chunk starts of the density
               + (size_t)nthr * sizeof(T2)              // chunk ends of the Raman sum
               + 64 * sizeof(T2) + 64 * sizeof(Rl) + 64;   // scan scratch, flags
    }
};

// a / b in the rows' precision: FP32 takes the fast reciprocal-based quotient (within 2 ulp;
// the denominators here, U + P I and I above the rate threshold, are normal numbers)
template <typename Rl> __device__ __forceinline__ Rl qdiv(Rl a, Rl b) { return a / b; }
template <> __device__ __forceinline__ float qdiv<float>(float a, float b) { return __fdividef(a, b); }

// the per-stage values of one RK4 stage of a row (the rest comes from the launch's arguments)
template <typename Rl> struct StageOv {
    Rl cdz;
    const typename Vec2<Rl>::T* kp;
    int track_max, ahead, stage;
    typename Vec2<Rl>::T* tape_e;
    Rl *tape_rho, *tape_q;
    int* row_ion;
    Rl next_cdz;     // != 0: this stage also leaves the next stage's input (A + next_cdz k) / N in E
    int preloaded;   // E holds this stage's input already
};

// LOGN > 0: rows of exactly 2^LOGN points (the row FFT with compile-time sizes and nothing
// else inlined); LOGN = 0: any fused row length.  LC = 16: launched with N/16 threads, so each
// thread's chunk is 16 consecutive samples starting at a multiple of 16 and its shared-memory
// slots are at constant offsets (pad16(t0 + i) = pad16(t0) + i, pad32(t0 + i) = pad32(t0) + i).
template <typename Rl, int LOGN, int LC>
__device__ __forceinline__ void nl_stage_row(const FftArgs<Rl>& f, const PlasmaArgs<Rl>& a,
                                             const typename Vec2<Rl>::T* __restrict__ A, const SpecArgs<Rl>& sp,
                                             const StageOv<Rl>& ov) {
    using T2 = C2<Rl>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = LOGN > 0 ? (1 << LOGN) : f.N;
    const int tid = threadIdx.x, nthr = blockDim.x;
    T2* E = reinterpret_cast<T2*>(smem_raw);
    T2* twh = E + padded_len(N);
    T2* twl = twh + N / 64;
    Rl* Wb = reinterpret_cast<Rl*>(twl + 64);
    Rl* s_start = Wb + wb_count(N);
    T2* cend = reinterpret_cast<T2*>(s_start + nthr);
    T2* scA = cend + nthr;
    T2* scB = scA + 32;
    Rl* rA = reinterpret_cast<Rl*>(scB + 32);
    Rl* rB = rA + 32;
    int* flag = reinterpret_cast<int*>(rB + 32);
    T2* cend_aL = reinterpret_cast<T2*>(reinterpret_cast<unsigned char*>(flag) + 16);   // a^L (flag area is 64 B)
    const size_t base = (size_t)blockIdx.x * N;

    // ---- stage input and inverse FFT (propagator.cu:386-396, 640-641)
    load_twiddles<Rl>(twh, twl, f.tw, N, tid, nthr);
    // N / nthr = 16 elements per thread (2 when N < 512): loads issued together
    Rl lmax = 0;
    const Rl cdz = (Rl)ov.cdz;
    const int per = N / nthr;
    // rows of 2^k points take the 1/N of the inverse transform on the input: scaling by a power
    // of two is exact and commutes with every rounding of the FFT, so IFFT(X/N) = IFFT(X)/N
    const bool pow2 = (N & (N - 1)) == 0;
    const Rl sc = pow2 ? (Rl)1 / (Rl)N : (Rl)1;
    if (ov.preloaded) {
        // the previous stage of this CTA left (A + c dz k) / N in E (four stages per launch)
    } else if (per == 16) {
        T2 v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = A[base + tid + u * nthr];
        if (ov.track_max) {
#pragma unroll
            for (int u = 0; u < 16; u++) lmax = fmax(lmax, v[u].x * v[u].x + v[u].y * v[u].y);
        }
        if (ov.cdz != 0) {
            T2 k[16];
#pragma unroll
            for (int u = 0; u < 16; u++) k[u] = ov.kp[base + tid + u * nthr];
#pragma unroll
            for (int u = 0; u < 16; u++) { v[u].x = v[u].x + cdz * k[u].x; v[u].y = v[u].y + cdz * k[u].y; }
        }
#pragma unroll
        for (int u = 0; u < 16; u++) E[pad16(tid + u * nthr)] = T2{v[u].x * sc, v[u].y * sc};
    } else {
        for (int i = tid; i < N; i += nthr) {
            T2 v = A[base + i];
            if (ov.track_max) lmax = fmax(lmax, v.x * v.x + v.y * v.y);
            if (ov.cdz != 0) {
                const T2 k = ov.kp[base + i];
                v.x = v.x + cdz * k.x;
                v.y = v.y + cdz * k.y;
            }
            E[pad16(i)] = T2{v.x * sc, v.y * sc};
        }
    }
    if (ov.track_max) {
        for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if ((tid & 31) == 0) atomic_max_nonneg(f.max_out, (double)lmax);
    }
    __syncthreads();
    // the row that takes this SM's next slot: its inputs travel to L2 while this row computes
    if (tid < 32 && ov.ahead > 0 && (int)blockIdx.x + ov.ahead < f.rows) {
        const size_t nbase = base + (size_t)ov.ahead * N;
        prefetch_row_l2(A + nbase, (size_t)N * sizeof(T2), tid);
        if (ov.cdz != 0) prefetch_row_l2(ov.kp + nbase, (size_t)N * sizeof(T2), tid - 4);
        if (ov.stage == 3) {
            prefetch_row_l2(sp.kst[0] + nbase, (size_t)N * sizeof(T2), tid - 8);
            prefetch_row_l2(sp.kst[1] + nbase, (size_t)N * sizeof(T2), tid - 12);
        }
    }
    const TwTab<Rl> tw{twh, twl, f.twb};
    if constexpr (LOGN > 0) smem_fft_ct<+1, Rl, LOGN>(E, tw, 1, tid, nthr);
    else smem_fft<+1, Rl>(E, N, f.logM, tw, 1, tid, nthr);
    const Rl rn = (Rl)N;
    const Rl ND = a.k.ND, tstep = a.k.tstep, U = a.k.U, Pc = a.k.Pc, AV = a.k.AV;
    const Rl invND = a.k.invND, invTAU = a.k.invTAU;
    auto g_of = [&](int t) -> Rl {
        if (t == 0) return (Rl)0;
        const T2 e = E[pad16(t)];
        const Rl I = e.x * e.x + e.y * e.y;
        return qdiv<Rl>(AV, U + Pc * I) * I;
    };
    const int L = LC > 0 ? LC : N / nthr;   // chunk of consecutive samples per thread
    const int c = tid;
    const int t0 = c * L;
    // shared-memory slots of sample t0 + i of this chunk
    const T2* Ec = E + pad16(t0);
    const Rl* Wc = Wb + pad32(t0);
    auto e_at = [&](int i) -> T2 { return LC == 16 ? Ec[i] : E[pad16(t0 + i)]; };
    auto w_at = [&](int i) -> Rl { return LC == 16 ? Wc[i] : Wb[pad32(t0 + i)]; };
    // ---- one pass over this thread's chunk: E /= N (rows whose length is not a power of two),
    // the rates W_t (the first sample is treated as E_0 = 0: W_0 = g_0 = 0) and the Raman
    // chunk sum z_t = a z_{t-1} + I_t.  Samples go in groups of 8; a warp computes rates only
    // when one of its samples is at or above the table threshold (or NaN, which the rate
    // function reports), and then issues the group's table reads together.
    const bool gas = a.gas != 0;
    const bool rscan = a.raman_scan != 0;
    const T2 ra = T2{a.k.a_re, a.k.a_im};
    bool anyw = false;   // some sample of this thread is above the rate table's threshold
    T2 zl = T2{0, 0}, aL = T2{1, 0};
    for (int g = 0; g < L; g += 8) {
        Rl Iv[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            Iv[u] = 0;
            if (g + u >= L) continue;   // chunks of 2 or 4 samples (short rows)
            T2 e = e_at(g + u);
            if (!pow2) {
                e.x = e.x / rn;
                e.y = e.y / rn;
                if (LC == 16) E[pad16(t0) + g + u] = e;
                else E[pad16(t0 + g + u)] = e;
            }
            Iv[u] = e.x * e.x + e.y * e.y;
            if (rscan) {
                zl = cmul(ra, zl);
                zl.x += Iv[u];
                aL = cmul(aL, ra);
            }
        }
        bool above = false;
#pragma unroll
        for (int u = 0; u < 8; u++) above = above || (g + u < L && t0 + g + u > 0 && !(Iv[u] < (Rl)(1e13 / 1e16)));
        Rl W[8];
        if (__any_sync(0xffffffffu, above)) {
            int n[8];
            Rl dl[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                dl[u] = 0;
                n[u] = (g + u < L && t0 + g + u > 0) ? photo_index<Rl>(Iv[u], &dl[u], a.err) : -1;
                if (n[u] >= 0 && !in_bounds(n[u] + 1 < 8192, a.err)) n[u] = -1;
            }
            Rl w0[8], w1[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                w0[u] = n[u] >= 0 ? __ldg(&a.rate[n[u]]) : (Rl)0;
                w1[u] = n[u] >= 0 ? __ldg(&a.rate[n[u] + 1]) : (Rl)0;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                W[u] = n[u] >= 0 ? photo_rate_from<Rl>(w0[u], w1[u], dl[u]) : (Rl)0;
                anyw = anyw || n[u] >= 0;
            }
        } else {
#pragma unroll
            for (int u = 0; u < 8; u++) W[u] = 0;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int t = t0 + g + u;
            if (g + u >= L) continue;
            const Rl w = gas ? gas_rate_slot<Rl>(t, Iv[u], W[u]) : W[u];
            if (LC == 16) Wb[pad32(t0) + g + u] = w;
            else Wb[pad32(t)] = w;
        }
    }
    // W > 0 somewhere (exp of the table is positive above its threshold) or rho starting above
    // 0: otherwise every Heun / gas step adds exactly 0 and the density stays 0 along the row
    const bool ion = __syncthreads_or(anyw ? 1 : 0) != 0 || a.k.rho0 != (Rl)0;
    // Raman: an exclusive scan of the chunk sums gives each chunk's start
    T2 zs = T2{0, 0}, zN = T2{0, 0};
    if (rscan) {
        if (c == 0) cend_aL[0] = aL;                   // a^L, common to all chunks
        T2 Am = aL, Bm = zl;
        block_affine_scan<T2>(Am, Bm, T2{1, 0}, T2{0, 0}, scA, scB);
        cend[c] = Bm;                                   // z at the end of chunk c
        __syncthreads();
        zs = (c == 0) ? T2{0, 0} : cend[c - 1];
        zN = cend[nthr - 1];
    }
    if (tid == 0 && ov.row_ion) ov.row_ion[blockIdx.x] = ion ? 1 : 0;

    // the exact recurrence over this thread's chunk from start value s (rho_{t0-1})
    auto run_chunk = [&](Rl s, Rl* dout) -> Rl {
        Rl ro = s, d = (Rl)1;
        if (gas) {   // ionization.cpp:45-60, one level
            Rl W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : (Rl)-1;
#pragma unroll 4
            for (int i = 0; i < L; i++) {
                const int t = t0 + i;
                const Rl W1 = w_at(i);
                if (t > 0) ro = gas_step<Rl>(ro, W0, W1, tstep, ND, &d);
                W0 = W1;
            }
            *dout = d;
            return ro;
        }
        Rl W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : (Rl)0, g0 = (t0 > 0) ? g_of(t0 - 1) : (Rl)0;
#pragma unroll 4
        for (int i = 0; i < L; i++) {
            const int t = t0 + i;
            const Rl W1 = w_at(i);
            const T2 e = e_at(i);
            const Rl I = e.x * e.x + e.y * e.y;
            const Rl g1 = (t == 0) ? (Rl)0 : qdiv<Rl>(AV, U + Pc * I) * I;
            if (t > 0) ro = heun_step<Rl>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
            W0 = W1;
            g0 = g1;
        }
        *dout = d;
        return ro;
    };

    // ---- carrier density by multiple shooting (Newton on the chunk starts)
    s_start[c] = (c == 0) ? a.k.rho0 : (Rl)0;
    if (tid == 0) *flag = 0;
    __syncthreads();
    // relative change of the starts at which Newton stops (quadratic convergence: the
    // starts then carry ~tol^2 + rounding).  Newton on a forward recurrence also ends in finitely
    // many steps: after k iterations the starts of chunks 0..k are those of the sequential
    // recurrence (each computed from an exact predecessor), so nthr + 1 iterations give the
    // sequential result whatever the stopping test does; typical rows stop after a few
    const Rl tol = sizeof(Rl) == 8 ? (Rl)1e-13 : (Rl)1e-5;
    for (int it = 0; it < (ion ? nthr + 1 : 0); it++) {   // no ionization: the starts stay 0
        const Rl sc = s_start[c];
        Rl D;
        const Rl e = run_chunk(sc, &D);
        Rl Am = D, Bm = e - D * sc;
        block_affine_scan<Rl>(Am, Bm, (Rl)1, (Rl)0, rA, rB);
        const Rl next = Am * s_start[0] + Bm;          // start of chunk c + 1
        Rl change = 0, mag = 0;
        __syncthreads();
        if (c + 1 < nthr) {
            change = fabs(next - s_start[c + 1]);
            mag = fabs(next);
            s_start[c + 1] = next;
        }
        for (int o = 16; o > 0; o >>= 1) {
            change = fmax(change, __shfl_xor_sync(0xffffffffu, change, o));
            mag = fmax(mag, __shfl_xor_sync(0xffffffffu, mag, o));
        }
        if ((tid & 31) == 0) { rA[tid >> 5] = change; rB[tid >> 5] = mag; }
        __syncthreads();
        if (tid == 0) {
            Rl cm = 0, mm = 0;
            for (int w = 0; w < (nthr >> 5); w++) { cm = fmax(cm, rA[w]); mm = fmax(mm, rB[w]); }
            *flag = (cm <= tol * mm && !a.shoot_exhaust) ? 1 : 0;
        }
        __syncthreads();
        if (*flag) break;
        __syncthreads();
    }

    // ---- final pass: density, Raman Q and the three source rows
    {
        Rl ro = s_start[c], d = 1;
        Rl W0 = (t0 > 0) ? Wb[pad32(t0 - 1)] : (Rl)0, g0 = (t0 > 0) ? g_of(t0 - 1) : (Rl)0;
        __syncthreads();   // every chunk has read its left neighbour's last sample: E is rewritten below
        T2 z = zs;
        T2 pw = T2{0, 0};
        if (rscan) {
            // a^{t0+1} = a (a^L)^c by binary powering (no transcendental per thread)
            T2 b = cend_aL[0], pr = T2{1, 0};
            for (int e = c; e > 0; e >>= 1) {
                if (e & 1) pr = cmul(pr, b);
                b = cmul(b, b);
            }
            pw = cmul(pr, ra);
        }
        const T2 oma = T2{a.k.oma_re, a.k.oma_im};
        const Rl fRM = a.k.fRM, omf = a.k.omf;
        if (gas && t0 == 0) W0 = (Rl)-1;
        // the common row (no ionization, solid, Raman recurrence): the Kerr source only.  It
        // takes this loop whether or not the stage is recorded, so that a recorded step (the
        // adjoint's re-run of a checkpoint segment) repeats an unrecorded one bit for bit
        const bool plain = !ion && !gas && rscan && !a.th;
#pragma unroll 4
        for (int i = 0; i < (plain ? L : 0); i++) {
            const T2 e = e_at(i);
            const Rl I = e.x * e.x + e.y * e.y;
            z = cmul(ra, z);
            z.x += I;
            const T2 v = cadd(cmul(oma, z), cmul(pw, zN));
            const Rl Q = omf * I + fRM * v.y;
            pw = cmul(pw, ra);
            const T2 src3 = T2{Q * e.x, Q * e.y};
            if (LC == 16) E[pad16(t0) + i] = src3;
            else E[pad16(t0 + i)] = src3;
            if (ov.tape_e) {   // what the adjoint of this stage reads back (no density: no ionization)
                ov.tape_e[base + t0 + i] = e;
                ov.tape_q[base + t0 + i] = Q;
            }
        }
#pragma unroll 4
        for (int i = 0; i < (plain ? 0 : L); i++) {
            const int t = t0 + i;
            const T2 e = e_at(i);
            const Rl I = e.x * e.x + e.y * e.y;
            const Rl W1 = w_at(i);
            T2 loss = T2{0, 0};
            if (!ion) {
                // the density stays 0 and there is no loss
            } else if (gas) {
                if (t > 0) ro = gas_step<Rl>(ro, W0, W1, tstep, ND, &d);
                W0 = W1;
                // loss[t] = tl E_t (ionization.cpp:60-81), where sample t is above the threshold
                if (t < N - 1 && W1 >= 0) {
                    const Rl sl = gas_loss_factor<Rl>(W1, ro, I, tstep, ND, U, Pc);
                    loss = T2{sl * e.x, sl * e.y};
                }
            } else {
                const Rl g1 = (t == 0) ? (Rl)0 : qdiv<Rl>(AV, U + Pc * I) * I;
                if (t > 0) ro = heun_step<Rl>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
                W0 = W1;
                g0 = g1;
                // loss[t] (ionization.cpp:43): W at (E_t, rho_t), the reference's log-threshold test
                if (t > 0 && t < N - 1 && I > (Rl)GS_ION_MIN_LN) {
                    const Rl W01 = (ro > ND) ? (Rl)0 : W1;
                    const Rl sl = qdiv<Rl>(-(Rl)0.5 * W01 * (U + Pc * I), I);
                    loss = T2{sl * e.x, sl * e.y};
                }
            }
            Rl Q = I;   // Kerr without Raman: |E|^2 E
            if (rscan) {
                z = cmul(ra, z);
                z.x += I;
                const T2 v = cadd(cmul(oma, z), cmul(pw, zN));
                Q = omf * I + fRM * v.y;
                pw = cmul(pw, ra);
            }
            T2 src3 = T2{Q * e.x, Q * e.y};
            if (a.th) {   // third harmonic (propagator.cu:712-720): + th_t E^3, same KERR profile
                const T2 e2 = cmul(e, e);
                const T2 h = cmul(a.th[t], cmul(e2, e));
                src3.x += h.x;
                src3.y += h.y;
            }
            // loss and plasma source rows in chunk-interleaved order (sample c L + i at i nthr + c):
            // the warp's stores are coalesced, and the order is undone when they are staged below;
            // rows without ionization have neither.  The Kerr source takes E's place.
            if (ion) {
                const size_t q = base + (size_t)i * nthr + c;
                a.u1[q] = loss;
                a.u2[q] = T2{ro * e.x, ro * e.y};
            }
            if (LC == 16) E[pad16(t0) + i] = src3;
            else E[pad16(t)] = src3;
            if (ov.tape_e) {   // what the adjoint of this stage reads back (rho only where it ionizes)
                ov.tape_e[base + t] = e;
                if (ion) ov.tape_rho[base + t] = ro;
                ov.tape_q[base + t] = Q;
            }
        }
    }

    // ---- second half: the spectra of the sources, their combination and the RK4 sums
    __syncthreads();   // the Kerr source is complete in E
    const bool kerr = sp.kerr_on != 0;
    auto fwd = [&]() {
        if constexpr (LOGN > 0) smem_fft_ct<-1, Rl, LOGN>(E, tw, 1, tid, nthr);
        else smem_fft<-1, Rl>(E, N, f.logM, tw, 1, tid, nthr);
    };
    auto stage_row = [&](const T2* in) {   // a source row in chunk-interleaved order into E
        if (L == 16) {
            T2 v[16];
#pragma unroll
            for (int u = 0; u < 16; u++) v[u] = in[base + tid + u * nthr];
#pragma unroll
            for (int u = 0; u < 16; u++) E[pad16(tid * 16 + u)] = v[u];
        } else {
            for (int q = tid; q < N; q += nthr) E[pad16((q % nthr) * L + q / nthr)] = in[base + q];
        }
        __syncthreads();
    };
    // source j = 0: Q E (in E already), 1: loss, 2: rho E (rows that ionize only).  On those
    // rows FFT(Q E) waits in U3 and FFT(loss) in U1 (staged already) while the next source
    // uses the row; the last spectrum stays in E for the combination
    for (int j = 0; j < 3; j++) {
        if (!(j == 0 ? kerr : ion)) continue;
        if (j > 0) stage_row(j == 1 ? sp.u1 : sp.u2);
        fwd();
        if (ion && j < 2) {
            T2* keep = (j == 0) ? sp.u3 : sp.u1;
            for (int p = tid; p < N; p += nthr) keep[base + p] = E[pad16(p)];
            __syncthreads();
        }
    }
    // N = FFT(loss) + PLASMA_FUNC FFT(rho E) - j KERR_PROFILE FFT(Q E).  Stages 0..2 write
    // their k; stage 3 forms (k1 + 2 k2 + 2 k3 + k4) / 6, accumulated in that order
    // (propagator.cu:412).  Batches of SB points per thread: every global read of a batch is
    // issued before use.
    Rl nmax = 0;
    T2* const kout = ov.stage == 0 ? sp.kst[0] : (ov.stage == 1 ? sp.kst[1] : sp.kst[2]);
    auto combine = [&](auto ion_c, auto last_c) {
        constexpr bool ION = decltype(ion_c)::value;
        constexpr bool last = decltype(last_c)::value;
        constexpr int SB = ION ? 2 : 4;
        for (int pb = tid; pb < N; pb += SB * nthr) {
            T2 v[SB], ac[SB], pf[SB], q[SB], k1[SB], k2[SB], k3[SB], an[SB];
            Rl kc[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int p = pb + u * nthr;
                const bool in = p < N;
                v[u] = (in && (ION || kerr)) ? E[pad16(p)] : T2{0, 0};
                if constexpr (ION) {
                    ac[u] = in ? sp.u1[base + p] : T2{0, 0};
                    pf[u] = in ? sp.pf[p] : T2{0, 0};
                    q[u] = (in && kerr) ? sp.u3[base + p] : T2{0, 0};
                }
                kc[u] = (in && kerr) ? -sp.kerr[p] : (Rl)0;
                if constexpr (last) {
                    k1[u] = in ? sp.kst[0][base + p] : T2{0, 0};
                    k2[u] = in ? sp.kst[1][base + p] : T2{0, 0};
                    k3[u] = in ? sp.kst[2][base + p] : T2{0, 0};
                } else {
                    an[u] = (in && ov.next_cdz != 0) ? A[base + p] : T2{0, 0};
                }
            }
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int p = pb + u * nthr;
                if (p >= N) continue;
                T2 k = T2{0, 0};
                T2 qs = v[u];
                if constexpr (ION) {
                    k = cadd(ac[u], cmul(v[u], pf[u]));   // FFT(loss) + FFT(rho E) PLASMA_FUNC
                    qs = q[u];
                }
                if (kerr) {                                 // += -j KERR_PROFILE FFT(Q E)
                    k.x += -kc[u] * qs.y;
                    k.y += kc[u] * qs.x;
                }
                if constexpr (!last) {
                    kout[base + p] = k;
                    if (ov.next_cdz != 0) {   // the next stage's input, as its load would form it
                        const Rl nc = ov.next_cdz;
                        T2 x = an[u];
                        x.x = x.x + nc * k.x;
                        x.y = x.y + nc * k.y;
                        E[pad16(p)] = T2{x.x * sc, x.y * sc};
                    }
                    continue;
                }
                T2 s = k1[u];
                s = T2{s.x + (Rl)2 * k2[u].x, s.y + (Rl)2 * k2[u].y};
                s = T2{s.x + (Rl)2 * k3[u].x, s.y + (Rl)2 * k3[u].y};
                const T2 nb = T2{(s.x + k.x) / (Rl)6, (s.y + k.y) / (Rl)6};
                nmax = fmax(nmax, nb.x * nb.x + nb.y * nb.y);
                sp.nb[base + p] = nb;
                if constexpr (sizeof(Rl) == 4) {
                    if (sp.nbc) {
                        const int c = __ldg(sp.cinv + p);
                        if (c >= 0 && in_bounds(c + 2 <= sp.ncw, a.err))
                            *reinterpret_cast<float2*>(sp.nbc + (size_t)blockIdx.x * sp.ncw + c) = make_float2(nb.x, nb.y);
                    }
                }
            }
        }
    };
    if (ov.stage == 3) {
        if (ion) combine(std::true_type{}, std::true_type{});
        else combine(std::false_type{}, std::true_type{});
    } else {
        if (ion) combine(std::true_type{}, std::false_type{});
        else combine(std::false_type{}, std::false_type{});
    }
    if (ov.stage == 3) {
        for (int o = 16; o > 0; o >>= 1) nmax = fmax(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
        if ((tid & 31) == 0) atomic_max_nonneg(sp.max_out, (double)nmax);
    }
}

// One RK4 stage (sp.stage) of every row.
template <typename Rl, int LOGN = 0, int LC = 0>
__global__ void __launch_bounds__(sizeof(Rl) == 8 ? 512 : 1024) nl_stage_kernel(FftArgs<Rl> f, PlasmaArgs<Rl> a,
                                                                              const typename Vec2<Rl>::T* __restrict__ A,
                                                                              SpecArgs<Rl> sp) {
    if (f.halt && *f.halt) return;   // gs_advance: the z-loop stopped
    Rl cdz = f.cdz;
    if (f.dz_dev) {   // gs_advance: c dz of this stage from the attempt's step size, as the host rounds it
        const double d = *f.dz_dev;
        cdz = (Rl)((sp.stage == 0) ? 0.0 : (sp.stage < 3 ? d * 0.5 : d));
    }
    const StageOv<Rl> ov{cdz, f.kp, f.track_max, f.ahead, sp.stage, a.tape_e, a.tape_rho, a.tape_q, a.row_ion,
                         (Rl)0, 0};
    nl_stage_row<Rl, LOGN, LC>(f, a, A, sp, ov);
}

// All four RK4 stages of every row in turn (step size f.dzs): stage s reads A and the k of
// stage s - 1 that the same CTA has just written (L2-resident), so between steps a row's state
// crosses HBM once.  A separate kernel, so that each keeps one inlined copy of the row body.
// (Rows of 16384 FP32 points at 1024 threads without a stage record take nl_row16k_kernel,
// gs_nl_row16k.cu, instead.)
template <typename Rl, int LOGN = 0, int LC = 0>
__global__ void __launch_bounds__(sizeof(Rl) == 8 ? 512 : 1024) nl_stage4_kernel(FftArgs<Rl> f, PlasmaArgs<Rl> a,
                                                                               const typename Vec2<Rl>::T* __restrict__ A,
                                                                               SpecArgs<Rl> sp) {
    if (f.halt && *f.halt) return;   // gs_advance: the z-loop stopped
    const double dzs = f.dz_dev ? *f.dz_dev : f.dzs;   // gs_advance: the attempt's step size
    for (int s = 0; s < 4; s++) {
        StageOv<Rl> ov{(Rl)(s == 0 ? 0.0 : (s < 3 ? dzs * 0.5 : dzs)),   // as the per-stage launches round it
                       s > 0 ? sp.kst[s - 1] : f.kp, s == 0, s == 0 ? f.ahead : 0, s,
                       a.tape_e, a.tape_rho, a.tape_q, a.row_ion,
                       (Rl)(s < 3 ? (s + 1 < 3 ? dzs * 0.5 : dzs) : 0.0),   // stage s + 1's c dz
                       s > 0};
        if (a.tape_e) {   // stage s's record for the adjoint
            const size_t o = (size_t)s * a.tape_stride;
            ov.tape_e = reinterpret_cast<typename Vec2<Rl>::T*>(reinterpret_cast<char*>(a.tape_e) + o);
            ov.tape_rho = reinterpret_cast<Rl*>(reinterpret_cast<char*>(a.tape_rho) + o);
            ov.tape_q = reinterpret_cast<Rl*>(reinterpret_cast<char*>(a.tape_q) + o);
            ov.row_ion = reinterpret_cast<int*>(reinterpret_cast<char*>(a.row_ion) + o);
        }
        if (s > 0) __syncthreads();   // k of stage s - 1 written by every thread of the CTA
        nl_stage_row<Rl, LOGN, LC>(f, a, A, sp, ov);
    }
}

template <typename Rl> static int fused_threads(int N) {
    const int maxt = sizeof(Rl) == 8 ? 512 : 1024;
    int t = N / 16;
    if (t < 32) t = 32;
    if (t > maxt) t = maxt;
    return t;
}

template <typename Rl> bool nl_fused_supported(int N) {
    const int nthr = fused_threads<Rl>(N);
    return N % nthr == 0 && FrontSmem<Rl>::bytes(N, nthr) <= 227 * 1024;
}

template <typename Rl> bool nl_fused_threads_ok(int N, int t) {
    const int maxt = sizeof(Rl) == 8 ? 512 : 1024;
    return t >= 32 && t <= maxt && t % 32 == 0 && N % t == 0 && FrontSmem<Rl>::bytes(N, t) <= 227 * 1024;
}

template <typename Rl> bool nl_stage_reads_compact(int N, int threads) {
    const int nthr = threads > 0 ? threads : fused_threads<Rl>(N);
    return sizeof(Rl) == 4 && nl_row16k_applies(N, nthr);   // nl_row16k_kernel
}

template <typename Rl> int nl_fused_default_threads(int N) { return fused_threads<Rl>(N); }

template <typename Rl> cudaError_t nl_fused_setup(int N) {
    // the attribute is a per-kernel ceiling shared by every handle of the process: set the
    // device maximum so that a handle on a smaller grid never lowers it for a larger one
    (void)N;
    cudaError_t e = cudaFuncSetAttribute(nl_stage_kernel<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(nl_stage4_kernel<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if constexpr (sizeof(Rl) == 4) {   // the FP32 rows of 16384
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(nl_stage_kernel<Rl, 14, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(nl_stage_kernel<Rl, 14>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(nl_stage4_kernel<Rl, 14, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(nl_stage4_kernel<Rl, 14>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e == cudaSuccess) e = nl_row16k_setup();
    }
    return e;
}

// CTAs of a kernel resident on the device at once (the prefetch distance of the fused
// kernels); the last query per kernel is kept, since the shapes rarely change
template <typename K> static int resident_ctas(K kern, int nthr, size_t smem) {
    struct Last { const void* k; int nthr; size_t smem; int dev; int ctas; };
    static thread_local Last last{nullptr, 0, 0, -1, 0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (last.k == (const void*)kern && last.nthr == nthr && last.smem == smem && last.dev == dev) return last.ctas;
    int per = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, nthr, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    last = Last{(const void*)kern, nthr, smem, dev, per * sms};
    return last.ctas;
}

template <typename Rl>
bool nl_stage_all_preferred(int N, int threads, int rows) {
    const int nthr = threads > 0 ? threads : fused_threads<Rl>(N);
    const size_t sm = FrontSmem<Rl>::bytes(N, nthr);
    int res = 0;
    if constexpr (sizeof(Rl) == 4) {
        if (N == 16384 && nthr == 1024) res = resident_ctas(nl_stage_kernel<Rl, 14, 16>, nthr, sm);
        else if (N == 16384) res = resident_ctas(nl_stage_kernel<Rl, 14>, nthr, sm);
    }
    if (res == 0) res = resident_ctas(nl_stage_kernel<Rl>, nthr, sm);
    // a row's four stages in one CTA pay off when the grid has several waves: each CTA then
    // reads the k it just wrote from L2; with fewer rows the per-stage launches keep more
    // rows in flight
    return res > 0 && rows >= 4 * res;
}

template <typename Rl>
cudaError_t launch_nl_stage(FftArgs<Rl> f, PlasmaArgs<Rl> a, const typename Vec2<Rl>::T* A, SpecArgs<Rl> s, int rows,
                            cudaStream_t st, long long* nl) {
    const int nthr = f.threads > 0 ? f.threads : fused_threads<Rl>(f.N);
    const size_t sm = FrontSmem<Rl>::bytes(f.N, nthr);
    f.rows = rows;
    // the instantiation for the launch shape, one stage or all four
    auto go = [&](auto k1, auto k4) {
        if (f.all_stages) {
            f.ahead = resident_ctas(k4, nthr, sm);
            k4<<<rows, nthr, sm, st>>>(f, a, A, s);
        } else {
            f.ahead = resident_ctas(k1, nthr, sm);
            k1<<<rows, nthr, sm, st>>>(f, a, A, s);
        }
    };
    // a compact FIELD is read by nl_row16k_kernel only (its four-stage launch, no stage record)
    if (s.ac && !(f.all_stages && !a.tape_e && nl_stage_reads_compact<Rl>(f.N, nthr))) return cudaErrorInvalidValue;
    bool done = false;
    if constexpr (sizeof(Rl) == 4) {
        if (f.all_stages && !a.tape_e && nl_row16k_applies(f.N, nthr)) {   // gs_nl_row16k.cu
            static thread_local int ctas = -1;
            if (ctas < 0 && nl_row16k_resident(&ctas) != 0) {
                (void)cudaGetLastError();
                ctas = 0;
            }
            return launch_nl_row16k(f, a, A, s, rows, ctas, st, nl);
        } else if (f.N == 16384 && nthr == 1024) {
            go(nl_stage_kernel<Rl, 14, 16>, nl_stage4_kernel<Rl, 14, 16>);
            done = true;
        } else if (f.N == 16384) {
            go(nl_stage_kernel<Rl, 14>, nl_stage4_kernel<Rl, 14>);
            done = true;
        }
    }
    if (!done) go(nl_stage_kernel<Rl>, nl_stage4_kernel<Rl>);
    (*nl)++;
    return cudaGetLastError();
}

#define GS_FUSED_INST(Rl)                                                                                         \
    template bool nl_fused_supported<Rl>(int);                                                                    \
    template cudaError_t nl_fused_setup<Rl>(int);                                                                 \
    template cudaError_t launch_nl_stage<Rl>(FftArgs<Rl>, PlasmaArgs<Rl>, const typename Vec2<Rl>::T*, SpecArgs<Rl>, \
                                             int, cudaStream_t, long long*);                                      \
    template bool nl_stage_all_preferred<Rl>(int, int, int);                                                     \
    template bool nl_stage_reads_compact<Rl>(int, int);                                                          \
    template bool nl_fused_threads_ok<Rl>(int, int);                                                             \
    template int nl_fused_default_threads<Rl>(int);
GS_FUSED_INST(double)
GS_FUSED_INST(float)

}  // namespace gs
