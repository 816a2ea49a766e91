// gs_nl_pair.cu -- one RK4 stage of calculate_NLstep for rows too long for one CTA's shared
// memory (FP32 N_t = 32768, FP64 N_t = 16384): each row is split over two CTAs, one per half.
//
// These rows are stored in the handle's two-level position order (P = 2, H = N/2; the
// staged kernels' fft_cross_kernel + H-point rows, gs_nl.cu): position h*H + pos_H(k1)
// holds frequency h + 2 k1.  Forward: y_h[q] = w_N^{q h} (x[q] + (-1)^h x[q+H]), then the
// H-point FFT of y_h.  Inverse: z_h = IFFT_H of half h, then x[q] = z_0[q] + w_N^{-q} z_1[q],
// x[q+H] = z_0[q] - w_N^{-q} z_1[q].
//
//   nl_pair_front_kernel  a cluster of two CTAs per row.  CTA h loads the spectral half h
//                         of the stage input A + c dz k_prev and inverts it (H points); the
//                         pair completes the radix-2 step through distributed shared memory,
//                         so CTA h holds the time samples [h H, h H + H) of E = IFFT/N.  The
//                         carrier density (ionization.cpp:9-95) is solved by multiple
//                         shooting over both halves' chunks: each CTA scans its own chunks, and
//                         the seam value (the density entering CTA 1's first chunk) and the
//                         stopping test cross the pair every Newton iteration.  The Raman
//                         recurrence carries z across the seam the same way.  The source rows
//                         go out in chunk-interleaved order within each half (sample
//                         h H + c L + i at h H + i nthr + c).  Whether the row ionizes at all
//                         is decided for the pair (an OR across the seam).
//   nl_pair_back_kernel   two independent CTAs per row (no cluster): CTA h reads both halves
//                         of each source, forms y_h on the fly, transforms it (H points) and
//                         combines the spectra and the RK4 sum of calculate_NLstep
//                         (propagator.cu:386-421, 679-710) on the positions of half h.
#include <cooperative_groups.h>

#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_plasma.cuh"

namespace cg = cooperative_groups;

namespace gs {

namespace {

constexpr int kPairL = 16;   // samples per chunk (per thread) in the recurrences

// exchange slots of the front kernel (T2 / Rl words in the xc / xr arrays)
enum { XC_ZEND = 0, XC_ZPEER = 1, XC_EPREV = 2, XC_COUNT = 4 };
enum { XR_SIN = 0, XR_CM = 2, XR_MM = 4, XR_PCM = 6, XR_PMM = 8, XR_WPREV = 10, XR_ION = 11, XR_COUNT = 12 };

// rows of N = 2^(LOGH + 1) per precision: FP32 32768, FP64 16384 (a half row of 16384 /
// 8192 complex, H/16 threads per CTA, fills one SM's shared memory with its rates)
template <typename Rl> struct PairShape {
    static constexpr int LOGH = sizeof(Rl) == 4 ? 14 : 13;
    static constexpr int H = 1 << LOGH;
    static constexpr int N = 2 * H;
    static constexpr int THREADS = H / kPairL;
};

template <typename Rl> __host__ __device__ inline size_t pair_front_smem() {
    using T2 = typename Vec2<Rl>::T;
    constexpr int N = PairShape<Rl>::N, H = PairShape<Rl>::H, nthr = PairShape<Rl>::THREADS;
    // E half (padded), twiddles of the full row, chunk ends of the Raman sum, scan scratch and
    // exchange slots (complex); then the rates W_t of the half, the chunk starts of the density,
    // scan scratch and exchange slots (real)
    return ((size_t)padded_len(H) + N / 64 + 64 + nthr + 64 + 4 * XC_COUNT) * sizeof(T2) +
           ((size_t)wb_count(H) + nthr + 64 + 4 * XR_COUNT) * sizeof(Rl);
}

template <typename Rl> __host__ __device__ inline size_t pair_back_smem() {
    return ((size_t)padded_len(PairShape<Rl>::H) + PairShape<Rl>::N / 64 + 64) * sizeof(typename Vec2<Rl>::T);
}

}  // namespace

template <typename Rl>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PairShape<Rl>::THREADS, 1)
    nl_pair_front_kernel(FftArgs<Rl> f, PlasmaArgs<Rl> a, const typename Vec2<Rl>::T* __restrict__ A) {
    using T2 = C2<Rl>;
    // gs_advance: the z-loop stopped (both CTAs of the pair read the same flag and return together)
    if (f.halt && *f.halt) return;
    constexpr int LOGH = PairShape<Rl>::LOGH, H = PairShape<Rl>::H, N = PairShape<Rl>::N;
    constexpr int L = kPairL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cl = cg::this_cluster();
    const int h = (int)cl.block_rank();
    const int tid = threadIdx.x, nthr = blockDim.x;
    T2* E = reinterpret_cast<T2*>(smem_raw);
    T2* twh = E + padded_len(H);
    T2* twl = twh + N / 64;
    T2* cend = twl + 64;
    T2* scA = cend + nthr;
    T2* scB = scA + 32;
    T2* xc = scB + 32;
    Rl* Wb = reinterpret_cast<Rl*>(xc + 4 * XC_COUNT);
    Rl* s_start = Wb + wb_count(H);
    Rl* rA = s_start + nthr;
    Rl* rB = rA + 32;
    Rl* xr = rB + 32;
    T2* Ep = cl.map_shared_rank(E, h ^ 1);
    T2* xcp = cl.map_shared_rank(xc, h ^ 1);
    Rl* Wbp = cl.map_shared_rank(Wb, h ^ 1);
    Rl* xrp = cl.map_shared_rank(xr, h ^ 1);
    const int row = blockIdx.x >> 1;
    const size_t rbase = (size_t)row * N;
    const size_t hbase = rbase + (size_t)h * H;
    const int tg0 = h * H;   // global time index of this CTA's first sample

    // ---- stage input (spectral half h, position order) and its H-point inverse FFT
    load_twiddles<Rl>(twh, twl, f.tw, N, tid, nthr);
    {
        Rl lmax = 0;
        // gs_advance: c dz from the attempt's step size, as the host rounds it
        const Rl cdz = f.dz_dev ? (Rl)(f.c_stage * *f.dz_dev) : f.cdz;
        T2 v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = A[hbase + tid + u * nthr];
        if (f.track_max) {
#pragma unroll
            for (int u = 0; u < 16; u++) lmax = fmax(lmax, v[u].x * v[u].x + v[u].y * v[u].y);
        }
        if (cdz != (Rl)0) {
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const T2 k = f.kp[hbase + tid + u * nthr];
                v[u].x = v[u].x + cdz * k.x;
                v[u].y = v[u].y + cdz * k.y;
            }
        }
#pragma unroll
        for (int u = 0; u < 16; u++) E[pad16(tid + u * nthr)] = v[u];
        if (f.track_max) {
            for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            if ((tid & 31) == 0) atomic_max_nonneg(f.max_out, (double)lmax);
        }
    }
    __syncthreads();
    const TwTab<Rl> tw{twh, twl, f.twb};
    smem_fft_ct<+1, Rl, LOGH>(E, tw, 2, tid, nthr);

    // ---- the radix-2 step across the pair: x[q + h H] = (z_0[q] +- w_N^{-q} z_1[q]) / N
    cl.sync();   // both halves transformed
    {
        // half of the results wait in registers, half in the rates area (not yet in use),
        // until the peer has read this CTA's z
        T2* stash = reinterpret_cast<T2*>(Wb);
        const Rl rn = (Rl)N;
        auto combine = [&](T2 peer, int q) -> T2 {
            const T2 own = E[pad16(q)];
            const T2 z0 = h == 0 ? own : peer;
            const T2 z1 = cmul(h == 0 ? peer : own, cconj(tw(q)));
            T2 x = h == 0 ? cadd(z0, z1) : csub(z0, z1);
            x.x = x.x / rn;
            x.y = x.y / rn;
            return x;
        };
        T2 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = Ep[pad16(tid + (u + 8) * nthr)];   // the peer's z
#pragma unroll
        for (int u = 0; u < 8; u++) stash[u * nthr + tid] = combine(v[u], tid + (u + 8) * nthr);
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = Ep[pad16(tid + u * nthr)];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = combine(v[u], tid + u * nthr);
        cl.sync();   // the peer has read this CTA's z
#pragma unroll
        for (int u = 0; u < 8; u++) E[pad16(tid + u * nthr)] = v[u];
#pragma unroll
        for (int u = 0; u < 8; u++) E[pad16(tid + (u + 8) * nthr)] = stash[u * nthr + tid];
    }
    __syncthreads();

    // ---- photoionization rates W_t of this half (W_0 = 0: the first sample sees E_0 = 0)
    const Rl ND = a.k.ND, tstep = a.k.tstep, U = a.k.U, Pc = a.k.Pc, AV = a.k.AV;
    const Rl invND = a.k.invND, invTAU = a.k.invTAU;
    const bool gas = a.gas != 0;
    bool anyw = false;
    for (int tb = tid; tb < H; tb += 8 * nthr) {
        int n[8];
        Rl dl[8], Iv[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int t = tb + u * nthr;
            n[u] = -1;
            dl[u] = 0;
            Iv[u] = 0;
            if (t < H) {
                const T2 e = E[pad16(t)];
                Iv[u] = e.x * e.x + e.y * e.y;
                if (tg0 + t > 0) n[u] = photo_index<Rl>(Iv[u], &dl[u], a.err);
            }
        }
        Rl w0[8], w1[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            w0[u] = n[u] >= 0 ? __ldg(&a.rate[n[u]]) : (Rl)0;
            w1[u] = n[u] >= 0 ? __ldg(&a.rate[n[u] + 1]) : (Rl)0;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int t = tb + u * nthr;
            if (t < H) {
                const Rl W = n[u] >= 0 ? photo_rate_from<Rl>(w0[u], w1[u], dl[u]) : (Rl)0;
                Wb[pad32(t)] = gas ? gas_rate_slot<Rl>(tg0 + t, Iv[u], W) : W;
                anyw = anyw || n[u] >= 0;
            }
        }
    }
    // whether this half has a sample with W > 0 (exp of the table is positive above its
    // threshold): the row ionizes if either half does, or if rho starts above 0
    const bool own_ion = __syncthreads_or(anyw ? 1 : 0) != 0;
    if (tid == 0) xrp[XR_ION] = own_ion ? (Rl)1 : (Rl)0;
    cl.sync();   // rates of both halves and the peer's flag are in place
    const bool ion = own_ion || xr[XR_ION] != (Rl)0 || a.k.rho0 != (Rl)0;   // the same on both sides
    if (h == 0 && tid == 0 && a.row_ion) a.row_ion[row] = ion ? 1 : 0;
    // the sample before CTA 1's first one lives in CTA 0
    if (h == 1 && tid == 0) {
        xc[XC_EPREV] = Ep[pad16(H - 1)];
        xr[XR_WPREV] = Wbp[pad32(H - 1)];
    }
    cl.sync();   // also: CTA 0 stays resident until CTA 1 has read its shared memory

    auto g_from = [&](T2 e) -> Rl {
        const Rl I = e.x * e.x + e.y * e.y;
        return AV / (U + Pc * I) * I;
    };
    const int c = tid;
    const int t0 = c * L;   // local index of this thread's first sample
    const T2* Ec = E + pad16(t0);   // t0 = 16 c: pad16(t0 + i) = pad16(t0) + i, i < 16
    const Rl* Wc = Wb + pad32(t0);  // t0 = 16 c: pad32(t0 + i) = pad32(t0) + i, i < 16
    // W and g of the sample before this chunk (global sample 0 has none: W = g = 0, or
    // W = -1 below the gas build's threshold)
    Rl Wprev0, gprev0;
    if (t0 > 0) {
        Wprev0 = Wb[pad32(t0 - 1)];
        gprev0 = g_from(E[pad16(t0 - 1)]);
    } else if (h == 1) {
        Wprev0 = xr[XR_WPREV];
        gprev0 = g_from(xc[XC_EPREV]);
    } else {
        Wprev0 = gas ? (Rl)-1 : (Rl)0;
        gprev0 = 0;
    }
    auto run_chunk = [&](Rl s, Rl* dout) -> Rl {
        Rl ro = s, d = (Rl)1;
        Rl W0 = Wprev0;
        if (gas) {   // ionization.cpp:45-60, one level
#pragma unroll 4
            for (int i = 0; i < L; i++) {
                const Rl W1 = Wc[i];
                if (tg0 + t0 + i > 0) ro = gas_step<Rl>(ro, W0, W1, tstep, ND, &d);
                W0 = W1;
            }
            *dout = d;
            return ro;
        }
        Rl g0 = gprev0;
#pragma unroll 4
        for (int i = 0; i < L; i++) {
            const int tg = tg0 + t0 + i;
            const Rl W1 = Wc[i];
            const Rl g1 = (tg == 0) ? (Rl)0 : g_from(Ec[i]);
            if (tg > 0) ro = heun_step<Rl>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
            W0 = W1;
            g0 = g1;
        }
        *dout = d;
        return ro;
    };

    // ---- carrier density: Newton on the chunk starts of both halves.  CTA 1's first start
    // (the seam) is CTA 0's last composed value; the stopping test is the pair's maximum.
    // Both CTAs take the same number of iterations (and cluster barriers).
    s_start[c] = (h == 0 && c == 0) ? a.k.rho0 : (Rl)0;
    __syncthreads();
    // after k iterations the starts of the pair's first k + 1 chunks equal the sequential
    // recurrence's, so 2 nthr + 1 iterations bound the loop with an exact result
    const Rl tol = sizeof(Rl) == 8 ? (Rl)1e-13 : (Rl)1e-5;
    for (int it = 0; it < (ion ? 2 * nthr + 1 : 0); it++) {
        const int par = it & 1;
        const Rl sc = s_start[c];
        Rl D;
        const Rl e = run_chunk(sc, &D);
        Rl Am = D, Bm = e - D * sc;
        block_affine_scan<Rl>(Am, Bm, (Rl)1, (Rl)0, rA, rB);
        const Rl next = Am * s_start[0] + Bm;   // start of chunk c + 1 (of the seam for c = nthr - 1)
        Rl change = 0, mag = 0;
        __syncthreads();
        if (c + 1 < nthr) {
            change = fabs(next - s_start[c + 1]);
            mag = fabs(next);
            s_start[c + 1] = next;
        } else if (h == 0) {
            xrp[XR_SIN + par] = next;
        }
        cl.sync();   // the seam value has arrived
        if (h == 1 && c == 0) {
            const Rl v = xr[XR_SIN + par];
            change = fmax(change, fabs(v - s_start[0]));
            mag = fmax(mag, fabs(v));
            s_start[0] = v;
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
            xr[XR_CM + par] = cm;
            xr[XR_MM + par] = mm;
            xrp[XR_PCM + par] = cm;
            xrp[XR_PMM + par] = mm;
        }
        cl.sync();   // both CTAs' maxima are in place: the same decision on both sides
        const Rl cm = fmax(xr[XR_CM + par], xr[XR_PCM + par]);
        const Rl mm = fmax(xr[XR_MM + par], xr[XR_PMM + par]);
        if (cm <= tol * mm && !a.shoot_exhaust) break;
    }

    // ---- Raman: z_t = a z_{t-1} + I_t; chunk sums, a scan per CTA, the carry across the seam
    const bool rscan = a.raman_scan != 0;
    const T2 ra = T2{a.k.a_re, a.k.a_im};
    T2 zs = T2{0, 0}, zN = T2{0, 0}, pw = T2{0, 0};
    if (rscan) {
        T2 zl = T2{0, 0}, aL = T2{1, 0};
#pragma unroll 4
        for (int i = 0; i < L; i++) {
            const T2 e = Ec[i];
            zl = cmul(ra, zl);
            zl.x += e.x * e.x + e.y * e.y;
            aL = cmul(aL, ra);
        }
        T2 Am = aL, Bm = zl;
        block_affine_scan<T2>(Am, Bm, T2{1, 0}, T2{0, 0}, scA, scB);
        cend[c] = Bm;   // z at the end of chunk c from z = 0 at this CTA's first sample
        if (c == nthr - 1) {
            xc[XC_ZEND] = Bm;
            xcp[XC_ZPEER] = Bm;
        }
        cl.sync();
        // (a^L)^c and a^H = (a^L)^nthr by binary powering (no transcendental per thread)
        T2 pc = T2{1, 0}, aH = T2{1, 0};
        {
            T2 b = aL;
            for (int k = c; k > 0; k >>= 1) {
                if (k & 1) pc = cmul(pc, b);
                b = cmul(b, b);
            }
            b = aL;
            for (int k = nthr; k > 0; k >>= 1) {
                if (k & 1) aH = cmul(aH, b);
                b = cmul(b, b);
            }
        }
        const T2 z0end = h == 0 ? xc[XC_ZEND] : xc[XC_ZPEER];   // z at sample H - 1
        const T2 z1loc = h == 0 ? xc[XC_ZPEER] : xc[XC_ZEND];   // CTA 1's own sum
        zN = cadd(z1loc, cmul(aH, z0end));
        zs = (c == 0) ? T2{0, 0} : cend[c - 1];
        if (h == 1) zs = cadd(zs, cmul(pc, z0end));
        // a^{t+1} at this chunk's first global sample t = h H + c L
        pw = cmul(h == 1 ? cmul(aH, pc) : pc, ra);
    }

    // ---- final pass: density, Raman Q and the three source rows
    {
        Rl ro = s_start[c], d = 1;
        Rl W0 = Wprev0, g0 = gprev0;
        T2 z = zs;
        const T2 oma = T2{a.k.oma_re, a.k.oma_im};
        const Rl fRM = a.k.fRM, omf = a.k.omf;
#pragma unroll 4
        for (int i = 0; i < L; i++) {
            const int tg = tg0 + t0 + i;
            const T2 e = Ec[i];
            const Rl I = e.x * e.x + e.y * e.y;
            const Rl W1 = Wc[i];
            T2 loss = T2{0, 0};
            if (!ion) {
                // the density stays 0 and there is no loss
            } else if (gas) {
                if (tg > 0) ro = gas_step<Rl>(ro, W0, W1, tstep, ND, &d);
                W0 = W1;
                if (tg < N - 1 && W1 >= 0) {   // ionization.cpp:60-81
                    const Rl sl = gas_loss_factor<Rl>(W1, ro, I, tstep, ND, U, Pc);
                    loss = T2{sl * e.x, sl * e.y};
                }
            } else {
                const Rl g1 = (tg == 0) ? (Rl)0 : AV / (U + Pc * I) * I;
                if (tg > 0) ro = heun_step<Rl>(ro, W0, g0, W1, g1, tstep, ND, invND, invTAU, &d);
                W0 = W1;
                g0 = g1;
                // loss[t] (ionization.cpp:43): W at (E_t, rho_t), the reference's log-threshold test
                if (tg > 0 && tg < N - 1 && I > (Rl)GS_ION_MIN_LN) {
                    const Rl W01 = (ro > ND) ? (Rl)0 : W1;
                    const Rl sl = -(Rl)0.5 * W01 * (U + Pc * I) / I;
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
                const T2 hh = cmul(a.th[tg], cmul(e2, e));
                src3.x += hh.x;
                src3.y += hh.y;
            }
            const size_t q = hbase + (size_t)i * nthr + c;   // chunk-interleaved within the half
            if (ion || !a.row_ion) {   // zero rows are not written: nl_pair_back skips their FFTs
                a.u1[q] = loss;
                a.u2[q] = T2{ro * e.x, ro * e.y};
            }
            a.u3[q] = src3;
        }
    }
}

template <typename Rl>
__global__ void __launch_bounds__(PairShape<Rl>::THREADS, 1) nl_pair_back_kernel(FftArgs<Rl> f, SpecArgs<Rl> s) {
    using T2 = C2<Rl>;
    if (f.halt && *f.halt) return;   // gs_advance: the z-loop stopped
    constexpr int LOGH = PairShape<Rl>::LOGH, H = PairShape<Rl>::H, N = PairShape<Rl>::N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int h = blockIdx.x & 1;
    const int row = blockIdx.x >> 1;
    const int tid = threadIdx.x, nthr = blockDim.x;
    T2* buf = reinterpret_cast<T2*>(smem_raw);
    T2* twh = buf + padded_len(H);
    T2* twl = twh + N / 64;
    const size_t rbase = (size_t)row * N;
    const size_t pbase = rbase + (size_t)h * H;   // this CTA's spectral positions
    load_twiddles<Rl>(twh, twl, f.tw, N, tid, nthr);
    __syncthreads();
    const TwTab<Rl> tw{twh, twl, f.twb};
    T2* acc = s.kp;   // the new k doubles as the accumulator of the three spectra
    Rl lmax = 0;
    // a row without ionization has loss = rho E = 0: only the Kerr source (FFT(0) = 0 adds
    // nothing), or, with Kerr off, no source at all (k = 0: one pass with a zero spectrum)
    const bool ion = s.row_ion ? s.row_ion[row] != 0 : true;
    const int lastsrc = s.kerr_on ? 2 : 1;
    const int first = ion ? 0 : lastsrc;
    const bool zero_src = !ion && !s.kerr_on;
    for (int src = first; src <= lastsrc; src++) {
        const T2* in = src == 0 ? s.u1 : (src == 1 ? s.u2 : s.u3);
        if (!zero_src) {
            // position u nthr + c of each half holds that half's sample c L + u: samples q and
            // q + H sit at the same offset of the two halves
#pragma unroll
            for (int ub = 0; ub < 16; ub += 8) {
                T2 x0[8], x1[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    x0[u] = in[rbase + tid + (ub + u) * nthr];
                    x1[u] = in[rbase + H + tid + (ub + u) * nthr];
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = tid * kPairL + ub + u;
                    buf[pad16(q)] = h == 0 ? cadd(x0[u], x1[u]) : cmul(csub(x0[u], x1[u]), tw(q));
                }
            }
            __syncthreads();
            smem_fft_ct<-1, Rl, LOGH>(buf, tw, 2, tid, nthr);
        }
        const bool last = src == lastsrc;
        constexpr int SB = 4;
        for (int pb = tid; pb < H; pb += SB * nthr) {
            T2 v[SB], ac[SB], o[SB], cf[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int p = pb + u * nthr;
                const int gp = h * H + p;
                v[u] = zero_src ? T2{0, 0} : buf[pad16(p)];
                ac[u] = src > first ? acc[rbase + gp] : T2{0, 0};
                // the spectral coefficient: PLASMA_FUNC for FFT(rho E), -j KERR_PROFILE for FFT(Q E)
                if (src == 1) cf[u] = s.pf[gp];
                else if (src == 2) cf[u] = T2{(Rl)0, -s.kerr[gp]};
                else cf[u] = T2{(Rl)1, (Rl)0};
                o[u] = (last && s.stage > 0) ? s.nb[rbase + gp] : T2{0, 0};
            }
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const size_t gi = pbase + pb + u * nthr;
                T2 k;
                if (src == 0) {
                    k = v[u];
                } else if (src == 1) {
                    k = cadd(ac[u], cmul(v[u], cf[u]));   // FFT(loss) + FFT(rho E) PLASMA_FUNC
                } else {
                    k = ac[u];                              // += -j KERR_PROFILE FFT(Q E)
                    k.x += -cf[u].y * v[u].y;
                    k.y += cf[u].y * v[u].x;
                }
                if (!last) {
                    acc[gi] = k;
                    continue;
                }
                // RK4: (k1 + 2 k2 + 2 k3 + k4) / 6 accumulated in that order (propagator.cu:412)
                T2 nb;
                if (s.stage == 0) {
                    nb = k;
                } else if (s.stage < 3) {
                    nb = T2{o[u].x + (Rl)2 * k.x, o[u].y + (Rl)2 * k.y};
                } else {
                    nb = T2{(o[u].x + k.x) / (Rl)6, (o[u].y + k.y) / (Rl)6};
                    lmax = fmax(lmax, nb.x * nb.x + nb.y * nb.y);
                }
                s.nb[gi] = nb;
                if (s.stage < 3) acc[gi] = k;
            }
        }
        __syncthreads();
    }
    if (s.stage == 3) {
        for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if ((tid & 31) == 0) atomic_max_nonneg(s.max_out, (double)lmax);
    }
}

template <typename Rl> bool nl_pair_supported(int N) {
    return N == PairShape<Rl>::N && pair_front_smem<Rl>() <= 227 * 1024 && pair_back_smem<Rl>() <= 227 * 1024;
}

template <typename Rl> cudaError_t nl_pair_setup(int N) {
    (void)N;
    cudaError_t e = cudaFuncSetAttribute(nl_pair_front_kernel<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pair_front_smem<Rl>());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(nl_pair_back_kernel<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)pair_back_smem<Rl>());
}

template <typename Rl>
cudaError_t launch_nl_pair_front(FftArgs<Rl> f, PlasmaArgs<Rl> a, const typename Vec2<Rl>::T* A, int rows,
                                 cudaStream_t st, long long* nl) {
    nl_pair_front_kernel<Rl><<<2 * rows, PairShape<Rl>::THREADS, pair_front_smem<Rl>(), st>>>(f, a, A);
    (*nl)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_nl_pair_back(FftArgs<Rl> f, SpecArgs<Rl> s, int rows, cudaStream_t st, long long* nl) {
    nl_pair_back_kernel<Rl><<<2 * rows, PairShape<Rl>::THREADS, pair_back_smem<Rl>(), st>>>(f, s);
    (*nl)++;
    return cudaGetLastError();
}

#define GS_PAIR_INST(Rl)                                                                                     \
    template bool nl_pair_supported<Rl>(int);                                                                \
    template cudaError_t nl_pair_setup<Rl>(int);                                                             \
    template cudaError_t launch_nl_pair_front<Rl>(FftArgs<Rl>, PlasmaArgs<Rl>, const typename Vec2<Rl>::T*, \
                                                  int, cudaStream_t, long long*);                            \
    template cudaError_t launch_nl_pair_back<Rl>(FftArgs<Rl>, SpecArgs<Rl>, int, cudaStream_t, long long*);
GS_PAIR_INST(float)
GS_PAIR_INST(double)

}  // namespace gs
