// gs_internal.cuh -- shared device helpers of the GB300 UPPE core.
//
// Complex numbers are double2 / float2 (re, im).  Spectral rows are stored in the
// FFT's "position order" (see fft_position_map in gs_abi.cu): the forward FFT leaves
// its output digit-reversed and the inverse FFT consumes that order, so no reordering
// pass is ever run on the device; every per-omega table is uploaded in the same order.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gs_kernels.h"

namespace gs {

template <typename R> using C2 = typename Vec2<R>::T;

template <typename T2> __device__ __forceinline__ T2 mk(double x, double y);
template <> __device__ __forceinline__ double2 mk<double2>(double x, double y) { return make_double2(x, y); }
template <> __device__ __forceinline__ float2 mk<float2>(double x, double y) { return make_float2((float)x, (float)y); }

template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { a.x += b.x; a.y += b.y; return a; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { a.x -= b.x; a.y -= b.y; return a; }
// (a.x + i a.y)(b.x + i b.y) with the naive formula (what std::complex gives for finite values)
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { a.y = -a.y; return a; }

// error word bits written by kernels (host maps them to the reference's exceptions; a
// GS_CHECK build's failed index test sets GS_ERRBIT_BOUNDS, gs_kernels.h)
enum : unsigned { ERRBIT_BLAST = 1u, ERRBIT_NAN = 2u };

// GS_CHECK builds (`python -m gsolver_gb300.build --check`: -DGS_CHECK=1, a library of its own
// under _build_check/) test the indices the hot kernels take from index tables (compact-column
// maps, rate-table rows) before each access: a failed test sets ERRBIT_BOUNDS in the error word
// and the access is skipped (no trap), and the call returns GS_ERR_CUDA "index out of bounds".
// Other builds compile the test away.
#ifndef GS_CHECK
#define GS_CHECK 0
#endif
__device__ __forceinline__ bool in_bounds(bool ok, unsigned* err) {
#if GS_CHECK
    if (!ok) {
        if (err) atomicOr(err, GS_ERRBIT_BOUNDS);
        return false;
    }
#else
    (void)ok;
    (void)err;
#endif
    return true;
}

// Non-negative doubles order like their bit patterns: max-reduce through 64-bit atomics.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Asynchronous prefetch of a row into L2 (cp.async.bulk.prefetch): lanes 0..3 of the calling
// warp each request a quarter (other lane values request nothing).  p 16-byte aligned, bytes
// a multiple of 64.
__device__ __forceinline__ void prefetch_row_l2(const void* p, size_t bytes, int lane) {
    if (lane >= 0 && lane < 4) {
        const size_t q = bytes / 4;
        const char* a = static_cast<const char*>(p) + lane * q;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)q) : "memory");
    }
}

// ------------------------------------------------------------------ register DFTs --
// Constant 16th roots of unity, cos / sin(2*pi*j/16) for j = 0..7.
__device__ __forceinline__ double root16c(int j) {
    const double c[8] = {1.0, 0.92387953251128674, 0.70710678118654757, 0.38268343236508978,
                         0.0, -0.38268343236508978, -0.70710678118654757, -0.92387953251128674};
    return c[j];
}
__device__ __forceinline__ double root16s(int j) {
    const double s[8] = {0.0, 0.38268343236508978, 0.70710678118654757, 0.92387953251128674,
                         1.0, 0.92387953251128674, 0.70710678118654757, 0.38268343236508978};
    return s[j];
}

// v * exp(SIGN * 2*pi*i * k / R)   (k < R/2, R | 16)
template <int R, int SIGN, typename Rl, typename T2>
__device__ __forceinline__ T2 twc(T2 v, int k) {
    const int j = k * (16 / R);
    if (j == 0) return v;
    if (j == 4) {  // multiply by SIGN*i
        T2 r;
        if (SIGN < 0) { r.x = v.y; r.y = -v.x; } else { r.x = -v.y; r.y = v.x; }
        return r;
    }
    const Rl c = (Rl)root16c(j), s = (Rl)(SIGN * root16s(j));
    T2 r;
    r.x = v.x * c - v.y * s;
    r.y = v.x * s + v.y * c;
    return r;
}

// The butterfly (e + t, e - t).  For FP32 pairs each is one packed instruction (add / sub
// .rn.f32x2): the same two correctly rounded results as the scalar form, half the issue slots.
template <typename T2> __device__ __forceinline__ void bfly(T2& a, T2& b, T2 e, T2 t) {
    a = cadd(e, t);
    b = csub(e, t);
}
#if defined(__CUDA_ARCH__)
template <> __device__ __forceinline__ void bfly<float2>(float2& a, float2& b, float2 e, float2 t) {
    unsigned long long re, rt, ra, rb;
    re = (unsigned long long)__float_as_uint(e.x) | ((unsigned long long)__float_as_uint(e.y) << 32);
    rt = (unsigned long long)__float_as_uint(t.x) | ((unsigned long long)__float_as_uint(t.y) << 32);
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(ra) : "l"(re), "l"(rt));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rb) : "l"(re), "l"(rt));
    a = make_float2(__uint_as_float((unsigned)ra), __uint_as_float((unsigned)(ra >> 32)));
    b = make_float2(__uint_as_float((unsigned)rb), __uint_as_float((unsigned)(rb >> 32)));
}
#endif

// In-register radix-2 decimation-in-time DFT of size R (1,2,4,8,16), natural order in/out.
template <int R, int SIGN, typename Rl, typename T2> struct RegDFT {
    static __device__ __forceinline__ void run(T2* x) {
        T2 e[R / 2], o[R / 2];
#pragma unroll
        for (int i = 0; i < R / 2; i++) { e[i] = x[2 * i]; o[i] = x[2 * i + 1]; }
        RegDFT<R / 2, SIGN, Rl, T2>::run(e);
        RegDFT<R / 2, SIGN, Rl, T2>::run(o);
#pragma unroll
        for (int k = 0; k < R / 2; k++) bfly(x[k], x[k + R / 2], e[k], twc<R, SIGN, Rl>(o[k], k));
    }
};
template <int SIGN, typename Rl, typename T2> struct RegDFT<1, SIGN, Rl, T2> {
    static __device__ __forceinline__ void run(T2*) {}
};

// -------------------------------------------------------------- shared-memory FFT --
// A row of M complex lives in shared memory with one pad slot per 16 elements
// (element i at pad16(i)): every radix-16/8/4/2 stage below then touches 16 distinct
// 8-byte bank pairs per half-warp (checked for each stage shape: sub >= 16, sub = 8, 4, 1).
__host__ __device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int padded_len(int M) { return M + (M >> 4); }
// real per-sample rows: one pad word per 32 (conflict-free for chunks of 16 consecutive samples)
__host__ __device__ __forceinline__ int pad32(int i) { return i + (i >> 5); }
// slots of such a row, rounded to 4 elements so that what follows stays 16-byte aligned
__host__ __device__ __forceinline__ int wb_count(int N) { return (N + N / 32 + 1 + 3) & ~3; }

// Twiddles w(j) = exp(-2 pi i j / N) from two shared tables: w = hi[j >> 6] * lo[j & 63].
// `base`, when set, is the per-stage base table below (global memory); the radix-16 stages
// then take their twiddles from it instead of hi * lo.
template <typename Rl> struct TwTab {
    const C2<Rl>* hi;
    const C2<Rl>* lo;
    const C2<Rl>* base = nullptr;
    __device__ __forceinline__ C2<Rl> operator()(int j) const { return cmul(hi[j >> 6], lo[j & 63]); }
};

// Per-stage base twiddles of an M-point FFT (M = 2^logM) on rows of N = M * twstride.
// Radix-16 stage j works on sub-problems of size S_j = M / 16^j with sub_j = S_j / 16
// butterfly offsets q and twiddles w_N^{q r scale_j}, r = 1..15, scale_j = (M / S_j) twstride.
// The table holds, per stage, six rows of sub_j entries: w_N^{q m scale_j} for
// m = 1, 2, 3, 4, 8, 12 (each rounded once from the double value); every other r is
// w^{q (r & 3)} w^{q (r & 12)}, one product of two tabulated values.  Rows are indexed by q:
// a warp's lanes (consecutive q) read consecutive words.
__host__ __device__ inline int tw_base_offset(int logM, int j) {
    int off = 0;
    for (int i = 0; i < j; i++) off += 6 * ((1 << logM) >> (4 * i + 4));
    return off;
}
__host__ __device__ inline int tw_base_count(int logM) { return tw_base_offset(logM, logM / 4); }

// x[r] *= w^{SIGN-sign q r} for r = 1..15 from the stage's base rows (conjugated for the
// inverse transform, SIGN > 0)
template <int SIGN, typename Rl>
__device__ __forceinline__ void apply_tw16(C2<Rl>* x, const C2<Rl>* __restrict__ stb, int sub, int q) {
    using T2 = C2<Rl>;
    // w^{q}, w^{2q}, w^{3q} are held; w^{4q}, w^{8q}, w^{12q} are read when used (registers)
    T2 b[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        b[k] = __ldg(stb + k * sub + q);
        if (SIGN > 0) b[k].y = -b[k].y;
    }
#pragma unroll
    for (int l = 1; l < 4; l++) x[l] = cmul(x[l], b[l - 1]);
#pragma unroll
    for (int hi = 1; hi < 4; hi++) {
        T2 bh = __ldg(stb + (2 + hi) * sub + q);
        if (SIGN > 0) bh.y = -bh.y;
        x[4 * hi] = cmul(x[4 * hi], bh);
#pragma unroll
        for (int l = 1; l < 4; l++) x[4 * hi + l] = cmul(x[4 * hi + l], cmul(bh, b[l - 1]));
    }
}

// fill hi[N/64] and lo[64] from the global table tw[j] = exp(-2 pi i j / N)
template <typename Rl>
__device__ __forceinline__ void load_twiddles(C2<Rl>* hi, C2<Rl>* lo, const C2<Rl>* __restrict__ tw, int N, int tid,
                                              int nthr) {
    for (int j = tid; j < N / 64; j += nthr) hi[j] = tw[j * 64];
    for (int j = tid; j < 64; j += nthr) lo[j] = tw[j];
}

// One radix-R stage on a padded row of length M.
// Forward (SIGN=-1, decimation in frequency): butterfly (q, block) reads R elements at
// stride sub=S/R, DFT_R, multiplies output r by w_S^{q r}, writes them back in place.
// Inverse (SIGN=+1) undoes the forward stage (conjugate twiddle first, then DFT_R).
// A sub-row of length M = N/twstride uses w_M^k = w_N^{k twstride}.
template <int R, int SIGN, typename Rl>
__device__ __forceinline__ void fft_stage(C2<Rl>* buf, int M, int S, const TwTab<Rl>& tw, int twstride, int tid,
                                          int nthr, const C2<Rl>* stb) {
    using T2 = C2<Rl>;
    const int sub = S / R;
    const int nb = M / R;
    const int scale = (M / S) * twstride;
    for (int b = tid; b < nb; b += nthr) {
        const int q = b & (sub - 1);
        const int base = (b / sub) * S + q;
        T2 x[R];
#pragma unroll
        for (int r = 0; r < R; r++) x[r] = buf[pad16(base + sub * r)];
        if (SIGN > 0 && q != 0) {
            if (R == 16 && stb) {
                apply_tw16<SIGN, Rl>(x, stb, sub, q);
            } else {
#pragma unroll
                for (int r = 1; r < R; r++) x[r] = cmul(x[r], cconj(tw(q * r * scale)));
            }
        }
        RegDFT<R, SIGN, Rl, T2>::run(x);
        if (SIGN < 0 && q != 0) {
            if (R == 16 && stb) {
                apply_tw16<SIGN, Rl>(x, stb, sub, q);
            } else {
#pragma unroll
                for (int r = 1; r < R; r++) x[r] = cmul(x[r], tw(q * r * scale));
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) buf[pad16(base + sub * r)] = x[r];
    }
}

template <int SIGN, typename Rl>
__device__ __forceinline__ void fft_stage_rt(int R, C2<Rl>* buf, int M, int S, const TwTab<Rl>& tw, int twstride,
                                             int tid, int nthr, const C2<Rl>* stb) {
    switch (R) {
        case 16: fft_stage<16, SIGN, Rl>(buf, M, S, tw, twstride, tid, nthr, stb); break;
        case 8: fft_stage<8, SIGN, Rl>(buf, M, S, tw, twstride, tid, nthr, nullptr); break;
        case 4: fft_stage<4, SIGN, Rl>(buf, M, S, tw, twstride, tid, nthr, nullptr); break;
        case 2: fft_stage<2, SIGN, Rl>(buf, M, S, tw, twstride, tid, nthr, nullptr); break;
        default: break;
    }
}

// Radix schedule of an M-point FFT (M = 2^m): 16, 16, ..., then 2^(m mod 4).
__host__ __device__ inline int fft_num_stages(int logM) { return logM / 4 + ((logM % 4) ? 1 : 0); }
__host__ __device__ inline int fft_stage_radix(int logM, int j) {
    return (j < logM / 4) ? 16 : (1 << (logM % 4));
}

// ---- the same transform with the row length fixed at compile time (the long rows).
// Element r of butterfly (q, block) of a stage sits at pad16(base) + pad16(sub r): exact
// for every stage here (sub a power of two; sub >= 16, or q < sub with sub | 16, or q = 0 in
// the last small-radix stage), so no index math is repeated per element: a butterfly
// computes one shared address and reads and writes at immediate offsets.
constexpr int ct_radix(int logM, int j) { return (j < logM / 4) ? 16 : (1 << (logM % 4)); }
constexpr int ct_stages(int logM) { return logM / 4 + ((logM % 4) ? 1 : 0); }
constexpr int ct_size(int logM, int j) {   // S_j = M / (R_0 ... R_{j-1})
    int S = 1 << logM;
    for (int i = 0; i < j; i++) S /= ct_radix(logM, i);
    return S;
}

template <int R, int SIGN, typename Rl, int M, int S>
__device__ __forceinline__ void fft_stage_ct(C2<Rl>* buf, const TwTab<Rl>& tw, int twstride, int tid, int nthr,
                                             const C2<Rl>* stb) {
    using T2 = C2<Rl>;
    constexpr int sub = S / R;
    constexpr int nb = M / R;
    for (int b = tid; b < nb; b += nthr) {
        const int q = b & (sub - 1);
        T2* p = buf + pad16((b / sub) * S + q);
        T2 x[R];
#pragma unroll
        for (int r = 0; r < R; r++) x[r] = p[pad16(sub * r)];
        if (SIGN > 0 && q != 0) {
            if (R == 16 && stb) {
                apply_tw16<SIGN, Rl>(x, stb, sub, q);
            } else {
                const int scale = (M / S) * twstride;
#pragma unroll
                for (int r = 1; r < R; r++) x[r] = cmul(x[r], cconj(tw(q * r * scale)));
            }
        }
        RegDFT<R, SIGN, Rl, T2>::run(x);
        if (SIGN < 0 && q != 0) {
            if (R == 16 && stb) {
                apply_tw16<SIGN, Rl>(x, stb, sub, q);
            } else {
                const int scale = (M / S) * twstride;
#pragma unroll
                for (int r = 1; r < R; r++) x[r] = cmul(x[r], tw(q * r * scale));
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) p[pad16(sub * r)] = x[r];
    }
}

template <int SIGN, typename Rl, int LOGM, int J>
__device__ __forceinline__ void fft_stage_ct_j(C2<Rl>* buf, const TwTab<Rl>& tw, int twstride, int tid, int nthr) {
    constexpr int R = ct_radix(LOGM, J);
    const C2<Rl>* stb = (R == 16 && tw.base) ? tw.base + tw_base_offset(LOGM, J) : nullptr;
    fft_stage_ct<R, SIGN, Rl, (1 << LOGM), ct_size(LOGM, J)>(buf, tw, twstride, tid, nthr, stb);
    __syncthreads();
}

template <int SIGN, typename Rl, int LOGM>
__device__ __forceinline__ void smem_fft_ct(C2<Rl>* buf, const TwTab<Rl>& tw, int twstride, int tid, int nthr) {
    constexpr int NS = ct_stages(LOGM);
    static_assert(NS >= 1 && NS <= 4, "rows of 2^4 .. 2^16");
    if constexpr (SIGN < 0) {   // forward: S_0 = M first
        fft_stage_ct_j<SIGN, Rl, LOGM, 0>(buf, tw, twstride, tid, nthr);
        if constexpr (NS > 1) fft_stage_ct_j<SIGN, Rl, LOGM, 1>(buf, tw, twstride, tid, nthr);
        if constexpr (NS > 2) fft_stage_ct_j<SIGN, Rl, LOGM, 2>(buf, tw, twstride, tid, nthr);
        if constexpr (NS > 3) fft_stage_ct_j<SIGN, Rl, LOGM, 3>(buf, tw, twstride, tid, nthr);
    } else {                    // inverse: the stages undone in reverse order
        if constexpr (NS > 3) fft_stage_ct_j<SIGN, Rl, LOGM, 3>(buf, tw, twstride, tid, nthr);
        if constexpr (NS > 2) fft_stage_ct_j<SIGN, Rl, LOGM, 2>(buf, tw, twstride, tid, nthr);
        if constexpr (NS > 1) fft_stage_ct_j<SIGN, Rl, LOGM, 1>(buf, tw, twstride, tid, nthr);
        fft_stage_ct_j<SIGN, Rl, LOGM, 0>(buf, tw, twstride, tid, nthr);
    }
}

// Full in-place M-point FFT of a padded shared row (caller syncs before; ends synced).
// Rows of 4096 .. 16384 points take the compile-time form above.
template <int SIGN, typename Rl>
__device__ void smem_fft(C2<Rl>* buf, int M, int logM, const TwTab<Rl>& tw, int twstride, int tid, int nthr) {
    switch (logM) {
        case 12: smem_fft_ct<SIGN, Rl, 12>(buf, tw, twstride, tid, nthr); return;
        case 13: smem_fft_ct<SIGN, Rl, 13>(buf, tw, twstride, tid, nthr); return;
        case 14: smem_fft_ct<SIGN, Rl, 14>(buf, tw, twstride, tid, nthr); return;
        default: break;
    }
    const int J = fft_num_stages(logM);
    if (SIGN < 0) {
        int S = M;
        for (int j = 0; j < J; j++) {
            const int R = fft_stage_radix(logM, j);
            const C2<Rl>* stb = (tw.base && R == 16) ? tw.base + tw_base_offset(logM, j) : nullptr;
            fft_stage_rt<SIGN, Rl>(R, buf, M, S, tw, twstride, tid, nthr, stb);
            __syncthreads();
            S /= R;
        }
    } else {
        // stage j works on sub-problems of size S_j = M / (R_0 ... R_{j-1})
        for (int j = J - 1; j >= 0; j--) {
            int S = M;
            for (int i = 0; i < j; i++) S /= fft_stage_radix(logM, i);
            const int R = fft_stage_radix(logM, j);
            const C2<Rl>* stb = (tw.base && R == 16) ? tw.base + tw_base_offset(logM, j) : nullptr;
            fft_stage_rt<SIGN, Rl>(R, buf, M, S, tw, twstride, tid, nthr, stb);
            __syncthreads();
        }
    }
}

}  // namespace gs
