// In-place, mixed-radix Stockham FFT on data held in shared memory, executed cooperatively by all
// threads of a CTA.  Used by every transform of the propagator: the transverse 2D FFTs of one
// frequency slice and the time-axis real FFTs of a tile of transverse points.
//
// Data: `nb` transforms of length N = 2^logN; element e of transform b sits at buf[b*bs + e*es].
// One radix-R stage (p = product of the radices already applied, k = i mod p):
//     u_r = buf[i + r N/R] * W_{pR}^{r k},  y = DFT_R(u),  buf'[(i-k)R + k + s p] = y_s
// which leaves the result in natural order after the last stage.  Each stage reads all of its
// inputs into registers, synchronises, then writes in place, so no second buffer is needed.
// Twiddles come from a table tw[j] = exp(-2 pi i j / NT) (computed in FP64 on the host), NT = 2^twLog
// >= N; the inverse transform uses conjugated twiddles and is unnormalised.
#pragma once
#include "common.cuh"

#define UPPE_SQRT1_2 0.70710678118654752440f

template <int R>
UPPE_DEV void dft_small(float2 (&u)[R], bool inv);

template <>
UPPE_DEV void dft_small<2>(float2 (&u)[2], bool) {
    float2 a = u[0], b = u[1];
    u[0] = cadd(a, b);
    u[1] = csub(a, b);
}

template <>
UPPE_DEV void dft_small<4>(float2 (&u)[4], bool inv) {
    float2 a0 = cadd(u[0], u[2]), a1 = csub(u[0], u[2]);
    float2 a2 = cadd(u[1], u[3]), a3 = csub(u[1], u[3]);
    // forward: y1 = a1 - i a3, y3 = a1 + i a3; inverse: signs swapped
    float2 t = inv ? cmul_i(a3) : cmul_mi(a3);
    u[0] = cadd(a0, a2);
    u[2] = csub(a0, a2);
    u[1] = cadd(a1, t);
    u[3] = csub(a1, t);
}

template <>
UPPE_DEV void dft_small<8>(float2 (&u)[8], bool inv) {
    float2 e[4] = {u[0], u[2], u[4], u[6]};
    float2 o[4] = {u[1], u[3], u[5], u[7]};
    dft_small<4>(e, inv);
    dft_small<4>(o, inv);
    const float sg = inv ? 1.f : -1.f;
    // W8^s = exp(sg * 2 pi i s / 8)
    float2 w1 = make_float2(UPPE_SQRT1_2, sg * UPPE_SQRT1_2);
    float2 w3 = make_float2(-UPPE_SQRT1_2, sg * UPPE_SQRT1_2);
    float2 t0 = o[0];
    float2 t1 = cmul(o[1], w1);
    float2 t2 = inv ? cmul_i(o[2]) : cmul_mi(o[2]);
    float2 t3 = cmul(o[3], w3);
    u[0] = cadd(e[0], t0);
    u[4] = csub(e[0], t0);
    u[1] = cadd(e[1], t1);
    u[5] = csub(e[1], t1);
    u[2] = cadd(e[2], t2);
    u[6] = csub(e[2], t2);
    u[3] = cadd(e[3], t3);
    u[7] = csub(e[3], t3);
}

// Twiddle sources: a global table of 2^log entries tw[j] = exp(-2 pi i j / 2^log), or a shared
// table holding the first half of such a table (the second half is its negative).
struct TwGlobal {
    const float2* __restrict__ p;
    int log;
    UPPE_DEV float2 get(int j) const { return __ldg(&p[j]); }
};
struct TwHalfShared {
    const float2* p;
    int log;
    UPPE_DEV float2 get(int j) const {
        const int half = 1 << (log - 1);
        float2 v = p[j & (half - 1)];
        return (j & half) ? make_float2(-v.x, -v.y) : v;
    }
};

// Row order of a transform in shared memory.  NoSwizzle: element e in row e.  RowSwizzle: element e
// in row e ^ key(e), key(e) = bits [sh, sh + 3) of e & mask, a permutation within every aligned
// group of 8 rows.  With rows of C batched transforms (batch-fast data), the rows 8 apart that a
// warp touches in a radix-8 stage with p = 1 (and in a sweep over consecutive segments of 8 rows)
// then fall on distinct banks: sh = 3 when C >= 2, sh = 4 when C = 1 (a warp then spans 16 such
// rows).  mask = N - 1 leaves row N (the Nyquist row of a half spectrum) in place; mask = 0 is the
// identity.  The time pass swizzles for C <= 4 (2- to 16-way conflicts without it); at C = 8 the
// conflicts are 2-way and the extra address registers cost more than they save; at C >= 16 the
// rows of a half-warp are conflict-free as they are.
struct NoSwizzle {
    UPPE_DEV int operator()(int e) const { return e; }
};
struct RowSwizzle {
    int mask, sh;
    UPPE_DEV int operator()(int e) const { return e ^ (((e & mask) >> sh) & 7); }
};

// One radix-R stage over all nb transforms; thread `tid` of `nthr` handles ITEMS butterflies.
// batch_fast: consecutive threads take consecutive transforms (use when es != 1 so that the
// accesses of a warp are contiguous in shared memory).
template <int R, int ITEMS, class TW, class SW = NoSwizzle>
UPPE_DEV void stockham_stage(float2* buf, int logN, int logp, int lognb, int bs, int es, const TW& tw, bool inv,
                             bool batch_fast, int tid, int nthr, const SW& sw = SW{}) {
    constexpr int LOGR = (R == 2) ? 1 : (R == 4) ? 2 : 3;
    const int logq = logN - LOGR;
    const int nq = 1 << logq;
    const int p = 1 << logp;
    float2 u[ITEMS][R];
    int dst[ITEMS], b_of[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
        const int g = tid + it * nthr;
        int b, i;
        if (batch_fast) {
            b = g & ((1 << lognb) - 1);
            i = g >> lognb;
        } else {
            i = g & (nq - 1);
            b = g >> logq;
        }
        const int k = i & (p - 1);
        const float2* base = buf + b * bs;
#pragma unroll
        for (int r = 0; r < R; ++r) u[it][r] = base[sw(i + r * nq) * es];
        if (logp > 0) {
            const int sh = tw.log - logp - LOGR;  // NT / (p R)
            if constexpr (R == 8) {
                // W^k, W^2k, W^4k from the table; the other powers as products of at most two of them
                float2 w1 = tw.get(k << sh), w2 = tw.get((2 * k) << sh), w4 = tw.get((4 * k) << sh);
                if (inv) {
                    w1.y = -w1.y;
                    w2.y = -w2.y;
                    w4.y = -w4.y;
                }
                const float2 w3 = cmul(w1, w2);
                u[it][1] = cmul(u[it][1], w1);
                u[it][2] = cmul(u[it][2], w2);
                u[it][3] = cmul(u[it][3], w3);
                u[it][4] = cmul(u[it][4], w4);
                u[it][5] = cmul(u[it][5], cmul(w4, w1));
                u[it][6] = cmul(u[it][6], cmul(w4, w2));
                u[it][7] = cmul(u[it][7], cmul(w4, w3));
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = tw.get((r * k) << sh);
                    if (inv) w.y = -w.y;
                    u[it][r] = cmul(u[it][r], w);
                }
            }
        }
        dft_small<R>(u[it], inv);
        dst[it] = ((i - k) << LOGR) + k;  // row of output r = 0; output r is p rows further
        b_of[it] = b * bs;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
#pragma unroll
        for (int r = 0; r < R; ++r) buf[b_of[it] + sw(dst[it] + r * p) * es] = u[it][r];
    }
    __syncthreads();
}

// Full transform along one axis.  ET = elements per thread = nb*N/nthr (compile time); radix 8
// stages first, then one radix-4 or radix-2 stage for the remainder.
template <int ET, class TW, class SW = NoSwizzle>
UPPE_DEV void fft_axis_tw(float2* buf, int logN, int lognb, int bs, int es, const TW& tw, bool inv, int tid,
                          int nthr, int batch_fast_mode = -1, const SW& sw = SW{}) {
    // batch_fast_mode: -1 = automatic (batch-fast when es != 1), 0 = element-fast, 1 = batch-fast
    const bool batch_fast = (batch_fast_mode < 0) ? (es != 1) : (batch_fast_mode != 0);
    int logp = 0;
    while (logp < logN) {
        const int rem = logN - logp;
        if constexpr (ET >= 8) {
            if (rem >= 3) {
                stockham_stage<8, ET / 8>(buf, logN, logp, lognb, bs, es, tw, inv, batch_fast, tid, nthr, sw);
                logp += 3;
                continue;
            }
        }
        if constexpr (ET >= 4) {
            if (rem >= 2) {
                stockham_stage<4, ET / 4>(buf, logN, logp, lognb, bs, es, tw, inv, batch_fast, tid, nthr, sw);
                logp += 2;
                continue;
            }
        }
        if constexpr (ET >= 2) {
            stockham_stage<2, ET / 2>(buf, logN, logp, lognb, bs, es, tw, inv, batch_fast, tid, nthr, sw);
            logp += 1;
        } else {
            break;  // unreachable for valid launches (ET >= 2 whenever logN >= 1)
        }
    }
}

// Global-table form (twLog = log2 of the table size).
template <int ET>
UPPE_DEV void fft_axis(float2* buf, int logN, int lognb, int bs, int es, const float2* __restrict__ tw, int twLog,
                       bool inv, int tid, int nthr) {
    fft_axis_tw<ET>(buf, logN, lognb, bs, es, TwGlobal{tw, twLog}, inv, tid, nthr);
}

// ---------------------------------------------------------------------------------------------
// Compile-time form for batch-fast data (element e of transform b at buf[b + sw(e) * NB], NB = 2^LOGNB
// transforms of 2^LOGN points, NB * N / ET threads, sw the RowSwizzle of ct_row_swizzle): every
// stride, offset and twiddle shift is a constant, so a stage is its loads, twiddles, butterfly and
// stores.  Twiddles from a shared half table of 2^(TWLOG-1) entries of exp(-2 pi i j / 2^TWLOG).
// ---------------------------------------------------------------------------------------------
template <int TWLOG>
struct TwHalfSharedCT {
    const float2* p;
    UPPE_DEV float2 get(int j) const {
        constexpr int half = 1 << (TWLOG - 1);
        const float2 v = p[j & (half - 1)];
        return (j & half) ? make_float2(-v.x, -v.y) : v;
    }
};

template <int LOGN, int LOGNB>
UPPE_DEV constexpr RowSwizzle ct_row_swizzle() {
    return RowSwizzle{LOGNB <= 2 ? (1 << LOGN) - 1 : 0, LOGNB == 0 ? 4 : 3};
}

template <int R, int ITEMS, int LOGN, int LOGP, int LOGNB, int TWLOG>
UPPE_DEV void stockham_stage_ct(float2* buf, const TwHalfSharedCT<TWLOG>& tw, bool inv, int tid) {
    constexpr int LOGR = (R == 2) ? 1 : (R == 4) ? 2 : 3;
    constexpr int NQ = 1 << (LOGN - LOGR), P = 1 << LOGP, NB = 1 << LOGNB;
    constexpr int NTHR = (NB << LOGN) / (R * ITEMS);
    constexpr int SH = TWLOG - LOGP - LOGR;
    constexpr RowSwizzle sw = ct_row_swizzle<LOGN, LOGNB>();
    float2 u[ITEMS][R];
    int dst[ITEMS], bs[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
        const int g = tid + it * NTHR;
        const int b = g & (NB - 1);
        const int i = g >> LOGNB;
        const int k = i & (P - 1);
#pragma unroll
        for (int r = 0; r < R; ++r) u[it][r] = buf[b + sw(i + r * NQ) * NB];
        if constexpr (LOGP > 0) {
            if constexpr (R == 8) {
                float2 w1 = tw.get(k << SH), w2 = tw.get((2 * k) << SH), w4 = tw.get((4 * k) << SH);
                if (inv) {
                    w1.y = -w1.y;
                    w2.y = -w2.y;
                    w4.y = -w4.y;
                }
                const float2 w3 = cmul(w1, w2);
                u[it][1] = cmul(u[it][1], w1);
                u[it][2] = cmul(u[it][2], w2);
                u[it][3] = cmul(u[it][3], w3);
                u[it][4] = cmul(u[it][4], w4);
                u[it][5] = cmul(u[it][5], cmul(w4, w1));
                u[it][6] = cmul(u[it][6], cmul(w4, w2));
                u[it][7] = cmul(u[it][7], cmul(w4, w3));
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = tw.get((r * k) << SH);
                    if (inv) w.y = -w.y;
                    u[it][r] = cmul(u[it][r], w);
                }
            }
        }
        dft_small<R>(u[it], inv);
        dst[it] = ((i - k) << LOGR) + k;  // row of output r = 0; output r is P rows further
        bs[it] = b;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
#pragma unroll
        for (int r = 0; r < R; ++r) buf[bs[it] + sw(dst[it] + r * P) * NB] = u[it][r];
    }
    __syncthreads();
}

template <int ET, int LOGN, int LOGNB, int TWLOG, int LOGP = 0>
UPPE_DEV void fft_axis_ct(float2* buf, const TwHalfSharedCT<TWLOG>& tw, bool inv, int tid) {
    if constexpr (LOGP < LOGN) {
        constexpr int REM = LOGN - LOGP;
        if constexpr (ET >= 8 && REM >= 3) {
            stockham_stage_ct<8, ET / 8, LOGN, LOGP, LOGNB, TWLOG>(buf, tw, inv, tid);
            fft_axis_ct<ET, LOGN, LOGNB, TWLOG, LOGP + 3>(buf, tw, inv, tid);
        } else if constexpr (ET >= 4 && REM >= 2) {
            stockham_stage_ct<4, ET / 4, LOGN, LOGP, LOGNB, TWLOG>(buf, tw, inv, tid);
            fft_axis_ct<ET, LOGN, LOGNB, TWLOG, LOGP + 2>(buf, tw, inv, tid);
        } else {
            stockham_stage_ct<2, ET / 2, LOGN, LOGP, LOGNB, TWLOG>(buf, tw, inv, tid);
            fft_axis_ct<ET, LOGN, LOGNB, TWLOG, LOGP + 1>(buf, tw, inv, tid);
        }
    }
}
