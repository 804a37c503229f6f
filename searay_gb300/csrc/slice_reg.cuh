// Cartesian frequency-slice passes with register-resident transverse FFTs (kernel templates; each
// slice_reg_*.cu instantiates one kernel family over the supported shapes and launches it).
//
// One CTA owns one N1 x N2 frequency slice (N1, N2 in {16, 32, 64, 128}); each of its T = N1 N2 / 16
// threads holds 16 points of the slice in registers through the whole pass.  A length-N = 16 R axis
// transform is split N = 16 x R (R = N / 16 threads per line):
//
//   natural -> mixed (n2m):  thread j of a line holds x[j + R m], m = 0..15
//       16-point DFT over m in registers -> a;  twiddle W_N^(j a);
//       exchange within the R threads of the line (warp-private shared memory);
//       R-point DFTs over j -> thread j holds X[j + R s + 16 b] (s < 16/R, b < R)
//   mixed -> natural (m2n):  the same steps in reverse order (the receiving lane j applies the
//       twiddle W_N^(j a) after the exchange, so both directions use one per-thread twiddle set).
//
// A 2D transform is n2m along y (rows, the contiguous axis), one transpose through shared memory,
// n2m along x; the inverse mirrors it.  Per slice that is six shared-memory round trips and six
// block barriers (the exchanges within a line only need the warp), against fourteen round trips
// and two barriers per radix stage for the generic in-place Stockham form (fft_smem.cuh), which
// remains the path for other slice shapes.  The pointwise work (the RK stage, the propagator
// phase) runs on the registers between the forward and the inverse transform.
//
// Shared memory (float2 units): the transpose buffer F[x][ky] at x * (N2 + 2) + ky (a pitch of
// N2 + 2 makes the column reads conflict-free and the row writes two-way), and, over the same
// storage, a 544-element exchange region per warp, line l of the warp at l * 17 R and element
// (j, a) at j * 17 + a (conflict-free both ways).
#pragma once
#include <math.h>

#include "common.cuh"
#include "dft_reg.cuh"
#include "fft_smem.cuh"
#include "rk_stage.cuh"
#include "uppe_internal.h"

template <bool INV>
UPPE_DEV float2 tw_at(const TwGlobal& tw, int k, int sh) {
    float2 t = tw.get(k << sh);
    if (INV) t.y = -t.y;
    return t;
}

// v[a] *= W_N^(j a), a = 1..15, N = 2^LOGN: applied one bit of a at a time (W^j, W^2j, W^4j, W^8j
// from the table), so a single twiddle is live; each v[a] takes at most four products.
template <bool INV, int LOGN>
UPPE_DEV void twiddle_line(float2 (&v)[16], int j, const TwGlobal& tw) {
    const int sh = tw.log - LOGN;
#pragma unroll
    for (int bit = 1; bit < 16; bit <<= 1) {
        const float2 t = tw_at<INV>(tw, j * bit, sh);
#pragma unroll
        for (int a = 1; a < 16; ++a)
            if (a & bit) v[a] = cmul(v[a], t);
    }
}

// Synchronisation of the threads of one line around an exchange: the R2 threads of a row line are
// lanes of one warp; the R1 threads of a column line are lanes l and l + 16 of R1/2 warps, which
// meet at a named barrier when R1 >= 4.
template <bool NAMED>
struct LineSync {
    int id, count;
    UPPE_DEV void operator()() const {
        if constexpr (NAMED)
            asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
        else
            __syncwarp();
    }
};

// R-point DFT across the lanes of a line after the exchange (R = 2, 4, 8, 16)
template <int R, bool INV>
UPPE_DEV void dft_line(float2 (&u)[R]) {
    if constexpr (R == 16)
        dft16<INV>(u);
    else
        dft_small<R>(u, INV);
}

// natural -> mixed along one axis of length 16 R; `ex` is this line's exchange region, j the
// thread's index within the line.  v[m] = x[j + R m]  ->  w[s R + b] = X[j + R s + 16 b].
template <int R, int LOGN, bool INV, class SY>
UPPE_DEV void reg_n2m(float2 (&v)[16], float2 (&w)[16], float2* ex, int j, const TwGlobal& tw, const SY& sync) {
    dft16<INV>(v);
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) w[a] = v[a];
    } else {
        twiddle_line<INV, LOGN>(v, j, tw);
#pragma unroll
        for (int a = 0; a < 16; ++a) ex[j * 17 + a] = v[a];
        sync();
#pragma unroll
        for (int s = 0; s < 16 / R; ++s) {
            float2 u[R];
#pragma unroll
            for (int jj = 0; jj < R; ++jj) u[jj] = ex[jj * 17 + j + R * s];
            dft_line<R, INV>(u);
#pragma unroll
            for (int b = 0; b < R; ++b) w[s * R + b] = u[b];
        }
    }
}

// mixed -> natural along one axis: w[s R + b] = X[j + R s + 16 b]  ->  v[m] = x[j + R m].
template <int R, int LOGN, bool INV, class SY>
UPPE_DEV void reg_m2n(float2 (&w)[16], float2 (&v)[16], float2* ex, int j, const TwGlobal& tw, const SY& sync) {
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) v[a] = w[a];
    } else {
        sync();  // the line's last reads of this region are done
#pragma unroll
        for (int s = 0; s < 16 / R; ++s) {
            float2 u[R];
#pragma unroll
            for (int b = 0; b < R; ++b) u[b] = w[s * R + b];
            dft_line<R, INV>(u);
            const int a = j + R * s;
#pragma unroll
            for (int jj = 0; jj < R; ++jj) ex[jj * 17 + a] = u[jj];
        }
        sync();
#pragma unroll
        for (int a = 0; a < 16; ++a) v[a] = ex[j * 17 + a];
        twiddle_line<INV, LOGN>(v, j, tw);  // the receiving lane applies W^(j a)
    }
    dft16<INV>(v);
}

// Kinds and arguments of the column pass of the slices above 128 x 128 (slice_big.cu) and of the
// cluster-fused tail of 256 x 256 slices (slice_cluster.cu).
enum BigColKind {
    BC_FUSED = 0,    // forward column FFT, RK stage (SPEC_STAGE1/STAGE23/FINISH), next phase, inverse column FFT
    BC_SPEC = 1,     // forward column FFT, spectral update (SPEC_* modes)
    BC_REAL = 2,     // pointwise from q (REAL_* modes), inverse column FFT
    BC_ADJ_IN = 3,   // ADJ_S / ADJ_LOAD pointwise, inverse column FFT (unnormalised)
    BC_ADJ_FWD = 4,  // forward column FFT, ADJ_E / ADJ_FIN pointwise with 1/S
    BC_ADJ_STAGE = 5,  // forward column FFT, ADJ_E, the reverse RK bookkeeping and (mode 1) ADJ_S at z1,
                       // inverse column FFT (the column part of k_adj_fused_reg)
};

struct BigColArgs {
    int kind, mode;
    const float2* src;
    float2* dst;
    float2 *q_out, *qf;  // BC_ADJ_STAGE: qf = the accumulated cotangent
    const float2 *qi, *k1;  // BC_ADJ_STAGE: qi = lam_f
    float Cs, Ce;           // BC_ADJ_STAGE: a_f, a_mu
    StepArgs z0, z1;
    float2* q_store;  // BC_FUSED: also store each stage estimate here (when set)
};

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int LN1, int LN2>
struct RegSlice {
    static constexpr int N1 = 1 << LN1, N2 = 1 << LN2, S = N1 * N2, T = S / 16;
    static constexpr int R1 = N1 / 16, R2 = N2 / 16;
    static constexpr int P = N2 + 2;
    static constexpr int EXW = 544;
    static constexpr int NWARP = (T + 31) / 32;
    static constexpr int QC = 17 * R1 + 1;  // column line region pitch (odd: conflict-free)
    static constexpr int A1 = N1 * P > NWARP * EXW ? N1 * P : NWARP * EXW;
    static constexpr int SMEM = (A1 > N2 * QC ? A1 : N2 * QC) * (int)sizeof(float2);
    static constexpr bool COL_NAMED = R1 >= 4;
};

// Thread coordinates of both layouts.
//  * Row layout: line x (row), lane jr; tid = x R2 + jr, so a row's R2 threads share a warp.
//  * Column layout: line ky (column), lane ic; a warp holds 16 consecutive ky and two ic, so that
//    its global accesses in this layout are two 128-byte row segments (the pointwise operands, the
//    spectral outputs).  A column's R1 threads are lanes l, l + 16 of R1/2 warps.
// exr / exc: the thread's line region for the exchanges (element (j, a) at j * LW + a, LW = 17 for
// sixteen-value exchanges, 9 for eight-value halves): per warp for rows, per ky for columns.
template <class RS>
struct RegCoords {
    int x, jr, ky, ic;
    float2 *exr, *exc;
    LineSync<RS::COL_NAMED> csync;
    LineSync<false> rsync;
    UPPE_DEV RegCoords(float2* xb, int tid, bool half) {
        x = tid / RS::R2;
        jr = tid % RS::R2;
        constexpr int KB = RS::N2 / 16;
        if constexpr (RS::R1 == 1) {
            ky = tid;
            ic = 0;
            csync.id = 1;
        } else {
            const int warp = tid >> 5, lane = tid & 31;
            ky = (warp % KB) * 16 + (lane & 15);
            ic = (warp / KB) * 2 + (lane >> 4);
            csync.id = 1 + warp % KB;
        }
        csync.count = 32 * (RS::R1 / 2 > 0 ? RS::R1 / 2 : 1);
        rsync.id = 0;
        rsync.count = 0;
        const int lw = half ? 9 : 17;
        exr = xb + (tid >> 5) * (half ? 288 : 544) + ((tid & 31) / RS::R2) * lw * RS::R2;
        exc = xb + ky * (lw * RS::R1 + 1);
    }
};

// F[x][ky] from the row layout (w[s R2 + b] at ky = jr + R2 s + 16 b) to the column layout
// (v[m] at x = ic + R1 m).
template <class RS>
UPPE_DEV void rows_to_cols(const float2 (&w)[16], float2 (&v)[16], float2* sm, const RegCoords<RS>& c) {
    __syncthreads();  // exchange regions overlap the transpose buffer
#pragma unroll
    for (int s = 0; s < 16 / RS::R2; ++s)
#pragma unroll
        for (int b = 0; b < RS::R2; ++b) sm[c.x * RS::P + c.jr + RS::R2 * s + 16 * b] = w[s * RS::R2 + b];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = sm[(c.ic + RS::R1 * m) * RS::P + c.ky];
    __syncthreads();
}

template <class RS>
UPPE_DEV void cols_to_rows(const float2 (&v)[16], float2 (&w)[16], float2* sm, const RegCoords<RS>& c) {
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 16; ++m) sm[(c.ic + RS::R1 * m) * RS::P + c.ky] = v[m];
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 16 / RS::R2; ++s)
#pragma unroll
        for (int b = 0; b < RS::R2; ++b) w[s * RS::R2 + b] = sm[c.x * RS::P + c.jr + RS::R2 * s + 16 * b];
    __syncthreads();
}

// Forward 2D transform: rows loaded from `src` (natural layout) -> w in the column layout, mixed order.
template <class RS, int LN1, int LN2, bool INV>
UPPE_DEV void slice_fwd_from_global(const float2* __restrict__ src, float2 (&w)[16], float2* sm,
                                    const RegCoords<RS>& c, const TwGlobal& tw) {
    float2 v[16];
    const float2* p = src + (size_t)c.x * RS::N2 + c.jr;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = p[RS::R2 * m];
    reg_n2m<RS::R2, LN2, INV>(v, w, c.exr, c.jr, tw, c.rsync);
    rows_to_cols<RS>(w, v, sm, c);
    reg_n2m<RS::R1, LN1, INV>(v, w, c.exc, c.ic, tw, c.csync);
}

// Inverse 2D transform: w in the column layout, mixed order -> v in the row layout, natural order
// (v[m] at (x, jr + R2 m)).
template <class RS, int LN1, int LN2, bool INV>
UPPE_DEV void slice_inv_to_rows(float2 (&w)[16], float2 (&v)[16], float2* sm, const RegCoords<RS>& c,
                                const TwGlobal& tw) {
    reg_m2n<RS::R1, LN1, INV>(w, v, c.exc, c.ic, tw, c.csync);
    cols_to_rows<RS>(v, w, sm, c);
    reg_m2n<RS::R2, LN2, INV>(w, v, c.exr, c.jr, tw, c.rsync);
}

// linear index (within the slice) of register r of the column layout
template <class RS>
UPPE_DEV int col_elem(const RegCoords<RS>& c, int r) {
    const int s = r / RS::R1, b = r % RS::R1;
    return (c.ic + RS::R1 * s + 16 * b) * RS::N2 + c.ky;
}

// ---------------------------------------------------------------------------------------------
// Half-size exchanges for the persistent fused pass.  The line exchanges go through a 288-element
// region per warp (line l at l * 9 R, element (j, a') at j * 9 + a', a' < 8) in two halves of eight
// values; the transpose goes through an N1 x (N2/2 + 2) buffer in two phases, the diagonal
// quadrants (top bit of x equal to the top bit of ky) and then the others.  In both layouts the top
// bit of a thread's line (x or ky) is the top bit of its thread index, so each phase moves eight of
// every thread's sixteen values and the register footprint stays at sixteen.
// ---------------------------------------------------------------------------------------------
template <int R, int LOGN, bool INV, class SY>
UPPE_DEV void reg_n2m_h(float2 (&v)[16], float2 (&w)[16], float2* ex, int j, const TwGlobal& tw, const SY& sync) {
    dft16<INV>(v);
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) w[a] = v[a];
    } else {
        twiddle_line<INV, LOGN>(v, j, tw);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h) sync();  // the line's reads of the first half are done
#pragma unroll
            for (int ap = 0; ap < 8; ++ap) ex[j * 9 + ap] = v[8 * h + ap];
            sync();
#pragma unroll
            for (int s = 8 * h / R; s < (8 * h + 8) / R; ++s) {
                float2 u[R];
#pragma unroll
                for (int jj = 0; jj < R; ++jj) u[jj] = ex[jj * 9 + j + R * s - 8 * h];
                dft_line<R, INV>(u);
#pragma unroll
                for (int b = 0; b < R; ++b) w[s * R + b] = u[b];
            }
        }
    }
}

template <int R, int LOGN, bool INV, class SY>
UPPE_DEV void reg_m2n_h(float2 (&w)[16], float2 (&v)[16], float2* ex, int j, const TwGlobal& tw, const SY& sync) {
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) v[a] = w[a];
    } else {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            sync();  // the line's previous reads of this region are done
#pragma unroll
            for (int s = 8 * h / R; s < (8 * h + 8) / R; ++s) {
                float2 u[R];
#pragma unroll
                for (int b = 0; b < R; ++b) u[b] = w[s * R + b];
                dft_line<R, INV>(u);
                const int a = j + R * s;
#pragma unroll
                for (int jj = 0; jj < R; ++jj) ex[jj * 9 + a - 8 * h] = u[jj];
            }
            sync();
#pragma unroll
            for (int ap = 0; ap < 8; ++ap) v[8 * h + ap] = ex[j * 9 + ap];
        }
        twiddle_line<INV, LOGN>(v, j, tw);  // the receiving lane applies W^(j a)
    }
    dft16<INV>(v);
}

// Register pairs of the two layouts whose points differ only in the top bit of the transposed
// axis: row layout pair i = (lo, hi) with ky(hi) = ky(lo) + N2/2; column layout pair (i, i + 8)
// with x differing by N1/2.  A phase moves one member of every pair, chosen by the thread's top
// bit with selects, so every register index stays compile-time.
template <class RS>
UPPE_DEV void row_pair(int i, int& lo, int& hi) {
    if constexpr (RS::R2 >= 2) {
        constexpr int HB = RS::R2 / 2;
        const int s = i / HB, b = i % HB;
        lo = s * RS::R2 + b;
        hi = lo + HB;
    } else {
        lo = i;
        hi = i + 8;
    }
}
template <class RS>
UPPE_DEV int row_pair_ky(int i, int jr) {  // ky of the lo member, top bit clear
    if constexpr (RS::R2 >= 2) {
        constexpr int HB = RS::R2 / 2;
        return jr + RS::R2 * (i / HB) + 16 * (i % HB);
    } else {
        return i;
    }
}

template <class RS>
UPPE_DEV void rows_to_cols_h(float2 (&w)[16], float2 (&v)[16], float2* xb, const RegCoords<RS>& c) {
    constexpr int PH = RS::N2 / 2 + 2, HM = RS::N2 / 2 - 1;
    const int top = c.x >> (ilog2c(RS::N1) - 1);   // row role: top bit of x
    const int topc = c.ky >> (ilog2c(RS::N2) - 1);  // column role: top bit of ky
    const int cshift = topc * (RS::N1 / 2) * PH;  // column-side offset of the phase-0 half
    float2 snd1[8], rcv0[8];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) {  // phase 0: the diagonal quadrants (top bit of x == top bit of ky)
        int lo, hi;
        row_pair<RS>(i, lo, hi);
        xb[c.x * PH + (row_pair_ky<RS>(i, c.jr) & HM)] = top ? w[hi] : w[lo];
        snd1[i] = top ? w[lo] : w[hi];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) rcv0[i] = xb[(c.ic + RS::R1 * i) * PH + cshift + (c.ky & HM)];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) xb[c.x * PH + (row_pair_ky<RS>(i, c.jr) & HM)] = snd1[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 r1 = xb[(c.ic + RS::R1 * i) * PH + ((RS::N1 / 2) * PH - cshift) + (c.ky & HM)];
        v[i] = topc ? r1 : rcv0[i];
        v[i + 8] = topc ? rcv0[i] : r1;
    }
    __syncthreads();
}

template <class RS>
UPPE_DEV void cols_to_rows_h(float2 (&v)[16], float2 (&w)[16], float2* xb, const RegCoords<RS>& c) {
    constexpr int PH = RS::N2 / 2 + 2, HM = RS::N2 / 2 - 1;
    const int top = c.x >> (ilog2c(RS::N1) - 1);
    const int topc = c.ky >> (ilog2c(RS::N2) - 1);
    const int cshift = topc * (RS::N1 / 2) * PH;
    float2 snd1[8], rcv0[8];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        xb[(c.ic + RS::R1 * i) * PH + cshift + (c.ky & HM)] = topc ? v[i + 8] : v[i];
        snd1[i] = topc ? v[i] : v[i + 8];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) rcv0[i] = xb[c.x * PH + (row_pair_ky<RS>(i, c.jr) & HM)];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) xb[(c.ic + RS::R1 * i) * PH + ((RS::N1 / 2) * PH - cshift) + (c.ky & HM)] = snd1[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int lo, hi;
        row_pair<RS>(i, lo, hi);
        const float2 r1 = xb[c.x * PH + (row_pair_ky<RS>(i, c.jr) & HM)];
        w[lo] = top ? r1 : rcv0[i];
        w[hi] = top ? rcv0[i] : r1;
    }
    __syncthreads();
}

// Shared-memory plan of the persistent fused pass.
//  * staging buffer: the next slice's current, row pitch N2 + 8 (conflict-free row-layout reads);
//    during the pointwise phase a ring of NSLOT operand slots, slot r % NSLOT holding K, qi and qf
//    of register r of every thread (T points per array, in thread order);
//  * the half-size exchange buffer.
// All copies are 16-byte cp.async.cg, which go from L2 to shared memory without allocating in L1:
// beside 200+ KB of shared memory the L1 is small, and L1-allocating loads in flight are capped by
// its size.  A ring copy moves the points (kx, ky) and (kx, ky + 1) at once, for the thread with
// even ky and for its neighbour in the next lane; a __syncwarp after the wait publishes it.
template <int LN1, int LN2>
struct FusedPlan {
    using RS = RegSlice<LN1, LN2>;
    static constexpr int JP = RS::N2 + 8;
    static constexpr int JSTAGE = RS::N1 * JP;
    static constexpr int SLOT = 3 * RS::T;
    static constexpr int XT = RS::N1 * (RS::N2 / 2 + 2);
    static constexpr int XE = RS::NWARP * 288;
    static constexpr int XC = RS::N2 * (9 * RS::R1 + 1);
    static constexpr int XBUF = (XT > XE ? XT : XE) > XC ? (XT > XE ? XT : XE) : XC;
    static constexpr int NSLOT = (JSTAGE / SLOT) < 6 ? (JSTAGE / SLOT) : 6;
    static constexpr int SMEM = (JSTAGE + XBUF) * (int)sizeof(float2);
    static constexpr unsigned WMASK = RS::T >= 32 ? 0xffffffffu : ((1u << RS::T) - 1u);
    static_assert(NSLOT >= 2, "operand ring too small");
    static_assert(RS::N2 % 2 == 0 && (JP * 8) % 16 == 0, "16-byte copies");
};

UPPE_DEV void stage_async16(float2* smem_dst, const float2* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}

// ---------------------------------------------------------------------------------------------
// Fused evaluation tail (the same contract as the generic k_fused_cart): forward 2D FFT of J,
// S = (i/2) exp(-i(kz+kg) z) J / Re kz and the RK stage, then E for the next evaluation,
// E = IFFT2(i kz exp(i(kz+kg) z_next) qw)  (uppe.cl:22-52,73-108; uppe_kernel.py:210-213).
//
// Persistent: one CTA per multiprocessor walks the slices iw = blockIdx.x, + gridDim.x, ...  The
// next slice's current is copied into the staging buffer during this slice's inverse transform;
// the pointwise operands stream through the ring during the forward transform and the pointwise
// loop.
// ---------------------------------------------------------------------------------------------
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_fused_reg(int mode, const float2* __restrict__ J, OpView opv, float2* __restrict__ qi_out,
                float2* __restrict__ qf, const float2* __restrict__ qi, float2* __restrict__ E, float Cs, float Ce,
                const float2* __restrict__ tw, int twLog, StepArgs z_rhs, StepArgs z_next, int n0,
                float2* __restrict__ q_store) {
    using RS = RegSlice<LN1, LN2>;
    using FP = FusedPlan<LN1, LN2>;
    extern __shared__ __align__(16) float2 sm[];
    float2* jst = sm;
    float2* xb = sm + FP::JSTAGE;
    const int tid = threadIdx.x;
    const PhaseArgs pr{z_rhs.zhi, z_rhs.zlo, z_rhs.plain};
    const PhaseArgs pn{z_next.zhi, z_next.zlo, z_next.plain};
    const bool need_qi = (mode != SPEC_FINISH), need_qf = (mode != SPEC_STAGE1);

    // the current of slice iw -> staging buffer, 16-byte chunks, consecutive threads on consecutive chunks
    auto issue_J = [&](int iw) {
        const float2* src = J + (size_t)iw * RS::S;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int ch = tid + k * RS::T;  // chunk of two points
            const int x = ch / (RS::N2 / 2), y = 2 * (ch % (RS::N2 / 2));
            stage_async16(jst + x * FP::JP + y, src + x * RS::N2 + y);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    if ((int)blockIdx.x < n0) issue_J(blockIdx.x);

    for (int iw = blockIdx.x; iw < n0; iw += gridDim.x) {
        const size_t base = (size_t)iw * RS::S;
        // The twiddles and thread coordinates are the same for every slice; taking the thread index
        // and the table address through asm here keeps the compiler from hoisting them out of the
        // slice loop into registers.
        int tl;
        const float2* twl;
        asm volatile("mov.u32 %0, %%tid.x;" : "=r"(tl));
        asm volatile("mov.b64 %0, %1;" : "=l"(twl) : "l"(tw));
        const TwGlobal twg{twl, twLog};
        const RegCoords<RS> c(xb, tl, true);
        // ring position of this thread: thread order; the pair (ky even, ky + 1) are adjacent lanes
        const int rpos = tl;
        const bool copier = (c.ky & 1) == 0;
        float2 w[16], v[16];

        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = jst[c.x * FP::JP + c.jr + RS::R2 * m];
        __syncthreads();  // staging buffer free: operand ring

        auto issue = [&](int r) {
            if (r < 16 && copier) {
                const size_t idx = base + col_elem(c, r);  // even ky: idx, idx + 1 are 16-byte aligned
                float2* slot = jst + (r % FP::NSLOT) * FP::SLOT + rpos;
                stage_async16(slot, opv.K + idx);
                if (need_qi) stage_async16(slot + RS::T, qi + idx);
                if (need_qf) stage_async16(slot + 2 * RS::T, qf + idx);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");  // empty groups keep the count uniform
        };
#pragma unroll
        for (int r = 0; r < FP::NSLOT; ++r) issue(r);

        reg_n2m_h<RS::R2, LN2, false>(v, w, c.exr, c.jr, twg, c.rsync);
        rows_to_cols_h<RS>(w, v, xb, c);
        reg_n2m_h<RS::R1, LN1, false>(v, w, c.exc, c.ic, twg, c.csync);

        const float cond = (iw < 4) ? 0.f : 1.f;
        const float2 kgw = opv.kg[iw];
        // Two registers per trip, then the register array rotates by two, so the loop body exists
        // once in the code rather than sixteen times (the fully unrolled form thrashed the
        // instruction cache); after eight trips w is back in order.
#pragma unroll 1
        for (int r0 = 0; r0 < 16; r0 += 2) {
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const int r = r0 + d;
                asm volatile("cp.async.wait_group %0;\n" ::"n"(FP::NSLOT - 1) : "memory");
                __syncwarp(FP::WMASK);  // the copying lane's data is visible to its neighbour
                const size_t idx = base + col_elem(c, r);
                const float2* slot = jst + (r % FP::NSLOT) * FP::SLOT + rpos;
                const float2 K = slot[0];
                const float2 qiv = need_qi ? slot[RS::T] : make_float2(0.f, 0.f);
                const float2 qfv = need_qf ? slot[2 * RS::T] : make_float2(0.f, 0.f);
                OpPoint o;
                o.Khi = K.x;
                o.Klo = K.y;
                o.kzr = (K.x - kgw.x) + (K.y - kgw.y);
                o.kzi = opv.ki ? opv.ki[idx] : 0.f;
                // S and the RK stage (the arithmetic of spec_update, on staged values)
                const float2 f = propagator_factor(o, pr, -1.f);
                const float2 sv = cscale(cmul_i(cmul(f, w[d])), 0.5f / o.kzr);
                float2 qw;
                if (mode == SPEC_STAGE1) {
                    qf[idx] = cadd(qiv, cscale(sv, Cs));
                    qw = cscale(cadd(qiv, cscale(sv, Ce)), cond);
                    if (q_store) q_store[idx] = qw;
                } else if (mode == SPEC_STAGE23) {
                    qf[idx] = cadd(qfv, cscale(sv, Cs));
                    qw = cscale(cadd(qiv, cscale(sv, Ce)), cond);
                    if (q_store) q_store[idx] = qw;
                } else {
                    qw = cscale(cadd(qfv, cscale(sv, Cs)), cond);
                    qi_out[idx] = qw;
                }
                w[d] = cmul(op_ikz(o), cmul(propagator_factor(o, pn, 1.f), qw));
                __syncwarp(FP::WMASK);  // both lanes of the pair have read the slot before it is refilled
                issue(r + FP::NSLOT);
            }
            const float2 t0 = w[0], t1 = w[1];
#pragma unroll
            for (int i = 0; i < 14; ++i) w[i] = w[i + 2];
            w[14] = t0;
            w[15] = t1;
        }
        __syncthreads();  // every ring slot has been read: the staging buffer takes the next current
        if (iw + (int)gridDim.x < n0) issue_J(iw + gridDim.x);

        reg_m2n_h<RS::R1, LN1, true>(w, v, c.exc, c.ic, twg, c.csync);
        cols_to_rows_h<RS>(v, w, xb, c);
        reg_m2n_h<RS::R2, LN2, true>(w, v, c.exr, c.jr, twg, c.rsync);
        float2* dst = E + base + (size_t)c.x * RS::N2 + c.jr;
        constexpr float scale = 1.0f / (float)RS::S;
#pragma unroll
        for (int m = 0; m < 16; ++m) dst[RS::R2 * m] = cscale(v[m], scale);
    }
}

// Inverse transverse transform (modes of k_real_cart): E = IFFT2(i kz e^{..} q), the finish form
// A = IFFT2(e^{..} q), E = i kz A, or the first RK stage from k1 followed by E.
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_real_reg(int mode, const float2* __restrict__ src, OpView opv, float2* __restrict__ E,
               float2* __restrict__ A_out, const float2* __restrict__ k1, float2* __restrict__ qf, float Cs, float Ce,
               const float2* __restrict__ tw, int twLog, StepArgs z, int iw0, float2* __restrict__ q_store) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x + iw0;
    const size_t base = (size_t)iw * RS::S;
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid, false);
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float2 kgw = opv.kg[iw];
    const float cond = (iw < 4) ? 0.f : 1.f;
    float2 w[16], v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const size_t idx = base + col_elem(c, r);
        const OpPoint o = op_at(opv, idx, kgw);
        float2 val;
        if (mode == REAL_APPLY1) {
            const float2 a = src[idx], s = k1[idx];
            qf[idx] = cadd(a, cscale(s, Cs));
            val = cscale(cadd(a, cscale(s, Ce)), cond);
        } else if (mode >= REAL_ZS1) {  // src: qi (stages 1-3) or qf (finish); qf: the array written
            const float2 a = src[idx];
            val = cscale(a, cond);
            if (mode == REAL_ZS1) qf[idx] = a;
            if (mode == REAL_ZSF) qf[idx] = val;
            if (mode != REAL_ZSF && q_store) q_store[idx] = val;
        } else {
            val = src[idx];
        }
        val = cmul(propagator_factor(o, pa, 1.f), val);
        if (mode != REAL_FINISH) val = cmul(op_ikz(o), val);
        w[r] = val;
    }
    slice_inv_to_rows<RS, LN1, LN2, true>(w, v, sm, c, twg);
    constexpr float scale = 1.0f / (float)RS::S;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const size_t e = base + (size_t)c.x * RS::N2 + c.jr + RS::R2 * m;
        const float2 val = cscale(v[m], scale);
        if (mode != REAL_FINISH) {
            E[e] = val;
        } else {
            if (A_out) A_out[e] = val;
            const OpPoint o = op_at(opv, e, kgw);
            E[e] = cmul(op_ikz(o), val);
        }
    }
}

// Forward transverse transform and the spectral update (modes of k_spec_cart).
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_spec_reg(int mode, const float2* __restrict__ src, OpView opv, float2* __restrict__ q_out,
               float2* __restrict__ qf, const float2* __restrict__ qi, float Cs, float Ce,
               const float2* __restrict__ tw, int twLog, StepArgs z) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x;
    const size_t base = (size_t)iw * RS::S;
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid, false);
    float2 w[16];
    slice_fwd_from_global<RS, LN1, LN2, false>(src + base, w, sm, c, twg);
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float cond = (iw < 4) ? 0.f : 1.f;
    const float2 kgw = (mode == SPEC_LOAD) ? make_float2(0.f, 0.f) : opv.kg[iw];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const size_t idx = base + col_elem(c, r);
        OpPoint o;
        if (mode != SPEC_LOAD) o = op_at(opv, idx, kgw);
        spec_update(mode, idx, w[r], o, cond, q_out, qf, qi, Cs, Ce, pa, true);
    }
}

// Vector-Jacobian products of the slice transforms (modes of k_adj_cart).
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_adj_reg(int mode, const float2* __restrict__ in, OpView opv, float2* __restrict__ out,
              const float2* __restrict__ tw, int twLog, StepArgs z) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x;
    const size_t base = (size_t)iw * RS::S;
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid, false);
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float2 kgw = opv.kg[iw];
    float2 w[16], v[16];
    if (mode == ADJ_S || mode == ADJ_LOAD) {
        // k-space cotangent -> F^H (unnormalised inverse transform)
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const size_t idx = base + col_elem(c, r);
            float2 val = in[idx];
            if (mode == ADJ_S) {
                const OpPoint o = op_at(opv, idx, kgw);
                // conj(D2) = (-i/2) conj(exp(-iKz) exp(Ki z)) / Re kz
                const float2 f = cconj(propagator_factor(o, pa, -1.f));
                val = cscale(cmul_mi(cmul(f, val)), 0.5f / o.kzr);
            }
            w[r] = val;
        }
        slice_inv_to_rows<RS, LN1, LN2, true>(w, v, sm, c, twg);
        float2* dst = out + base + (size_t)c.x * RS::N2 + c.jr;
#pragma unroll
        for (int m = 0; m < 16; ++m) dst[RS::R2 * m] = v[m];
    } else {
        slice_fwd_from_global<RS, LN1, LN2, false>(in + base, w, sm, c, twg);
        constexpr float scale = 1.0f / (float)RS::S;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const size_t idx = base + col_elem(c, r);
            const OpPoint o = op_at(opv, idx, kgw);
            float2 val = cmul(cconj(propagator_factor(o, pa, 1.f)), cscale(w[r], scale));
            if (mode == ADJ_E) val = cmul(cconj(op_ikz(o)), val);
            out[idx] = val;
        }
    }
}

// The end of one stage of the reverse RK4 sweep fused with the start of the next (the kernels
// k_adj_reg ADJ_E, k_adj_rk and k_adj_reg ADJ_S in one pass over a slice):
//   mu = conj(D0) (1/N) F g  at z_e (the cotangent of q from the cotangent g of E),
//   mode 1: cm = cond mu, acc += cm, lam_k = a_f lam_f + a_mu cm, out = F^H( conj(D2) lam_k ) at z_s
//           (the cotangent of J for the next stage's time pass);
//   mode 2: lam_in = acc + mu (the cotangent of the step's input, written to out).
// mu and lam_k stay in registers.
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_adj_fused_reg(int mode, const float2* __restrict__ g, OpView opv, const float2* __restrict__ lam_f,
                    float2* __restrict__ acc, float2* __restrict__ out, float a_f, float a_mu,
                    const float2* __restrict__ tw, int twLog, StepArgs z_e, StepArgs z_s) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x;
    const size_t base = (size_t)iw * RS::S;
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid, false);
    const PhaseArgs pe{z_e.zhi, z_e.zlo, z_e.plain};
    const PhaseArgs ps{z_s.zhi, z_s.zlo, z_s.plain};
    const float2 kgw = opv.kg[iw];
    const float cond = (iw < opv.ncond) ? 0.f : 1.f;
    // the pointwise operands of this thread's 16 points are asked into L2 while the forward slice
    // transform runs, so that their loads after it find them there
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const size_t idx = base + col_elem(c, r);
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(opv.K + idx));
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(acc + idx));
        if (mode != 2) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(lam_f + idx));
    }
    float2 w[16], v[16];
    slice_fwd_from_global<RS, LN1, LN2, false>(g + base, w, sm, c, twg);
    constexpr float scale = 1.0f / (float)RS::S;
    // The operands of two points are loaded before any store of those points: the operator's
    // pointers live in a struct, so the compiler must assume a store to acc or out may alias the next
    // point's loads, which otherwise puts every point behind a full memory latency.
#pragma unroll
    for (int r4 = 0; r4 < 16; r4 += 2) {
        float2 K4[2], A4[2], L4[2];
        float ki4[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const size_t idx = base + col_elem(c, r4 + j);
            K4[j] = opv.K[idx];
            ki4[j] = opv.ki ? opv.ki[idx] : 0.f;
            A4[j] = acc[idx];
            L4[j] = (mode == 2) ? make_float2(0.f, 0.f) : lam_f[idx];
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int r = r4 + j;
            const size_t idx = base + col_elem(c, r);
            OpPoint o;
            o.Khi = K4[j].x;
            o.Klo = K4[j].y;
            o.kzr = opv.envelope ? kgw.x : (K4[j].x - kgw.x) + (K4[j].y - kgw.y);
            o.kzi = ki4[j];
            const float2 mu = cmul(cconj(op_ikz(o)), cmul(cconj(propagator_factor(o, pe, 1.f)), cscale(w[r], scale)));
            if (mode == 2) {
                out[idx] = cadd(A4[j], mu);
            } else {
                const float2 cm = cscale(mu, cond);
                acc[idx] = cadd(A4[j], cm);
                const float2 lk = cadd(cscale(L4[j], a_f), cscale(cm, a_mu));
                const float2 f = cconj(propagator_factor(o, ps, -1.f));
                w[r] = cscale(cmul_mi(cmul(f, lk)), 0.5f / o.kzr);
            }
        }
    }
    if (mode == 2) return;
    slice_inv_to_rows<RS, LN1, LN2, true>(w, v, sm, c, twg);
    float2* dst = out + base + (size_t)c.x * RS::N2 + c.jr;
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[RS::R2 * m] = v[m];
}

// Supported shapes (log2 N1, log2 N2).
#define UPPE_REG_SHAPES(X) \
    X(4, 4) X(4, 5) X(4, 6) X(4, 7) X(5, 4) X(5, 5) X(5, 6) X(5, 7) X(6, 4) X(6, 5) X(6, 6) X(6, 7) X(7, 4) X(7, 5) X(7, 6) X(7, 7)

// Calls F<LN1, LN2>::run(args...) for the handle's slice shape.
template <template <int, int> class F, class... A>
static cudaError_t reg_dispatch(UppeHandle* h, A&&... args) {
    const int l1 = ilog2_exact(h->N1), l2 = ilog2_exact(h->N2);
    h->launches++;
#define UPPE_REG_CASE(A_, B_) \
    if (l1 == A_ && l2 == B_) return F<A_, B_>::run(h, args...);
    UPPE_REG_SHAPES(UPPE_REG_CASE)
#undef UPPE_REG_CASE
    return cudaErrorInvalidValue;
}

