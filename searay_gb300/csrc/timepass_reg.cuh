// Shapes and per-column transforms of the register-resident time-axis passes (timepass_reg.cu:
// the forward pass k_time_reg; timepass_adj_reg.cu: its vector-Jacobian product k_time_adj_reg).
//
// Per column, with k = t + TC a (frequency) and m = b + R1 c (time, packed pairs):
//   F layout (frequency): lane t holds Z[t + TC a], a < R1 = M / TC;
//   T layout (time):      lane t holds z[b + R1 c] for b = t + TC j (j < NB = R1 / TC), c < TC.
// The inverse transform is the four-step split W_M^(-(t + TC a)(b + R1 c)) = W_R1^(-a b)
// W_M^(-t b) W_TC^(-t c); the forward transform is its mirror image (T layout in, F layout out).
#pragma once

#include "common.cuh"
#include "dft_reg.cuh"

template <int LOGM>
struct TRegShape;
// TC lanes per column, R1 complex values per lane, NC columns per 256-thread block, MINB blocks per
// multiprocessor (the register budget: 128 registers at 2, 80 at 3).
template <>
struct TRegShape<8> {
    static constexpr int TC = 16, R1 = 16, NC = 16, MINB = 2;
};
template <>
struct TRegShape<9> {
    static constexpr int TC = 32, R1 = 16, NC = 8, MINB = 3;
};
template <>
struct TRegShape<10> {
    static constexpr int TC = 32, R1 = 32, NC = 8, MINB = 2;
};


__host__ __device__ constexpr int tr_max(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int tr_log2(int n) { return n <= 1 ? 0 : 1 + tr_log2(n / 2); }

template <int LOGM>
struct TReg {
    static constexpr int M = 1 << LOGM, NT = 2 * M;
    static constexpr int TC = TRegShape<LOGM>::TC, R1 = TRegShape<LOGM>::R1, NC = TRegShape<LOGM>::NC;
    // H = 1: R1 = NB TC, lane t holds the time lines b = t + TC j; H = 2: TC = 2 R1, the lane pair
    // (b, h = 0, 1) shares line b (the TC-point DFT over c split into a radix-2 step across the pair)
    static constexpr int H = TC > R1 ? TC / R1 : 1;
    static constexpr int NB = TC > R1 ? 1 : R1 / TC;
    static constexpr int MINB = TRegShape<LOGM>::MINB;
    static constexpr int THREADS = NC * TC;
    static constexpr int SEG = M / TC;  // packed pairs per lane in the contiguous (scan) layout
    static constexpr int LSEG = tr_log2(SEG);
    // column buffer: staged half spectrum (M + 1), exchange 1 (R1 rows of TC + 1), exchange 2 (TC
    // rows of R1 + 1), the padded natural-order scan array (M + M / SEG).  Its pitch sets the banks of
    // the staging and output accesses, where a half-warp touches 16 / NC rows of NC columns: odd for
    // NC = 16, 2 mod 16 (in float2 units) for NC = 8, so those 16 accesses fall on distinct banks.
    static constexpr int LD0 = tr_max(tr_max(M + 1, R1 * (TC + 1)), tr_max(TC * (R1 + 1), M + M / SEG));
    static constexpr int LD = (NC == 16) ? (LD0 | 1) : ((LD0 + 13) / 16) * 16 + 2;
    static constexpr size_t SMEM = (size_t)NC * LD * sizeof(float2);
    static_assert((H == 1 ? NB * TC == R1 : (H == 2 && 2 * R1 == TC && R1 == 16)) && THREADS == 256 &&
                      (NC == 16 || NC == 8) && LD >= LD0,
                  "time-pass shape");
    // T layout: the time pair m held in register r of lane t
    static UPPE_DEV int tm(int t, int r) {
        if constexpr (H == 1)
            return t + TC * (r / TC) + R1 * (r % TC);
        else
            return (t % R1) + R1 * (R1 * (t / R1) + r);
    }
};

// The radix-2 step of a 32-point DFT split over a lane pair (lanes t and t ^ 16 hold the two
// halves of one line): W32^C constants per register, C = 0 .. 15.
template <int C, bool INV>
UPPE_DEV void tr_pair_inverse(float2 (&v)[16], bool h) {
    if constexpr (C < 16) {
        // z[c] = E0[c] + W32^-c E1[c], z[c + 16] = E0[c] - W32^-c E1[c]: lane h = 0 keeps the first
        const float2 p = make_float2(__shfl_xor_sync(0xffffffffu, v[C].x, 16), __shfl_xor_sync(0xffffffffu, v[C].y, 16));
        const float2 e = h ? p : v[C];
        const float2 o = mul_w32<C, INV>(h ? v[C] : p);
        v[C] = h ? csub(e, o) : cadd(e, o);
        tr_pair_inverse<C + 1, INV>(v, h);
    }
}
template <int C>
UPPE_DEV void tr_pair_forward(float2 (&v)[16], bool h) {
    if constexpr (C < 16) {
        // even outputs from x0 + x1 (lane h = 0), odd ones from (x0 - x1) W32^c (lane h = 1)
        const float2 p = make_float2(__shfl_xor_sync(0xffffffffu, v[C].x, 16), __shfl_xor_sync(0xffffffffu, v[C].y, 16));
        v[C] = h ? mul_w32<C, false>(csub(p, v[C])) : cadd(v[C], p);
        tr_pair_forward<C + 1>(v, h);
    }
}

// natural pair index m -> padded position in the column buffer (a pad after every SEG pairs keeps
// both the lane-consecutive and the segment-strided accesses conflict-free)
template <int LSEG>
UPPE_DEV int tr_pad(int m) {
    return m + (m >> LSEG);
}

template <int LOGM>
UPPE_DEV void tr_forward_lines(float2 (&v)[TReg<LOGM>::R1], float2* buf, const float2* __restrict__ twF, int t);

// Forward transform of the packed sequence in the T layout (v[j TC + c] = z[t + TC j + R1 c]) into
// the F layout (v[a] = Z[t + TC a]); buf is the column's buffer, twF the forward twiddles.
template <int LOGM>
UPPE_DEV void tr_forward(float2 (&v)[TReg<LOGM>::R1], float2* buf, const float2* __restrict__ twF, int t) {
    using G = TReg<LOGM>;
    if constexpr (G::H == 2) {
        // lane t = b + R1 h holds z[b + R1 (R1 h + c)]: radix-2 across the pair, R1-point DFT over c,
        // giving Y_b[k1] for k1 = 2 i + h; then W_M^(b k1) (twF[i TC + t])
        const int b = t % G::R1;
        const bool h = t >= G::R1;
        tr_pair_forward<0>(v, h);
        dft_at<G::R1, 0, false>(v);
#pragma unroll
        for (int i = 0; i < G::R1; ++i) v[i] = cmul(v[i], __ldg(&twF[i * G::TC + t]));
        __syncwarp();  // the column's earlier reads of buf are done
#pragma unroll
        for (int i = 0; i < G::R1; ++i) buf[(2 * i + (h ? 1 : 0)) * (G::R1 + 1) + b] = v[i];
        __syncwarp();
        // lane t = k1 takes every b; R1-point DFT over b -> k2: Z[t + TC k2]
#pragma unroll
        for (int bb = 0; bb < G::R1; ++bb) v[bb] = buf[t * (G::R1 + 1) + bb];
        dft_at<G::R1, 0, false>(v);
    } else {
        tr_forward_lines<LOGM>(v, buf, twF, t);
    }
}

// tr_forward for H = 1: lane t holds whole time lines.
template <int LOGM>
UPPE_DEV void tr_forward_lines(float2 (&v)[TReg<LOGM>::R1], float2* buf, const float2* __restrict__ twF, int t) {
    using G = TReg<LOGM>;
    // stage 1: TC-point DFTs over c -> k1, then W_M^(b k1), b = t + TC j
    dft_at<G::TC, 0, false>(v);
    if constexpr (G::NB == 2) dft_at<G::TC, G::TC, false>(v);
#pragma unroll
    for (int j = 0; j < G::NB; ++j)
#pragma unroll
        for (int k1 = 1; k1 < G::TC; ++k1)
            v[j * G::TC + k1] = cmul(v[j * G::TC + k1], __ldg(&twF[(j * G::TC + k1) * G::TC + t]));
    __syncwarp();  // the column's earlier reads of buf are done
#pragma unroll
    for (int j = 0; j < G::NB; ++j)
#pragma unroll
        for (int k1 = 0; k1 < G::TC; ++k1) buf[k1 * (G::R1 + 1) + t + G::TC * j] = v[j * G::TC + k1];
    __syncwarp();
    // stage 2: lane t = k1 takes every b; R1-point DFT over b -> k2: Z[t + TC k2]
#pragma unroll
    for (int b = 0; b < G::R1; ++b) v[b] = buf[t * (G::R1 + 1) + b];
    dft_at<G::R1, 0, false>(v);
}

// Real spectrum of the packed signal from the F layout (the partner value Z[(M - k) mod M] comes
// from lane (TC - t) mod TC of the column, register R1 - 1 - a; lane 0 pairs a with (R1 - a) mod R1
// in its own registers), passed to emit(k, X[k]) for every k of this lane (and k = M by lane 0).
template <int LOGM, class Emit>
UPPE_DEV void tr_unpack(const float2 (&v)[TReg<LOGM>::R1], const float2* __restrict__ twP, int t, int lane,
                        Emit emit) {
    using G = TReg<LOGM>;
    const int partner = (lane & ~(G::TC - 1)) | ((G::TC - t) & (G::TC - 1));
#pragma unroll
    for (int a = 0; a < G::R1; ++a) {
        const float2 send = v[G::R1 - 1 - a];
        float2 got;
        got.x = __shfl_sync(0xffffffffu, send.x, partner);
        got.y = __shfl_sync(0xffffffffu, send.y, partner);
        if (t == 0) got = v[(G::R1 - a) & (G::R1 - 1)];
        const float2 twk = __ldg(&twP[a * G::TC + t]);  // e^{-2 pi i k / Nt}
        // X[k] = (Za + conj Zb)/2 - (i/2) e^{-2 pi i k/Nt} (Za - conj Zb)
        const float2 Zb = cconj(got);
        const float2 s = cadd(v[a], Zb);
        const float2 d = cmul(twk, csub(v[a], Zb));
        emit(t + G::TC * a, cscale(csub(s, cmul_i(d)), 0.5f));
    }
    if (t == 0) {  // Nyquist: X[M] = Re Z[0] - Im Z[0]
        emit(G::M, make_float2(v[0].x - v[0].y, 0.f));
    }
}


// Even/odd packing of the half spectrum X(k), k in [0, M] (xk(k) gives X[k]; its imaginary parts
// at k = 0 and M do not enter irfft), into the F layout, then the inverse transform into the T
// layout: v[j TC + c] = z[t + TC j + R1 c] with z[m] = Nt (x(2m) + i x(2m+1)) of x = irfft(X).
// xk reads the column's staged spectrum from buf; every read is done before buf serves the exchange.
// Inverse transform from the F layout (v[a] = Z[t + TC a]) into the T layout; every earlier read of
// buf by the column is done before buf serves the exchange.
template <int LOGM>
UPPE_DEV void tr_inverse(float2 (&v)[TReg<LOGM>::R1], float2* buf, const float2* __restrict__ twI, int t) {
    using G = TReg<LOGM>;
    constexpr int TC = G::TC, R1 = G::R1, NB = G::NB;
    // R1-point DFT over a, twiddle, exchange, TC-point DFTs over t
    dft_at<R1, 0, true>(v);
#pragma unroll
    for (int b = 1; b < R1; ++b) v[b] = cmul(v[b], cconj(__ldg(&twI[b * TC + t])));
    __syncwarp();  // the packing reads of buf are done
#pragma unroll
    for (int b = 0; b < R1; ++b) buf[b * (TC + 1) + t] = v[b];
    __syncwarp();
    if constexpr (G::H == 2) {
        // lane b + R1 h: the R1-point DFT of line b over the lanes t = h + 2 i, then the radix-2 step
        // across the pair: v[c] = z[b + R1 (R1 h + c)]
        const int b = t % R1;
        const bool h = t >= R1;
#pragma unroll
        for (int i = 0; i < R1; ++i) v[i] = buf[b * (TC + 1) + (h ? 1 : 0) + 2 * i];
        dft_at<R1, 0, true>(v);
        tr_pair_inverse<0, true>(v, h);
    } else {
#pragma unroll
        for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int tt = 0; tt < TC; ++tt) v[j * TC + tt] = buf[(t + TC * j) * (TC + 1) + tt];
        dft_at<TC, 0, true>(v);
        if constexpr (NB == 2) dft_at<TC, TC, true>(v);
    }
}

template <int LOGM, class XK>
UPPE_DEV void tr_pack_inverse(float2 (&v)[TReg<LOGM>::R1], float2* buf, const float2* __restrict__ twI,
                              const float2* __restrict__ twP, int t, XK xk) {
    using G = TReg<LOGM>;
    constexpr int TC = G::TC, R1 = G::R1, M = G::M;
    // Z[k] = (X[k] + conj X[M-k]) + i e^{2 pi i k/Nt} (X[k] - conj X[M-k])
#pragma unroll
    for (int a = 0; a < R1; ++a) {
        const int k = t + TC * a;
        float2 Xa = xk(k);
        float2 Xm = xk(M - k);
        if (a == 0 && t == 0) {
            Xa.y = 0.f;
            Xm.y = 0.f;
        }
        const float2 tk = cconj(__ldg(&twP[a * TC + t]));  // e^{+2 pi i k / Nt}
        const float2 b = cconj(Xm);
        v[a] = cadd(cadd(Xa, b), cmul_i(cmul(tk, csub(Xa, b))));
    }
    tr_inverse<LOGM>(v, buf, twI, t);
}
