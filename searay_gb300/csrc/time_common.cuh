// Device pieces shared by the UPPE time pass (timepass.cu) and the paraxial envelope time pass
// (envelope.cu): rate models, the density scan helpers, the block-wide segment sums, packed f32x2
// arithmetic and the rotational Raman pass.
#pragma once
#include <math.h>

#include "common.cuh"
#include "uppe_internal.h"

struct TimeParams {
    int Nt, logNt, M, logM, C, logC, S, spt;
    float inv_nt, hdt, redchi3, damping;
    int rate_form;
    float fconv, cutoff;
    float y0, ypow, yexp;  // explicit form: rate = 2^(y0 + ypow log2(Em) + yexp / Em)
    float lrc2;            // series form: log2(rate_conv)
    float c2[6];           // series form: log2(e) * c_i, polynomial in L = ln(Em)
    float em_min;          // below this Em the rate is below FP32's smallest normal (taken as 0)
    int wcut, wwid, plain;
    int cut_on, cut_off;   // NL filter: J is kept for cut_on <= k < cut_off (uppe_kernel.py:122-125)
    // rotational Raman: transitions in pairs, 20 float4 per pair (constants and powers of h^2) and
    // the phasor table p0[pair][segment] (raman_pass)
    int rot_pairs;
    const float4* rot_tab;
    const float4* rot_p0;
    // TIME_J with atc set: J goes straight into the split operand tiles of the forward tensor-core
    // Hankel transform (hankel_tc.cuh, azimuthal mode 0) instead of out0
    uint8_t* atc;
    int atc_nwt, atc_nkt;
};

#define UPPE_LN2 0.69314718055994530942f

// Ionization rate in simulation units from the field in simulation units.
__device__ __forceinline__ float ion_rate(const TimeParams& tp, float e) {
    const float em = fmaf(tp.fconv, fabsf(e), tp.cutoff);
    if (em < tp.em_min) return 0.f;
    const float l2 = __log2f(em);
    if (tp.rate_form == UPPE_RATE_EXPLICIT) {
        return exp2f(fmaf(tp.ypow, l2, fmaf(tp.yexp, __frcp_rn(em), tp.y0)));
    }
    const float L = l2 * UPPE_LN2;
    float p = tp.c2[5];
    p = fmaf(p, L, tp.c2[4]);
    p = fmaf(p, L, tp.c2[3]);
    p = fmaf(p, L, tp.c2[2]);
    p = fmaf(p, L, tp.c2[1]);
    p = fmaf(p, L, tp.c2[0]);
    return exp2f(tp.lrc2 + p);
}

__device__ __forceinline__ float smooth5(float q) { return q * q * q * (10.f - 15.f * q + 6.f * q * q); }

__device__ __forceinline__ float soft_window(int i, int Ni, int cut, int wid) {
    float f = 1.f;
    if (i < cut || i > Ni - cut - 1) f = 0.f;
    if (i >= cut && i < cut + wid) f *= smooth5((float)(i - cut) / (float)wid);
    if (i <= Ni - cut - 1 && i > Ni - cut - wid - 1) f *= smooth5((float)(Ni - cut - 1 - i) / (float)wid);
    return f;
}

// 1 - exp(-S) for S >= 0: the Taylor series of -expm1(-S) through S^8 (truncation below 1e-11
// relative) for S < 1/4, where 1 - exp(-S) would cancel, and 1 - expf(-S) above.
__device__ __forceinline__ float one_minus_exp_neg(float S) {
    if (S == 0.f) return 0.f;
    if (S < 0.25f) {
        const float x = -S;
        float p = 1.f / 40320.f;
        p = fmaf(p, x, 1.f / 5040.f);
        p = fmaf(p, x, 1.f / 720.f);
        p = fmaf(p, x, 1.f / 120.f);
        p = fmaf(p, x, 1.f / 24.f);
        p = fmaf(p, x, 1.f / 6.f);
        p = fmaf(p, x, 0.5f);
        p = fmaf(p, x, 1.f);
        return -x * p;
    }
    return 1.f - expf(-S);
}

__device__ __forceinline__ void acc_add(ffloat& s, float p, int plain) {
    if (plain)
        s.hi += p;
    else
        s = ff_add_f(s, p);
}

__device__ __forceinline__ void cp_async16_time(void* smem_dst, const void* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc));
}

__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc));
}

// Shuffle of a value of N floats (a complex number, a float-float, a float4) down the warp.
template <class V>
__device__ __forceinline__ V shfl_down_v(V v, int d) {
    constexpr int N = sizeof(V) / sizeof(float);
    V r;
#pragma unroll
    for (int i = 0; i < N; ++i)
        reinterpret_cast<float*>(&r)[i] = __shfl_down_sync(0xffffffffu, reinterpret_cast<const float*>(&v)[i], d);
    return r;
}

// Sum of `part` over the later segments (seg' > seg) of this thread's column, for threads laid
// out as (seg, c) = (tid >> logC, tid & (C - 1)): a shuffle suffix scan within the warp (a warp
// holds 32/C consecutive segments of each column) and the warps' column totals through `tot`
// (T entries of V; (T/32) C entries when T >= 32).  C <= 32.  Synchronises the block first, so `tot` may still
// be read by a previous call; a caller that alternates between two disjoint `tot` areas of (T/32) C
// entries passes entry_sync = false (blocks of fewer than 32 threads synchronise regardless).
template <class V, class Add>
__device__ __forceinline__ V later_segments_sum(V part, V zero, V* tot, int C, int logC, int T, int tid, Add add,
                                                bool entry_sync = true) {
    const int c = tid & (C - 1);
    V acc = zero;
    if (entry_sync || T < 32) __syncthreads();
    if (T < 32) {
        tot[tid] = part;
        __syncthreads();
        for (int s2 = (tid >> logC) + 1; s2 < (T >> logC); ++s2) acc = add(acc, tot[(s2 << logC) + c]);
        return acc;
    }
    const int lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    V incl = part;
    for (int d = C; d < 32; d <<= 1) {
        const V o = shfl_down_v(incl, d);
        if (lane + d < 32) incl = add(incl, o);
    }
    const V nxt = shfl_down_v(incl, C);
    if (lane + C < 32) acc = nxt;
    if (lane < C) tot[warp * C + lane] = incl;
    __syncthreads();
    for (int w2 = warp + 1; w2 < nwarps; ++w2) acc = add(acc, tot[w2 * C + c]);
    return acc;
}

template <class V>
__device__ __forceinline__ V shfl_up_v(V v, int d) {
    constexpr int N = sizeof(V) / sizeof(float);
    V r;
#pragma unroll
    for (int i = 0; i < N; ++i)
        reinterpret_cast<float*>(&r)[i] = __shfl_up_sync(0xffffffffu, reinterpret_cast<const float*>(&v)[i], d);
    return r;
}

// Sum of `part` over the earlier segments (seg' < seg) of this thread's column: the prefix
// counterpart of later_segments_sum, with the same layout, `tot` and barrier rules.
template <class V, class Add>
__device__ __forceinline__ V earlier_segments_sum(V part, V zero, V* tot, int C, int logC, int T, int tid, Add add,
                                                  bool entry_sync = true) {
    const int c = tid & (C - 1);
    V acc = zero;
    if (entry_sync || T < 32) __syncthreads();
    if (T < 32) {
        tot[tid] = part;
        __syncthreads();
        for (int s2 = 0; s2 < (tid >> logC); ++s2) acc = add(acc, tot[(s2 << logC) + c]);
        return acc;
    }
    const int lane = tid & 31, warp = tid >> 5;
    V incl = part;
    for (int d = C; d < 32; d <<= 1) {
        const V o = shfl_up_v(incl, d);
        if (lane >= d) incl = add(o, incl);
    }
    const V prv = shfl_up_v(incl, C);
    if (lane >= C) acc = prv;
    if (lane >= 32 - C) tot[warp * C + (lane & (C - 1))] = incl;  // the warp's total of column `lane & (C-1)`
    __syncthreads();
    V before = zero;
    for (int w2 = 0; w2 < warp; ++w2) before = add(before, tot[w2 * C + c]);
    return add(before, acc);
}

// Two FP32 lanes in one 64-bit register for the packed f32x2 arithmetic of sm_100 and later.
struct f2x {
    unsigned long long v;
};
__device__ __forceinline__ f2x pk2(float lo, float hi) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 up2(f2x a) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a.v));
    return r;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}

// Rotational Raman susceptibility of this thread's SPT consecutive time samples of one column
// (AddChiUPPE, rotations.cl:85-129; AddChiParaxial, rotations.cl:30-78; rotations.py:40-73).
// pairF(k) gives the drive F of samples 2k and 2k+1 of the segment (in the field scale that the
// host folded into cq); store(k, chi0, chi1) receives their susceptibility.
//
// For every j -> j-2 transition the reference runs, in its time order n = Nt-1-t, with
// h = e^{i wdt/2}, wdt = W_j dt, p_n = h^{2n+1}, F = (dalpha/hbar) E^2 / 2:
//     R_n = sum_{m<n} F_m p_m,   chi_n += sum_{n'<=n} 2 dalpha ng Im(T_j S_j wdt (-i dt) R_n' conj(h^{2n'})).
// With u_n = R_n conj(p_n) and rho_n = |p_n|^2 the output is Im(cq u_n), cq = 2 dalpha T_j S_j wdt
// (-i dt) conj(1/h) (times the field scales), and u obeys u_{n+1} = (u_n + F_n rho_n) conj(h^2),
// rho_{n+1} = rho_n |h^2|^2.  Per transition: pass 1 forms the segment's sum of F_m p_m as
// p0 sum_i F_i h^{2i} from the powers h^{2i}, i < 16 (p0: the phasor of the segment's first sample,
// tabulated in FP64 on the host), the sums of the later segments give R at the segment's first
// sample, and pass 2 runs the u recurrence.
//
// Transitions go in pairs (A, B), one per lane of the packed f32x2 registers, with one block-wide
// carry exchange per pair; an odd count is padded on the host with a transition that adds exactly
// zero.  Per pair, in shared memory (Rs): four float4 {h2.re A, B, h2.im A, B}, {-h2.im A, B,
// |h2|^2 A, B}, {cq.re A, B, cq.im A, B}, unused, then 16 float4 {Re h^{2i} A, B, Im h^{2i} A, B};
// in global memory the phasors p0[pair][segment] = {p.re A, B, p.im A, B}.  The pair terms of each
// sample add up in registers; a last suffix sum (float-float in the mixed form) over t gives chi.
// KEEPF: hold the segment's F = z^2 packed in registers across the pairs (for the variant with
// registers to spare) rather than forming it again in each pass.
template <int SPT, bool KEEPF, class PairF, class Store>
__device__ __forceinline__ void raman_pass(const TimeParams& tp, const float4* Rs, ffloat* tot, int C, int logC,
                                           int T, int tid, int seg, float ngc, PairF pairF, Store store) {
    constexpr int MPS = SPT / 2;
    const int nseg = T >> logC;
    const int npair = tp.rot_pairs;
    f2x g2[SPT];
#pragma unroll
    for (int i = 0; i < SPT; ++i) g2[i] = pk2(0.f, 0.f);
    f2x Fk[KEEPF ? SPT : 1];
    if constexpr (KEEPF) {
#pragma unroll
        for (int k = 0; k < MPS; ++k) {
            const float2 f = pairF(k);
            Fk[2 * k] = pk2(f.x, f.x);
            Fk[2 * k + 1] = pk2(f.y, f.y);
        }
    }
    const auto Fat = [&](int k, int h) -> f2x {
        if constexpr (KEEPF) {
            return Fk[2 * k + h];
        } else {
            const float2 f = pairF(k);
            const float v = h ? f.y : f.x;
            return pk2(v, v);
        }
    };
    // segment totals alternate between two areas of (T/32) C float4 (one barrier per pair)
    float4* tot4 = reinterpret_cast<float4*>(tot);
    const int half4 = (T >= 32) ? (T >> 5) * C : 0;
    const auto add4 = [](float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); };
    float4 p0n = make_float4(0.f, 0.f, 0.f, 0.f);
    if (npair > 0) p0n = __ldg(&tp.rot_p0[seg]);
    for (int r = 0; r < npair; ++r) {
        const float4 p0 = p0n;
        if (r + 1 < npair) p0n = __ldg(&tp.rot_p0[(size_t)(r + 1) * nseg + seg]);
        const float4* Rp = Rs + 20 * r;
        // pass 1: S = sum_i F_i h^{2i}, i the position in the reference's time order (t descending)
        f2x sre = pk2(0.f, 0.f), sim = pk2(0.f, 0.f);
#pragma unroll
        for (int k = MPS - 1; k >= 0; --k) {
#pragma unroll
            for (int h = 1; h >= 0; --h) {
                const float4 H = Rp[4 + 2 * (MPS - 1 - k) + (1 - h)];
                const f2x F = Fat(k, h);
                sre = fma2(F, pk2(H.x, H.y), sre);
                sim = fma2(F, pk2(H.z, H.w), sim);
            }
        }
        // segment total p0 S, then the sums of the later segments: R at this segment's first sample
        const f2x p0re = pk2(p0.x, p0.y), p0im = pk2(p0.z, p0.w), np0im = pk2(-p0.z, -p0.w);
        const float2 a0 = up2(fma2(p0re, sre, mul2(np0im, sim))), a1 = up2(fma2(p0re, sim, mul2(p0im, sre)));
        const float4 R = later_segments_sum(make_float4(a0.x, a0.y, a1.x, a1.y), make_float4(0.f, 0.f, 0.f, 0.f),
                                            tot4 + (r & 1) * half4, C, logC, T, tid, add4, r < 2);
        // pass 2: u = R conj(p0), rho = |p0|^2; u <- (u + F rho) conj(h2), rho <- rho |h2|^2
        const float4 t0 = Rp[0], t1 = Rp[1], t2 = Rp[2];
        const f2x hre = pk2(t0.x, t0.y), him = pk2(t0.z, t0.w), nhim = pk2(t1.x, t1.y);
        const f2x Rre = pk2(R.x, R.y), Rim = pk2(R.z, R.w);
        f2x ure = fma2(Rre, p0re, mul2(Rim, p0im));
        f2x uim = fma2(Rim, p0re, mul2(Rre, np0im));
        f2x rho = fma2(p0re, p0re, mul2(p0im, p0im));
        const f2x d2 = pk2(t1.z, t1.w), cqre = pk2(t2.x, t2.y), cqim = pk2(t2.z, t2.w);
#pragma unroll
        for (int k = MPS - 1; k >= 0; --k) {
#pragma unroll
            for (int h = 1; h >= 0; --h) {
                g2[2 * k + h] = fma2(cqim, ure, fma2(cqre, uim, g2[2 * k + h]));
                ure = fma2(Fat(k, h), rho, ure);
                const f2x nre = fma2(ure, hre, mul2(uim, him));
                uim = fma2(ure, nhim, mul2(uim, hre));
                ure = nre;
                rho = mul2(rho, d2);
            }
        }
    }
    // chi(t) = ng sum_{t' >= t} g(t')
    float g[SPT];
#pragma unroll
    for (int i = 0; i < SPT; ++i) {
        const float2 v = up2(g2[i]);
        g[i] = v.x + v.y;
    }
    ffloat part = {0.f, 0.f};
#pragma unroll
    for (int i = SPT - 1; i >= 0; --i) acc_add(part, g[i], tp.plain);
    const int plain = tp.plain;
    ffloat cum = later_segments_sum(part, ffloat{0.f, 0.f}, tot, C, logC, T, tid, [plain](ffloat x, ffloat y) {
        if (plain) return ffloat{x.hi + y.hi, 0.f};
        return ff_add(x, y);
    });
#pragma unroll
    for (int k = MPS - 1; k >= 0; --k) {
        acc_add(cum, g[2 * k + 1], tp.plain);
        const float chi1 = ngc * ff_value(cum);
        acc_add(cum, g[2 * k], tp.plain);
        const float chi0 = ngc * ff_value(cum);
        store(k, chi0, chi1);
    }
    __syncthreads();  // `tot` is reused by the density scan
}


// Transpose of raman_pass: the cotangent of the drive F of this thread's SPT consecutive samples
// (t ascending, index i = t - t0) from the cotangent ybar of the Raman susceptibility at the same
// samples.  With p_n = h^{2n+1}, n = Nt - 1 - t the reference's time order, the forward map is
//     chi_n = sum_{n' <= n} g_{n'},   g_n = ng Im(cq conj(p_n) R_n),   R_n = sum_{m < n} F_m p_m,
// so, with gbar_n = sum_{n' >= n} ybar_{n'} (a prefix sum along t), its transpose is
//     Fbar_m = ng Im(cq p_m W_m),   W_m = sum_{n > m} gbar_n conj(p_n)   (a prefix sum along t).
// Per transition: the segment's sum of gbar conj(p) as conj(p0) sum_i gbar_i conj(h^{2i'}) (i' the
// position in the reference's order, the powers and p0 from the same tables as raman_pass), the sums of
// the earlier segments give W at the segment's first sample, then a running sum along t.  The prefix
// sum of ybar is float-float in the mixed form; the transition sums are FP32, as in raman_pass.
template <int SPT>
__device__ __forceinline__ void raman_adjoint_pass(const TimeParams& tp, const float4* Rs, ffloat* tot, int C,
                                                   int logC, int T, int tid, int seg, float ngc,
                                                   const float (&ybar)[SPT], float (&Fbar)[SPT]) {
    const int nseg = T >> logC;
    const int plain = tp.plain;
    // gbar(t) = sum_{t' <= t} ybar(t')
    ffloat part = {0.f, 0.f};
#pragma unroll
    for (int i = 0; i < SPT; ++i) acc_add(part, ybar[i], plain);
    ffloat run = earlier_segments_sum(part, ffloat{0.f, 0.f}, tot, C, logC, T, tid, [plain](ffloat x, ffloat y) {
        if (plain) return ffloat{x.hi + y.hi, 0.f};
        return ff_add(x, y);
    });
    float gbar[SPT];
#pragma unroll
    for (int i = 0; i < SPT; ++i) {
        acc_add(run, ybar[i], plain);
        gbar[i] = ff_value(run);
        Fbar[i] = 0.f;
    }
    float4* tot4 = reinterpret_cast<float4*>(tot);
    const auto add4 = [](float4 x, float4 y) { return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w); };
    for (int r = 0; r < tp.rot_pairs; ++r) {
        const float4* Rp = Rs + 20 * r;
        const float4 p0 = __ldg(&tp.rot_p0[(size_t)r * nseg + seg]);  // {re A, re B, im A, im B}
        const float4 cq4 = Rp[2];
        // segment sums of gbar conj(p), p(i) = p0 h^{2 i'}, i' = SPT - 1 - i, both transitions of the pair
        float2 sA = make_float2(0.f, 0.f), sB = sA;
#pragma unroll
        for (int i = 0; i < SPT; ++i) {
            const float4 H = Rp[4 + (SPT - 1 - i)];
            const float2 pA = cmul(make_float2(p0.x, p0.z), make_float2(H.x, H.z));
            const float2 pB = cmul(make_float2(p0.y, p0.w), make_float2(H.y, H.w));
            sA = cadd(sA, cscale(cconj(pA), gbar[i]));
            sB = cadd(sB, cscale(cconj(pB), gbar[i]));
        }
        const float4 Wc = earlier_segments_sum(make_float4(sA.x, sB.x, sA.y, sB.y), make_float4(0.f, 0.f, 0.f, 0.f),
                                               tot4, C, logC, T, tid, add4);
        float2 WA = make_float2(Wc.x, Wc.z), WB = make_float2(Wc.y, Wc.w);
        const float2 cqA = make_float2(cq4.x, cq4.z), cqB = make_float2(cq4.y, cq4.w);
#pragma unroll
        for (int i = 0; i < SPT; ++i) {
            const float4 H = Rp[4 + (SPT - 1 - i)];
            const float2 pA = cmul(make_float2(p0.x, p0.z), make_float2(H.x, H.z));
            const float2 pB = cmul(make_float2(p0.y, p0.w), make_float2(H.y, H.w));
            Fbar[i] += ngc * (cmul(cqA, cmul(pA, WA)).y + cmul(cqB, cmul(pB, WB)).y);
            WA = cadd(WA, cscale(cconj(pA), gbar[i]));
            WB = cadd(WB, cscale(cconj(pB), gbar[i]));
        }
    }
    __syncthreads();  // `tot` is reused by the caller
}

// Host: the time-pass parameters of a handle (timepass.cu).
TimeParams uppe_time_params(const UppeHandle* h);
