// Register-resident time-axis pass (TIME_J) for M = Nt/2 = 256, 512 and 1024: the same work as
// k_time (timepass.cu; SeaRay's update_current, modules/uppe_kernel.py:139-186), arranged so that
// each transverse point ("column") lives in TC lanes of one warp and its transforms stay in
// registers.
//
// Per column, with k = t + TC a (frequency) and m = b + R1 c (time, packed pairs):
//   F layout (frequency): lane t holds Z[t + TC a], a < R1 = M / TC;
//   T layout (time):      lane t holds z[b + R1 c] for b = t + TC j (j < NB = R1 / TC), c < TC.
// The inverse transform z[m] = sum_k Z[k] W_M^(-m k) is the four-step split
//   W_M^(-(t + TC a)(b + R1 c)) = W_R1^(-a b) W_M^(-t b) W_TC^(-t c):
//   an R1-point DFT over a in registers, the twiddle, one exchange through the column's shared
//   memory, TC-point DFTs over t in registers.  The forward transform is its mirror image and
//   starts from the T layout and ends in the F layout, so the two transforms of one evaluation need
//   one exchange each, and no block-wide barrier.
// Around them, as in k_time: the even/odd packing of the half spectrum (irfft, fft.cl:257-280),
// Kerr chi = ng chi3/nref E^2 and P = chi E (uppe.cl:132-165), and on the way out the real spectrum
// of the packed P, J = -i w P (+ Jpl / (0.1 - i w)), times the NL filter (fft.cl:282-329).
//
// Ionization (ionization.cl:22-44 / 71-97 rates, 127-155 density, fft.cl:331-355 window): where a
// column holds a field above the rate threshold (a warp vote), the rates go to shared memory in
// natural time order, each lane scans a contiguous segment (float-float in the mixed form, the
// later segments' sums by a shuffle suffix scan), the density comes back, and Jpl = ne E is formed.
// The two forward transforms (P, Jpl) cannot both sit in registers, so this path parks Jpl (time
// order) and then the P part of J (frequency order) in a global scratch array, column-contiguous
// (coalesced), until the Jpl transform is done.
//
// Block: NC columns x TC lanes = 256 threads.  The half spectra of the NC columns are staged into
// shared memory with 8-byte cp.async (rows of NC columns: coalesced), one buffer of LD complex
// values per column that then serves the exchanges, the density scan and the output staging; J is
// written back the same way.
#include <math.h>

#include "hankel_tc.cuh"
#include "time_common.cuh"
#include "timepass_reg.cuh"
#include "uppe_internal.h"

template <int LOGM>
__global__ void __launch_bounds__(256, TReg<LOGM>::MINB)
    k_time_reg(const float2* __restrict__ E, float2* __restrict__ Jout, const float* __restrict__ ng,
               const float* __restrict__ wv, const float2* __restrict__ twt,
               float2* __restrict__ tscr, TimeParams tp) {
    using G = TReg<LOGM>;
    constexpr int M = G::M, TC = G::TC, R1 = G::R1, NC = G::NC, LD = G::LD;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x;
    const size_t S = (size_t)tp.S;
    const size_t col0 = (size_t)blockIdx.x * NC;

    pdl_begin();
    // ---- stage the NC half spectra X[k][c] (k <= M) into the column buffers ----
    for (int i = tid; i < (M + 1) * NC; i += G::THREADS) {
        const int c = i & (NC - 1), k = i / NC;
        cp_async8(&sm[c * LD + k], &E[(size_t)k * S + col0 + c]);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int cl = (TC == 32) ? warp : 2 * warp + (lane >> 4);
    const int t = lane & (TC - 1);
    float2* buf = sm + cl * LD;
    const size_t col = col0 + cl;
    const float2* twI = twt;
    const float2* twF = twt + M;
    const float2* twP = twt + 2 * M;

    // ---- irfft of the staged half spectrum into the T layout ----
    float2 v[R1];
    tr_pack_inverse<LOGM>(v, buf, twI, twP, t, [&](int k) { return buf[k]; });
    // v[j TC + c] = Nt (E(2m) + i E(2m+1)), m = t + TC j + R1 c

    const float inv = tp.inv_nt;
    const float ngc = ng[col];
    const float kerr = ngc * tp.redchi3;
    const bool ionize = tp.rate_form != UPPE_RATE_NONE;
    bool live = false;
    if (ionize) {
        // any sample with Em = fconv |e| + cutoff >= em_min: Em grows with |e| (fconv > 0), so the
        // largest |e| of the lane decides (the same roundings as per sample)
        float mx = 0.f;
#pragma unroll
        for (int r = 0; r < R1; ++r) mx = fmaxf(mx, fmaxf(fabsf(v[r].x), fabsf(v[r].y)));
        const bool any = fmaf(tp.fconv, mx * inv, tp.cutoff) >= tp.em_min;
        live = __any_sync(0xffffffffu, any);  // warp-uniform (both columns of a warp when TC = 16)
    }
    // the column's parking place in the scratch array (ionizing columns only): [0, M) Jpl by m,
    // [M + 1, 2M + 2) the P part of J by k
    float2* park = live ? tscr + col * (size_t)(2 * (M + 1)) : nullptr;
    if (live) {
        // rates in natural order (padded positions)
        __syncwarp();  // exchange reads of buf are done
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const int m = G::tm(t, r);
            const float2 z = v[r];
            const float r0 = ion_rate(tp, z.x * inv);
            const float r1 = (2 * m + 1 == G::NT - 1) ? 0.f : ion_rate(tp, z.y * inv);
            buf[tr_pad<G::LSEG>(m)] = make_float2(r0, r1);
        }
        __syncwarp();
        // density: lane t scans the pairs [t SEG, (t+1) SEG) from high to low time
        const int mb = t * G::SEG;
        const float r_next = (t < TC - 1) ? buf[tr_pad<G::LSEG>(mb + G::SEG)].x : 0.f;
        ffloat part = {0.f, 0.f};
        {
            float rn = r_next;
            for (int i = G::SEG - 1; i >= 0; --i) {
                const int m = mb + i;
                const float2 rr = buf[tr_pad<G::LSEG>(m)];
                if (2 * m + 1 <= G::NT - 2) {
                    const float p1 = tp.hdt * (rr.y + rn);
                    if (p1 != 0.f) acc_add(part, p1, tp.plain);
                }
                const float p0 = tp.hdt * (rr.x + rr.y);
                if (p0 != 0.f) acc_add(part, p0, tp.plain);
                rn = rr.x;
            }
        }
        // sum over the later lanes of the column
        ffloat incl = part;
#pragma unroll
        for (int d = 1; d < TC; d <<= 1) {
            const float hi = __shfl_down_sync(0xffffffffu, incl.hi, d, TC);
            const float lo = __shfl_down_sync(0xffffffffu, incl.lo, d, TC);
            if (t + d < TC) {
                if (tp.plain)
                    incl.hi += hi;
                else
                    incl = ff_add(incl, ffloat{hi, lo});
            }
        }
        ffloat Sacc;
        Sacc.hi = __shfl_down_sync(0xffffffffu, incl.hi, 1, TC);
        Sacc.lo = __shfl_down_sync(0xffffffffu, incl.lo, 1, TC);
        if (t == TC - 1) Sacc = ffloat{0.f, 0.f};
        __syncwarp();  // every lane has read its neighbour's first rate
        {
            const int wlo = tp.wcut + tp.wwid, whi = G::NT - tp.wcut - tp.wwid - 1;  // window is 1 on [wlo, whi]
            float rn = r_next;
            for (int i = G::SEG - 1; i >= 0; --i) {
                const int m = mb + i;
                const float2 rr = buf[tr_pad<G::LSEG>(m)];
                const int t1 = 2 * m + 1;
                if (t1 <= G::NT - 2) acc_add(Sacc, tp.hdt * (rr.y + rn), tp.plain);
                float ne1 = ngc * one_minus_exp_neg(ff_value(Sacc));
                if (t1 < wlo || t1 > whi) ne1 *= soft_window(t1, G::NT, tp.wcut, tp.wwid);
                acc_add(Sacc, tp.hdt * (rr.x + rr.y), tp.plain);
                float ne0 = ngc * one_minus_exp_neg(ff_value(Sacc));
                if (t1 - 1 < wlo || t1 - 1 > whi) ne0 *= soft_window(t1 - 1, G::NT, tp.wcut, tp.wwid);
                rn = rr.x;
                buf[tr_pad<G::LSEG>(m)] = make_float2(ne0, ne1);
            }
        }
        __syncwarp();
        // Jpl = ne E, parked in time order; P = chi E in registers
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const int m = G::tm(t, r);
            const float2 ne = buf[tr_pad<G::LSEG>(m)];
            const float e0 = v[r].x * inv, e1 = v[r].y * inv;
            park[m] = make_float2(ne.x * e0, ne.y * e1);
            v[r] = make_float2(kerr * e0 * e0 * e0, kerr * e1 * e1 * e1);
        }
    } else {
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const float e0 = v[r].x * inv, e1 = v[r].y * inv;
            v[r] = make_float2(kerr * e0 * e0 * e0, kerr * e1 * e1 * e1);
        }
    }

    // ---- forward transform of P and its real spectrum: J = -i w P (x filter) ----
    tr_forward<LOGM>(v, buf, twF, t);
    __syncwarp();  // the exchange reads of buf are done before the output staging
    // the NL filter (0 or 1 per bin) from its cut indices
    const auto kept = [&](int k) { return k >= tp.cut_on && k < tp.cut_off; };
    if (!live) {
        tr_unpack<LOGM>(v, twP, t, lane, [&](int k, float2 P) {
            buf[k] = kept(k) ? cmul_mi(cscale(P, __ldg(&wv[k]))) : make_float2(0.f, 0.f);
        });
    } else {
        float2* parkJ = park + (M + 1);
        tr_unpack<LOGM>(v, twP, t, lane, [&](int k, float2 P) {
            parkJ[k] = kept(k) ? cmul_mi(cscale(P, __ldg(&wv[k]))) : make_float2(0.f, 0.f);
        });
        // Jpl from its parking place (this lane's own entries), forward transform, and
        // J += Jpl(w) (damping + i w) / (damping^2 + w^2) (x filter)
#pragma unroll
        for (int r = 0; r < R1; ++r) v[r] = park[G::tm(t, r)];
        tr_forward<LOGM>(v, buf, twF, t);
        __syncwarp();
        const float damp = tp.damping;
        tr_unpack<LOGM>(v, twP, t, lane, [&](int k, float2 Q) {
            const float wk = __ldg(&wv[k]);
            const float rden = __frcp_rn(fmaf(wk, wk, damp * damp));
            const float2 q = cscale(cmul(Q, make_float2(damp, wk)), rden);
            buf[k] = kept(k) ? cadd(parkJ[k], q) : make_float2(0.f, 0.f);
        });
    }

    // ---- write J back: rows of NC columns ----
    __syncthreads();
    for (int i = tid; i < (M + 1) * NC; i += G::THREADS) {
        const int c = i & (NC - 1), k = i / NC;
        if (tp.atc)
            tc_store_split(tp.atc, tp.atc_nwt, tp.atc_nkt, 0, k, (int)(col0 + c), sm[c * LD + k]);
        else
            Jout[(size_t)k * S + col0 + c] = sm[c * LD + k];
    }
}

// ---- host side ----

bool time_reg_supported(const UppeHandle* h) {
    if (h->cfg.envelope || h->rot_pairs > 0) return false;
    if (h->M != 256 && h->M != 512 && h->M != 1024) return false;
    const int nc = (h->M == 1024) ? TReg<10>::NC : (h->M == 512) ? TReg<9>::NC : TReg<8>::NC;
    return h->S % nc == 0;
}

size_t time_reg_table_len(int M) { return (size_t)3 * M; }

// twI[b TC + t] = W_M^(t b); twF[(j TC + k1) TC + t] = W_M^((t + TC j) k1); twP[a TC + t] =
// e^{-2 pi i (t + TC a) / Nt}; computed in FP64.
int time_reg_tables(int M, float2* host) {
    int TC, R1;
    if (M == 256) {
        TC = TReg<8>::TC;
        R1 = TReg<8>::R1;
    } else if (M == 512) {
        TC = TReg<9>::TC;
        R1 = TReg<9>::R1;
    } else if (M == 1024) {
        TC = TReg<10>::TC;
        R1 = TReg<10>::R1;
    } else {
        return -1;
    }
    const double two_pi = 6.283185307179586476925286766559;
    auto w = [&](long long e, long long n) {
        const double a = -two_pi * (double)(e % n) / (double)n;
        return make_float2((float)cos(a), (float)sin(a));
    };
    for (int b = 0; b < R1; ++b)
        for (int t = 0; t < TC; ++t) host[b * TC + t] = w((long long)t * b, M);
    if (TC > R1) {
        // lane pairs (TC = 2 R1): twF[i TC + t] = W_M^(b (2 i + h)), t = b + R1 h
        for (int i = 0; i < R1; ++i)
            for (int t = 0; t < TC; ++t) host[M + i * TC + t] = w((long long)(t % R1) * (2 * i + t / R1), M);
    } else {
        const int NB = R1 / TC;
        for (int j = 0; j < NB; ++j)
            for (int k1 = 0; k1 < TC; ++k1)
                for (int t = 0; t < TC; ++t) host[M + (j * TC + k1) * TC + t] = w((long long)(t + TC * j) * k1, M);
    }
    for (int a = 0; a < R1; ++a)
        for (int t = 0; t < TC; ++t) host[2 * M + a * TC + t] = w(t + (long long)TC * a, 2 * M);
    return 0;
}

size_t time_reg_scratch_len(const UppeHandle* h) { return (size_t)h->S * 2 * (h->M + 1); }

cudaError_t uppe_configure_time_reg() {
    cudaError_t e = cudaFuncSetAttribute(k_time_reg<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TReg<8>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_reg<9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TReg<9>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_reg<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TReg<10>::SMEM);
    return e;
}

cudaError_t launch_time_reg(UppeHandle* h, const float2* E, float2* J) {
    const TimeParams tp = uppe_time_params(h);
    h->launches++;
    switch (h->M) {
        case 256:
            launch_pdl(k_time_reg<8>, dim3(h->S / TReg<8>::NC), dim3(TReg<8>::THREADS), TReg<8>::SMEM, h->stream, E, J, h->ng, h->w, h->tw_reg, h->tscr, tp);
            break;
        case 512:
            launch_pdl(k_time_reg<9>, dim3(h->S / TReg<9>::NC), dim3(TReg<9>::THREADS), TReg<9>::SMEM, h->stream, E, J, h->ng, h->w, h->tw_reg, h->tscr, tp);
            break;
        default:
            launch_pdl(k_time_reg<10>, dim3(h->S / TReg<10>::NC), dim3(TReg<10>::THREADS), TReg<10>::SMEM, h->stream, E, J, h->ng, h->w, h->tw_reg, h->tscr, tp);
            break;
    }
    return cudaGetLastError();
}
