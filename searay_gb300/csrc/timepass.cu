// Time-axis pass of one UPPE right-hand-side evaluation: the part of SeaRay's update_current
// (modules/uppe_kernel.py:139-186) that runs along t for every transverse point.
//
// One CTA takes C adjacent transverse points ("columns") and all N0 = M + 1 frequencies:
//   1. irfft along w (fft.cl:257-280, 1/Nt normalised) as an M-point complex inverse FFT of the
//      even/odd packing Z[k] = (X[k] + conj X[M-k]) + i e^{2 pi i k/Nt} (X[k] - conj X[M-k]),
//      which leaves z[m] = Nt (E(2m) + i E(2m+1)),
//   2. per time sample: Kerr chi = ng chi3/nref E^2 (uppe.cl:132-151), the ionization rate
//      (ionization.cl:22-44 explicit / 71-97 series), the electron density by the reverse
//      trapezoid sum with rate(Nt-1) = 0 and depletion ne = ng (1 - exp(-S)) (ionization.cl:127-155),
//      SoftTimeWindow on ne (fft.cl:331-355), P = chi E and Jpl = ne E (uppe.cl:153-165,
//      uppe_kernel.py:169); P and Jpl are written back packed as even/odd pairs, in place,
//   3. two M-point forward FFTs (P, then Jpl), split into the real spectra and
//      J = -i w P + Jpl / (0.1 - i w), times the NL filter (fft.cl:282-329, uppe_kernel.py:171-186).
// The density sum is a two-pass blocked scan: every thread sums its own consecutive samples, then
// adds the totals of all later segments of its column (the sum runs from high to low t).
// The sums are float-float in the mixed form.
#include <math.h>

#include "common.cuh"
#include "fft_smem.cuh"
#include "hankel_tc.cuh"
#include "time_common.cuh"
#include "uppe_internal.h"

// Real spectrum X[k], k in [0, M], of the real signal packed as z[m] = x(2m) + i x(2m+1) whose
// M-point FFT is Zc: X[k] = (Za + Zb)/2 - (i/2) e^{-2 pi i k/Nt} (Za - Zb), Za = Zc[k mod M],
// Zb = conj Zc[(M-k) mod M].
__device__ __forceinline__ float2 real_spectrum(float2 Za, float2 Zb_raw, float2 twk) {
    const float2 Zb = cconj(Zb_raw);
    const float2 s = cadd(Za, Zb);
    const float2 d = cmul(twk, csub(Za, Zb));
    return cscale(csub(s, cmul_i(d)), 0.5f);
}

// ET: complex FFT elements per thread (16: 256 threads for C*Nt = 8192; 8: 512 threads)
// LOGM > 0: compile-time sizes M = 2^LOGM, C = 2^LOGC (constant-folded index arithmetic and the
// compile-time Stockham transforms); LOGM = 0: sizes from the parameters.
// RAMAN: adds the rotational Raman susceptibility (raman_pass, 16 samples per thread; the segment
// totals take 2T entries, followed by a third array Zr [M][C] for the Raman chi pairs and the pair
// tables Rs, 20 float4 per pair).  RAMAN = 1: one block per multiprocessor, F kept in registers;
// RAMAN = 2: two blocks per multiprocessor.
template <int ET, int LOGM = 0, int LOGC = -1, int RAMAN = 0>
// (three blocks per multiprocessor where shared memory allows it: M <= 512)
__global__ void __launch_bounds__(ET == 16 ? 256 : 512,
                                  RAMAN ? RAMAN : (ET == 16 ? 3 : ((LOGM > 0 && LOGM <= 9) ? 3 : 2))) k_time(int mode, const float2* __restrict__ E, float2* __restrict__ out0,
                                                  float2* __restrict__ out1, const float* __restrict__ ng,
                                                  const float* __restrict__ wv, const float* __restrict__ filt,
                                                  const float2* __restrict__ tw, int twLog, TimeParams tp) {
    // shared layout: Zp [M+1][C] (E pairs, then P pairs), Zj [M+1][C] (the raw half spectrum X
    // while loading, then the rates (r(2m), r(2m+1)), then Jpl pairs), twiddles e^{-2 pi i j/Nt}
    // for j < Nt/2, one float-float segment total per thread.  Rows of C float2 keep the
    // column-batched FFT accesses of a warp on distinct banks.
    extern __shared__ float2 Zp[];
    constexpr bool CT = LOGM > 0;
    const int C = CT ? (1 << LOGC) : tp.C, logC = CT ? LOGC : tp.logC;
    const int Nt = CT ? (2 << LOGM) : tp.Nt, M = CT ? (1 << LOGM) : tp.M, S = tp.S;
    float2* Zj = Zp + (size_t)(M + 1) * C;
    float2* twl = Zj + (size_t)(M + 1) * C;
    ffloat* tot = reinterpret_cast<ffloat*>(twl + (Nt >> 1));
    const int tid = threadIdx.x, T = CT ? ((2 << LOGM) << LOGC) / (2 * ET) : (int)blockDim.x;
    const size_t col0 = (size_t)blockIdx.x * C;
    const bool ionize = tp.rate_form != UPPE_RATE_NONE;
    const TwHalfShared tws{twl, tp.logNt};
    // rows of the transforms in the row-swizzled order of the shared-memory FFTs (RowSwizzle; on for
    // blocks of at most 4 columns)
    const RowSwizzle sw{logC <= 2 ? M - 1 : 0, logC == 0 ? 4 : 3};

    pdl_begin();
    // ---- 1. stage the half spectrum X[k][c], k in [0, M], with asynchronous copies ----
    if (C >= 2) {
        const int hC = C >> 1;  // 16-byte copies of two adjacent columns
        for (int it = tid; it < (M + 1) * hC; it += T) {
            const int c2 = it & (hC - 1);
            const int k = it >> (logC > 0 ? logC - 1 : 0);  // (this branch runs only with C >= 2)
            cp_async16_time(&Zj[sw(k) * C + 2 * c2], &E[(size_t)k * S + col0 + 2 * c2]);
        }
    } else {
        for (int it = tid; it < (M + 1) * C; it += T) {
            const int c = it & (C - 1);
            const int k = it >> logC;
            cp_async8(&Zj[sw(k) * C + c], &E[(size_t)k * S + col0 + c]);
        }
    }
    float2* Zr = reinterpret_cast<float2*>(tot + 2 * T);
    float4* Rs = reinterpret_cast<float4*>(Zr + (size_t)M * C);
    if constexpr (RAMAN != 0)
        for (int i = tid; i < 20 * tp.rot_pairs; i += T) cp_async16_time(&Rs[i], &tp.rot_tab[i]);
    asm volatile("cp.async.commit_group;\n" ::);
    for (int j = tid; j < (Nt >> 1); j += T) twl[j] = __ldg(&tw[j << (twLog - tp.logNt)]);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
    // even/odd packing Z[k] = (X[k] + conj X[M-k]) + i e^{2 pi i k/Nt} (X[k] - conj X[M-k])
    const int npairs = (M / 2 + 1) * C;
    for (int it = tid; it < npairs; it += T) {
        const int c = it & (C - 1);
        const int k = it >> logC;
        float2 Xa = Zj[sw(k) * C + c];
        float2 Xm = Zj[sw(M - k) * C + c];
        if (k == 0) {
            Xa.y = 0.f;
            Xm.y = 0.f;
        }
        const float2 t = cconj(tws.get(k));  // e^{+2 pi i k / Nt}
        const float2 b = cconj(Xm);
        Zp[sw(k) * C + c] = cadd(cadd(Xa, b), cmul_i(cmul(t, csub(Xa, b))));
        if (k != 0 && 2 * k != M) {
            const float2 t2 = make_float2(-t.x, t.y);  // e^{2 pi i (M-k)/Nt}
            const float2 b2 = cconj(Xa);
            Zp[sw(M - k) * C + c] = cadd(cadd(Xm, b2), cmul_i(cmul(t2, csub(Xm, b2))));
        }
    }
    __syncthreads();
    if constexpr (CT)
        fft_axis_ct<ET, LOGM, LOGC, LOGM + 1>(Zp, TwHalfSharedCT<LOGM + 1>{twl}, true, tid);
    else
        fft_axis_tw<ET>(Zp, tp.logM, logC, 1, C, tws, true, tid, T, -1, sw);

    // ---- 2. sources, in place ----
    const int c = tid & (C - 1);
    const int seg = tid >> logC;
    const int mps = CT ? 8 : (tp.spt >> 1);  // packed pairs per thread (16 samples with compile-time sizes)
    const int m0 = seg * mps;
    const int t1 = 2 * (m0 + mps);  // first sample of the next segment
    const float ngc = ng[col0 + c];
    const float kerr = ngc * tp.redchi3;
    const float inv = tp.inv_nt;
    if constexpr (RAMAN != 0) {  // F = z^2 of the packed pairs z = Nt (E(2m), E(2m+1))
        raman_pass<16, RAMAN == 1>(
            tp, Rs, tot, C, logC, T, tid, seg, ngc,
            [&](int k) {
                const float2 zv = Zp[sw(m0 + k) * C + c];
                return make_float2(zv.x * zv.x, zv.y * zv.y);
            },
            [&](int k, float chi0, float chi1) { Zr[sw(m0 + k) * C + c] = make_float2(chi0, chi1); });
    }
    float r_next = 0.f;
    ffloat part = {0.f, 0.f};
    bool live = false;  // a nonzero rate in this segment (zero increments leave a float-float sum exactly as it is)
    if (ionize) {
        if (t1 <= Nt - 2) r_next = ion_rate(tp, Zp[sw(t1 >> 1) * C + c].x * inv);
        float rn = r_next;
#pragma unroll(CT ? 8 : 1)
        for (int m = m0 + mps - 1; m >= m0; --m) {
            const float2 zv = Zp[sw(m) * C + c];
            const int t = 2 * m + 1;
            const float r1 = (t == Nt - 1) ? 0.f : ion_rate(tp, zv.y * inv);
            const float p1 = tp.hdt * (r1 + rn);
            if (t <= Nt - 2 && p1 != 0.f) acc_add(part, p1, tp.plain);
            const float r0 = ion_rate(tp, zv.x * inv);
            const float p0 = tp.hdt * (r0 + r1);
            if (p0 != 0.f) acc_add(part, p0, tp.plain);
            live = live || r0 != 0.f || r1 != 0.f;
            rn = r0;
            Zj[sw(m) * C + c] = make_float2(r0, r1);  // this thread's own slot, reused below
        }
        live = live || r_next != 0.f;
    }
    // Sum of the later segments of this column.  A warp holds 32/C consecutive segments of each of
    // the C columns (lanes C apart): a shuffle suffix scan gives the sums within the warp, and the
    // warps' column totals, published in shared memory, the sums beyond it.
    ffloat Sacc = {0.f, 0.f};
    if (ionize && T < 32) {  // a block smaller than a warp (17 frequencies, under 16 points): sequential
        tot[tid] = part;
        __syncthreads();
        for (int s2 = seg + 1; s2 < (T >> logC); ++s2) {
            const ffloat v = tot[(s2 << logC) + c];
            if (tp.plain)
                Sacc.hi += v.hi;
            else
                Sacc = ff_add(Sacc, v);
        }
    } else if (ionize) {
        const int lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
        ffloat incl = part;
        for (int d = C; d < 32; d <<= 1) {
            const float hi = __shfl_down_sync(0xffffffffu, incl.hi, d);
            const float lo = __shfl_down_sync(0xffffffffu, incl.lo, d);
            if (lane + d < 32) {
                if (tp.plain)
                    incl.hi += hi;
                else
                    incl = ff_add(incl, ffloat{hi, lo});
            }
        }
        Sacc.hi = __shfl_down_sync(0xffffffffu, incl.hi, C);
        Sacc.lo = __shfl_down_sync(0xffffffffu, incl.lo, C);
        if (lane + C >= 32) Sacc = ffloat{0.f, 0.f};
        if (lane < C) tot[warp * C + lane] = incl;  // this warp's total of column `lane`
        __syncthreads();
        for (int w2 = warp + 1; w2 < nwarps; ++w2) {
            const ffloat v = tot[w2 * C + c];
            if (tp.plain)
                Sacc.hi += v.hi;
            else
                Sacc = ff_add(Sacc, v);
        }
    } else {
        __syncthreads();  // pass 2 overwrites pairs that pass 1 of the previous segment read
    }
    // no rate in this segment and none in the later ones: the density is zero throughout
    const bool dens = ionize && (live || Sacc.hi != 0.f || Sacc.lo != 0.f);
    {
        float rn = r_next;
        const int wlo = tp.wcut + tp.wwid, whi = Nt - tp.wcut - tp.wwid - 1;  // window is 1 on [wlo, whi]
#pragma unroll(CT ? 8 : 1)
        for (int m = m0 + mps - 1; m >= m0; --m) {
            const float2 zv = Zp[sw(m) * C + c];
            const float e1 = zv.y * inv, e0 = zv.x * inv;
            float ne1 = 0.f, ne0 = 0.f;
            if (dens) {
                const float2 rr = Zj[sw(m) * C + c];
                const int t = 2 * m + 1;
                if (t <= Nt - 2) acc_add(Sacc, tp.hdt * (rr.y + rn), tp.plain);
                ne1 = ngc * one_minus_exp_neg(ff_value(Sacc));
                if (t < wlo || t > whi) ne1 *= soft_window(t, Nt, tp.wcut, tp.wwid);
                acc_add(Sacc, tp.hdt * (rr.x + rr.y), tp.plain);
                rn = rr.x;
                ne0 = ngc * one_minus_exp_neg(ff_value(Sacc));
                if (t - 1 < wlo || t - 1 > whi) ne0 *= soft_window(t - 1, Nt, tp.wcut, tp.wwid);
            }
            float chi1 = kerr * e1 * e1, chi0 = kerr * e0 * e0;
            if constexpr (RAMAN != 0) {  // the Raman chi comes first in the reference's sum (uppe_kernel.py:173-179)
                const float2 zr = Zr[sw(m) * C + c];
                chi1 = zr.y + chi1;
                chi0 = zr.x + chi0;
            }
            if (mode == TIME_J) {
                Zp[sw(m) * C + c] = make_float2(chi0 * e0, chi1 * e1);
                Zj[sw(m) * C + c] = make_float2(ne0 * e0, ne1 * e1);
            } else {
                Zp[sw(m) * C + c] = make_float2(chi0, chi1);
                Zj[sw(m) * C + c] = make_float2(ne0, ne1);
            }
        }
    }
    // a block whose density is zero everywhere has Jpl = 0: its transform is left out (exactly zero)
    const bool any_ne = __syncthreads_or(dens ? 1 : 0) != 0;

    // ---- 3. forward FFTs (P, then Jpl) and the current ----
    const bool two = any_ne || mode == TIME_CHI_NE;
    if constexpr (CT) {
        fft_axis_ct<ET, LOGM, LOGC, LOGM + 1>(Zp, TwHalfSharedCT<LOGM + 1>{twl}, false, tid);
        if (two) fft_axis_ct<ET, LOGM, LOGC, LOGM + 1>(Zj, TwHalfSharedCT<LOGM + 1>{twl}, false, tid);
    } else {
        fft_axis_tw<ET>(Zp, tp.logM, logC, 1, C, tws, false, tid, T, -1, sw);
        if (two) fft_axis_tw<ET>(Zj, tp.logM, logC, 1, C, tws, false, tid, T, -1, sw);
    }
    for (int it = tid; it < (M + 1) * C; it += T) {
        const int cc = it & (C - 1);
        const int k = it >> logC;
        const int ka = k & (M - 1), kb = (M - k) & (M - 1);
        const float2 twk = tws.get(k);  // e^{-2 pi i k / Nt}
        const float2 P = real_spectrum(Zp[sw(ka) * C + cc], Zp[sw(kb) * C + cc], twk);
        const float2 Q = two ? real_spectrum(Zj[sw(ka) * C + cc], Zj[sw(kb) * C + cc], twk) : make_float2(0.f, 0.f);
        const size_t o = (size_t)k * S + col0 + cc;
        if (mode == TIME_J) {
            const float wk = wv[k];
            float2 J = cmul_mi(cscale(P, wk));  // -i w P
            if (two) {  // Jpl / (damping - i w) = Jpl (damping + i w) / (damping^2 + w^2)
                const float rden = __frcp_rn(fmaf(wk, wk, tp.damping * tp.damping));
                J = cadd(J, cscale(cmul(Q, make_float2(tp.damping, wk)), rden));
            }
            if (tp.atc)
                tc_store_split(tp.atc, tp.atc_nwt, tp.atc_nkt, 0, k, (int)(col0 + cc), cscale(J, filt[k]));
            else
                out0[o] = cscale(J, filt[k]);
        } else {
            if (out0) out0[o] = P;
            if (out1) out1[o] = ionize ? Q : make_float2(0.f, 0.f);
        }
    }
}

// The time-pass shapes with compile-time sizes: C Nt = 8192 with 16 samples per thread (512 threads),
// M = 256 .. 2048.
#define UPPE_TIME_CT(X) X(8, 4) X(9, 3) X(10, 2) X(11, 1)

cudaError_t uppe_configure_time_kernel(size_t smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_time<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_time<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
#define UPPE_TIME_CONF(A_, B_) \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_time<8, A_, B_>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    UPPE_TIME_CT(UPPE_TIME_CONF)
#undef UPPE_TIME_CONF
#define UPPE_TIME_RCONF(A_, B_)                                                                                     \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_time<8, A_, B_, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes); \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_time<8, A_, B_, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    UPPE_TIME_CT(UPPE_TIME_RCONF)
    UPPE_TIME_RCONF(0, -1)
#undef UPPE_TIME_RCONF
    return e;
}

TimeParams uppe_time_params(const UppeHandle* h) {
    const UppeConfig& c = h->cfg;
    TimeParams tp;
    tp.Nt = h->Nt;
    tp.logNt = ilog2_exact(h->Nt);
    tp.M = h->M;
    tp.logM = ilog2_exact(h->M);
    tp.C = h->time_cols;
    tp.logC = ilog2_exact(h->time_cols);
    tp.S = h->S;
    tp.spt = h->time_spt;
    tp.inv_nt = (float)(1.0 / (double)h->Nt);
    tp.hdt = (float)(0.5 * c.dt);
    tp.redchi3 = (float)h->redchi3;
    tp.damping = (float)c.damping;
    tp.rate_form = c.rate_form;
    tp.fconv = (float)c.field_conv;
    tp.cutoff = (float)c.field_cutoff;
    const double log2e = 1.4426950408889634;
    tp.y0 = (c.rate_form == UPPE_RATE_EXPLICIT) ? (float)log2(c.rate_conv * c.c_pre) : 0.f;
    tp.ypow = (float)c.c_pow;
    tp.yexp = (float)(c.c_exp * log2e);
    tp.lrc2 = (c.rate_conv > 0) ? (float)log2(c.rate_conv) : 0.f;
    for (int i = 0; i < 6; ++i) tp.c2[i] = (float)(c.clog[i] * log2e);
    tp.wcut = c.window_cutoff;
    tp.cut_on = c.nl_cut_on;
    tp.cut_off = c.nl_cut_off;
    tp.wwid = c.window_width;
    tp.plain = (c.precision == UPPE_PREC_FP32);
    tp.rot_pairs = h->rot_pairs;
    tp.rot_tab = reinterpret_cast<const float4*>(h->rot);
    tp.rot_p0 = reinterpret_cast<const float4*>(h->rot + 80 * h->rot_pairs);
    tp.atc = nullptr;
    tp.atc_nwt = tp.atc_nkt = 0;
    if (h->time_atc && h->Atc) {
        tp.atc = h->Atc;
        tp.atc_nwt = (h->N0 + TC_W - 1) / TC_W;
        tp.atc_nkt = (h->N1 + TC_K - 1) / TC_K;
    }
    tp.em_min = 0.f;
    if (c.rate_form != UPPE_RATE_NONE) {
        // log2(rate) as a function of Em (atomic units); it rises from -inf at Em -> 0 for physical
        // rate models.  Bisect for the Em where it crosses -150, well below FP32's 2^-126.
        auto log2rate = [&](double em) {
            if (c.rate_form == UPPE_RATE_EXPLICIT)
                return log2(c.rate_conv * c.c_pre) + c.c_pow * log2(em) + c.c_exp * log2e / em;
            const double L = log(em);
            double p = c.clog[5];
            for (int i = 4; i >= 0; --i) p = p * L + c.clog[i];
            return log2(c.rate_conv) + p * log2e;
        };
        double lo = c.field_cutoff, hi = 10.0;
        if (log2rate(lo) < -150.0 && log2rate(hi) > -150.0) {
            for (int it = 0; it < 80; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (log2rate(mid) < -150.0)
                    lo = mid;
                else
                    hi = mid;
            }
            // only trust the threshold if the rate really stays below it on [cutoff, lo]
            bool mono = true;
            for (int i = 0; i <= 64; ++i) {
                const double em = c.field_cutoff + (lo - c.field_cutoff) * i / 64.0;
                if (log2rate(em) > -150.0) mono = false;
            }
            if (mono) tp.em_min = (float)lo;
        }
    }
    return tp;
}

cudaError_t launch_time_pass(UppeHandle* h, int mode, const float2* E, float2* out0, float2* out1) {
    if (h->cfg.envelope) return launch_time_env(h, mode, E, out0, out1);
    // the register-resident pass (timepass_reg.cu) for the current J at M = 256, 512, 1024;
    // SEARAY_UPPE_TIME=smem selects the shared-memory form below for every grid
    if (mode == TIME_J && h->time_reg && h->tw_reg && time_reg_supported(h)) return launch_time_reg(h, E, out0);
    const TimeParams tp = uppe_time_params(h);
    const int C = h->time_cols;
    const int T = h->Nt * C / h->time_spt;
    const size_t smem = ((size_t)(h->M + 1) * 2 * C + h->Nt / 2) * sizeof(float2) + (size_t)T * sizeof(ffloat);
    h->launches++;
    if (h->rot_pairs > 0) {  // 16 samples per thread; Zr and the pair tables after the segment totals
        TimeParams tr = tp;
        tr.spt = 16;
        const int Tr = h->Nt * h->time_cols / 16;
        const size_t smem_r = ((size_t)(h->M + 1) * 2 * h->time_cols + h->Nt / 2) * sizeof(float2) +
                              (size_t)2 * Tr * sizeof(ffloat) + (size_t)h->M * h->time_cols * sizeof(float2) +
                              (size_t)20 * h->rot_pairs * sizeof(float4);
        // two blocks per multiprocessor where their shared memory fits (64 registers, F formed in each
        // pass), else one block with the segment's F held in registers (128 registers)
        const bool occ2 = 2 * (smem_r + 1024) <= (size_t)h->smem_per_sm;
#define UPPE_TIME_RCASE(A_, B_)                                                                                     \
        if (tp.logM == A_ && tp.logC == B_) {                                                                          \
            if (occ2)                                                                                                 \
                launch_pdl(k_time<8, A_, B_, 2>, dim3(h->S / h->time_cols), dim3(Tr), smem_r, h->stream, mode, E, out0, out1, h->ng, h->w, \
                                                                                 h->nlfilt, h->tw, h->twLog, tr);    \
            else                                                                                                      \
                launch_pdl(k_time<8, A_, B_, 1>, dim3(h->S / h->time_cols), dim3(Tr), smem_r, h->stream, mode, E, out0, out1, h->ng, h->w, \
                                                                                 h->nlfilt, h->tw, h->twLog, tr);    \
            return cudaGetLastError();                                                                             \
        }
        UPPE_TIME_CT(UPPE_TIME_RCASE)
#undef UPPE_TIME_RCASE
        if (occ2)
            launch_pdl(k_time<8, 0, -1, 2>, dim3(h->S / h->time_cols), dim3(Tr), smem_r, h->stream, mode, E, out0, out1, h->ng, h->w,
                                                                              h->nlfilt, h->tw, h->twLog, tr);
        else
            launch_pdl(k_time<8, 0, -1, 1>, dim3(h->S / h->time_cols), dim3(Tr), smem_r, h->stream, mode, E, out0, out1, h->ng, h->w,
                                                                              h->nlfilt, h->tw, h->twLog, tr);
        return cudaGetLastError();
    }
    if (h->time_spt == 16)
    {
#define UPPE_TIME_CASE(A_, B_)                                                                                      \
        if (tp.logM == A_ && tp.logC == B_) {                                                                          \
            launch_pdl(k_time<8, A_, B_>, dim3(h->S / C), dim3(T), smem, h->stream, mode, E, out0, out1, h->ng, h->w, h->nlfilt, \
                                                                            h->tw, h->twLog, tp);                    \
            return cudaGetLastError();                                                                             \
        }
        UPPE_TIME_CT(UPPE_TIME_CASE)
#undef UPPE_TIME_CASE
        launch_pdl(k_time<8>, dim3(h->S / C), dim3(T), smem, h->stream, mode, E, out0, out1, h->ng, h->w, h->nlfilt, h->tw,
                                                               h->twLog, tp);
    }
    else
        launch_pdl(k_time<16>, dim3(h->S / C), dim3(T), smem, h->stream, mode, E, out0, out1, h->ng, h->w, h->nlfilt, h->tw,
                                                                h->twLog, tp);
    return cudaGetLastError();
}

// =============================================================================================
// Adjoint of the time pass (vector-Jacobian product of J(E) for one evaluation).
//
// Given the forward input E(w) and the cotangent G(w) of the current J(w) (after the transposed
// forward transverse transform and conj of the RHS factor), writes the cotangent gE(w) of E(w):
//   P(w)   = rfft(p),  p = kappa e^3         J = filt (-i w P + Ppl / (0.1 - i w)),  Ppl = rfft(ne e)
//   gp(t)  = Re sum_k Gp_k e^{2 pi i k t/Nt},  Gp = conj(filt (-i w)) G   (transpose of rfft)
//   gpl(t) = Re sum_k Gl_k e^{2 pi i k t/Nt},  Gl = conj(filt / (0.1 - i w)) G
//   ge(t)  = 3 kappa e^2 gp + ne gpl + dr/de(t) hdt (Pfx(t) + Pfx(t-1)),
//            Pfx(j) = sum_{t <= j} gpl(t) e(t) ng w(t) exp(-S(t))   (transpose of the reverse scan)
//   gE(w)  = (1/Nt) W2 rfft(ge),  W2 = 1 at w = 0 and the last bin, 2 elsewhere   (transpose of irfft)
// and adds sum gp ng e^3 (the derivative with respect to chi3/nref) to *dred.
// =============================================================================================
__device__ __forceinline__ float ion_rate_deriv(const TimeParams& tp, float e, float r) {
    // d rate / d e = rate * d(log rate)/d(Em) * fconv * sign(e)
    const float em = fmaf(tp.fconv, fabsf(e), tp.cutoff);
    const float inv = __frcp_rn(em);
    float dl;
    if (tp.rate_form == UPPE_RATE_EXPLICIT) {
        // d/dEm [C_pow ln Em + C_exp / Em] = (C_pow - C_exp / Em) / Em, C_exp = ln2 * yexp
        dl = (tp.ypow - UPPE_LN2 * tp.yexp * inv) * inv;
    } else {
        const float L = __log2f(em) * UPPE_LN2;
        float dp = 5.f * tp.c2[5];
        dp = fmaf(dp, L, 4.f * tp.c2[4]);
        dp = fmaf(dp, L, 3.f * tp.c2[3]);
        dp = fmaf(dp, L, 2.f * tp.c2[2]);
        dp = fmaf(dp, L, tp.c2[1]);
        dl = dp * UPPE_LN2 * inv;
    }
    const float sg = (e > 0.f) ? 1.f : ((e < 0.f) ? -1.f : 0.f);
    return r * dl * tp.fconv * sg;
}

// even/odd packing of a half spectrum X(k) = f(k) into z for the M-point inverse FFT (rows of Z in
// the order sw).  Every thread reads the pair X(k), X(M-k) and writes only rows k and M-k of Z, so Z
// may hold X itself (packing in place).
template <class F>
__device__ __forceinline__ void pack_half_spectrum(float2* Z, int C, int logC, int M, const TwHalfShared& tws, F X,
                                                   int tid, int T, const RowSwizzle& sw) {
    const int npairs = (M / 2 + 1) * C;
    for (int it = tid; it < npairs; it += T) {
        const int c = it & (C - 1);
        const int k = it >> logC;
        float2 Xa = X(k, c), Xm = X(M - k, c);
        if (k == 0) {
            Xa.y = 0.f;
            Xm.y = 0.f;
        }
        const float2 t = cconj(tws.get(k));
        const float2 b = cconj(Xm);
        const float2 zk = cadd(cadd(Xa, b), cmul_i(cmul(t, csub(Xa, b))));
        float2 zm = zk;
        if (k != 0 && 2 * k != M) {
            const float2 t2 = make_float2(-t.x, t.y);
            const float2 b2 = cconj(Xa);
            zm = cadd(cadd(Xm, b2), cmul_i(cmul(t2, csub(Xm, b2))));
        }
        Z[sw(k) * C + c] = zk;
        if (k != 0 && 2 * k != M) Z[sw(M - k) * C + c] = zm;
    }
}

// 16 time samples per thread, 8 complex FFT elements per thread.  LOGM > 0: compile-time sizes
// M = 2^LOGM, C = 2^LOGC (the compile-time Stockham transforms, unrolled segment loops); LOGM = 0:
// sizes from the parameters.
//
// Shared layout: Ze [M+1][C] (e pairs, then ge pairs), Zn [M+1][C] (the raw E, then the rate pairs,
// then the pairs of the density exponent S), Zp [M+1][C] (gp pairs), Zl [M+1][C] (the raw G, then,
// in blocks with a nonzero rate, the gpl pairs), the half twiddle table, one float-float segment total per thread.  ne and
// ng w exp(-S) are formed from S where they are used.  Rows in the order of RowSwizzle.
// The three inverse transforms of the adjoint time pass share one out-of-line copy of the
// compile-time Stockham transform (inlined three times, with the segment loops, the kernel's
// code outgrew the instruction cache).
template <int LOGM, int LOGC>
__device__ __noinline__ void adj_inverse_fft_ct(float2* Z, const float2* twl, int tid) {
    fft_axis_ct<8, LOGM, LOGC, LOGM + 1>(Z, TwHalfSharedCT<LOGM + 1>{twl}, true, tid);
}

// RAMAN = 1 adds the rotational Raman response (the handle has a rotator): chi_R is recomputed by
// raman_pass and its transpose applied by raman_adjoint_pass; their contribution to the cotangent of
// e(t), chi_R gp + (dF/de) Fbar, goes to a fifth array Zr [M][C] that step 4 adds.  The segment totals
// then take 2T entries (float4 carries), and the pair tables Rs follow Zr.
template <int LOGM = 0, int LOGC = -1, int RAMAN = 0>
__global__ void __launch_bounds__(LOGM > 0 ? 256 : 512, RAMAN ? 1 : (LOGM > 0 ? 3 : 1)) k_time_adj(const float2* __restrict__ E,
                                                                   const float2* __restrict__ G,
                                                                   float2* __restrict__ gE,
                                                                   const float* __restrict__ ng,
                                                                   const float* __restrict__ wv,
                                                                   const float* __restrict__ filt,
                                                                   const float2* __restrict__ tw, int twLog,
                                                                   TimeParams tp, double* dred,
                                                                   const int* __restrict__ list) {
    extern __shared__ float2 sa[];
    constexpr bool CT = LOGM > 0;
    const int C = CT ? (1 << LOGC) : tp.C, logC = CT ? LOGC : tp.logC;
    const int Nt = CT ? (2 << LOGM) : tp.Nt, M = CT ? (1 << LOGM) : tp.M, S = tp.S;
    const int R = (M + 1) * C;
    float2* Ze = sa;
    float2* Zn = sa + R;
    float2* Zp = sa + 2 * R;
    float2* Zl = sa + 3 * R;
    float2* twl = sa + 4 * R;
    ffloat* tot = reinterpret_cast<ffloat*>(twl + (Nt >> 1));
    __shared__ double red_sh[32];
    const int tid = threadIdx.x, T = CT ? ((2 << LOGM) << LOGC) / 16 : (int)blockDim.x;
    float2* Zr = reinterpret_cast<float2*>(tot + 2 * T);  // RAMAN only
    float4* Rs = reinterpret_cast<float4*>(Zr + (((size_t)M * C + 1) & ~(size_t)1));
    const bool ionize = tp.rate_form != UPPE_RATE_NONE;
    const TwHalfShared tws{twl, tp.logNt};
    const RowSwizzle sw{logC <= 2 ? M - 1 : 0, logC == 0 ? 4 : 3};
    const auto inv_fft = [&](float2* Z) {
        if constexpr (CT)
            adj_inverse_fft_ct<LOGM, LOGC>(Z, twl, tid);
        else
            fft_axis_tw<8>(Z, tp.logM, logC, 1, C, tws, true, tid, T, -1, sw);
    };

    // One column group per pass of the loop: blockIdx.x alone, or (list != NULL) the groups list[1 ..
    // list[0]] taken in turn by the blocks of a smaller grid.
    for (int gi = (int)blockIdx.x;; gi += (int)gridDim.x) {
        size_t col0;
        if (list) {
            if (gi >= list[0]) break;
            col0 = (size_t)list[1 + gi] * C;
        } else {
            if (gi != (int)blockIdx.x) break;
            col0 = (size_t)blockIdx.x * C;
        }
        // ---- 1. stage E and G, recompute e(t), form the transposed-rfft inputs ----
        for (int it = tid; it < R; it += T) {
            const int c = it & (C - 1);
            const int k = it >> logC;
            cp_async8(&Zn[sw(k) * C + c], &E[(size_t)k * S + col0 + c]);
            cp_async8(&Zl[sw(k) * C + c], &G[(size_t)k * S + col0 + c]);
        }
        if constexpr (RAMAN != 0)
            for (int i = tid; i < 20 * tp.rot_pairs; i += T) cp_async16_time(&Rs[i], &tp.rot_tab[i]);
        asm volatile("cp.async.commit_group;\n" ::);
        for (int j = tid; j < (Nt >> 1); j += T) twl[j] = __ldg(&tw[j << (twLog - tp.logNt)]);
        asm volatile("cp.async.wait_group 0;\n" ::);
        __syncthreads();
        pack_half_spectrum(Ze, C, logC, M, tws, [&](int k, int c) { return Zn[sw(k) * C + c]; }, tid, T, sw);
        // Gp_k = W_k filt_k (i w_k) G_k ; Gl_k = W_k filt_k G_k / (0.1 + i w_k), W = 1/2 inside the band
        pack_half_spectrum(Zp, C, logC, M, tws, [&](int k, int c) {
            const float wk = wv[k];
            const float wt = (k == 0 || k == M) ? 1.f : 0.5f;
            return cscale(cmul_i(Zl[sw(k) * C + c]), wk * wt * filt[k]);
        }, tid, T, sw);
        __syncthreads();
        inv_fft(Ze);
        inv_fft(Zp);

        // ---- 2. forward sources along t (rates and the density exponent S), as in k_time ----
        const int c = tid & (C - 1);
        const int seg = tid >> logC;
        constexpr int MPS = 8;  // packed pairs (16 samples) per thread
        const int m0 = seg * MPS;
        const int t1 = 2 * (m0 + MPS);
        const float ngc = ng[col0 + c];
        const float kerr = ngc * tp.redchi3;
        const float inv = tp.inv_nt;
        const int plain = tp.plain;
        const auto ffsum = [plain](ffloat x, ffloat y) {
            if (plain) return ffloat{x.hi + y.hi, 0.f};
            return ff_add(x, y);
        };
        if constexpr (RAMAN != 0) {
            // chi_R of this thread's 16 samples (the forward's raman_pass on e), then the transpose of the
            // Raman map applied to ybar = gp e (P = chi e); Zr gets chi_R gp + (dF/de) Fbar with the
            // drive F = z^2 of the unnormalised field z = Nt e, dF/de = 2 Nt z
            float chiR[16], ybar[16], Fbar[16];
            raman_pass<16, false>(
                tp, Rs, tot, C, logC, T, tid, seg, ngc,
                [&](int k) {
                    const float2 zv = Ze[sw(m0 + k) * C + c];
                    return make_float2(zv.x * zv.x, zv.y * zv.y);
                },
                [&](int k, float chi0, float chi1) {
                    chiR[2 * k] = chi0;
                    chiR[2 * k + 1] = chi1;
                });
#pragma unroll
            for (int k = 0; k < MPS; ++k) {
                const float2 zv = Ze[sw(m0 + k) * C + c], gv = Zp[sw(m0 + k) * C + c];
                ybar[2 * k] = gv.x * zv.x * inv;
                ybar[2 * k + 1] = gv.y * zv.y * inv;
            }
            raman_adjoint_pass<16>(tp, Rs, tot, C, logC, T, tid, seg, ngc, ybar, Fbar);
            const float two_nt = 2.f * (float)Nt;
#pragma unroll
            for (int k = 0; k < MPS; ++k) {
                const float2 zv = Ze[sw(m0 + k) * C + c], gv = Zp[sw(m0 + k) * C + c];
                Zr[sw(m0 + k) * C + c] = make_float2(fmaf(chiR[2 * k], gv.x, two_nt * zv.x * Fbar[2 * k]),
                                                     fmaf(chiR[2 * k + 1], gv.y, two_nt * zv.y * Fbar[2 * k + 1]));
            }
        }
        // With no nonzero rate anywhere in the block the density, the plasma-current cotangent and the
        // rate-derivative terms are all zero: `ion` leaves them out (and the inverse FFT of gpl).
        bool ion = false;
        float r_next = 0.f;
        ffloat part = {0.f, 0.f};
        if (ionize) {
            if (t1 <= Nt - 2) r_next = ion_rate(tp, Ze[sw(t1 >> 1) * C + c].x * inv);
            float rn = r_next;
            bool live = r_next != 0.f;
#pragma unroll 1
            for (int j = MPS - 1; j >= 0; --j) {
                const int m = m0 + j;
                const float2 zv = Ze[sw(m) * C + c];
                const int t = 2 * m + 1;
                const float r1 = (t == Nt - 1) ? 0.f : ion_rate(tp, zv.y * inv);
                if (t <= Nt - 2) acc_add(part, tp.hdt * (r1 + rn), tp.plain);
                const float r0 = ion_rate(tp, zv.x * inv);
                acc_add(part, tp.hdt * (r0 + r1), tp.plain);
                live = live || r0 != 0.f || r1 != 0.f;
                rn = r0;
                Zn[sw(m) * C + c] = make_float2(r0, r1);
            }
            ion = __syncthreads_or(live ? 1 : 0) != 0;
        }
        if (ion) {
            ffloat Sacc = later_segments_sum(part, ffloat{0.f, 0.f}, tot, C, logC, T, tid, ffsum);
            float rn = r_next;
#pragma unroll 1
            for (int j = MPS - 1; j >= 0; --j) {
                const int m = m0 + j;
                const float2 rr = Zn[sw(m) * C + c];
                const int t = 2 * m + 1;
                if (t <= Nt - 2) acc_add(Sacc, tp.hdt * (rr.y + rn), tp.plain);
                const float S1 = ff_value(Sacc);
                acc_add(Sacc, tp.hdt * (rr.x + rr.y), tp.plain);
                rn = rr.x;
                Zn[sw(m) * C + c] = make_float2(ff_value(Sacc), S1);
            }
            // Gl over the raw G, which Zl has held since staging (its pack reads every G it overwrites)
            pack_half_spectrum(Zl, C, logC, M, tws, [&](int k, int c) {
                const float wk = wv[k];
                const float wt = (k == 0 || k == M) ? 1.f : 0.5f;
                const float rden = __frcp_rn(fmaf(wk, wk, tp.damping * tp.damping));
                return cscale(cmul(Zl[sw(k) * C + c], make_float2(tp.damping, -wk)), rden * wt * filt[k]);
            }, tid, T, sw);
            __syncthreads();  // the packed Gl is complete; the segment totals are reused below
            inv_fft(Zl);
        }

        // ---- 3. transposed scan: Pfx(j) = sum_{t <= j} gpl e a, a = ng w exp(-S), increasing t ----
        ffloat carry = {0.f, 0.f};
        if (ion) {
            ffloat part = {0.f, 0.f};
#pragma unroll 1
            for (int j = 0; j < MPS; ++j) {
                const int m = m0 + j;
                const float2 e2 = Ze[sw(m) * C + c], l2 = Zl[sw(m) * C + c], s2 = Zn[sw(m) * C + c];
                const float a0 = ngc * soft_window(2 * m, Nt, tp.wcut, tp.wwid) * expf(-s2.x);
                const float a1 = ngc * soft_window(2 * m + 1, Nt, tp.wcut, tp.wwid) * expf(-s2.y);
                acc_add(part, l2.x * e2.x * inv * a0, tp.plain);
                acc_add(part, l2.y * e2.y * inv * a1, tp.plain);
            }
            carry = earlier_segments_sum(part, ffloat{0.f, 0.f}, tot, C, logC, T, tid, ffsum);
        }
        // ---- 4. pointwise cotangent of e(t), written over the e pairs ----
        float dred_part = 0.f;
        {
            ffloat Pprev = carry;  // Pfx(t - 1)
#pragma unroll 1
            for (int j = 0; j < MPS; ++j) {
                const int m = m0 + j;
                const float2 e2 = Ze[sw(m) * C + c];
                const float2 p2 = Zp[sw(m) * C + c];
                float ge[2];
                const float ev[2] = {e2.x * inv, e2.y * inv};
                const float gp[2] = {p2.x, p2.y};
                float2 l2 = make_float2(0.f, 0.f), s2 = l2, r2 = l2;
                if constexpr (RAMAN != 0) r2 = Zr[sw(m) * C + c];
                if (ion) {
                    l2 = Zl[sw(m) * C + c];
                    s2 = Zn[sw(m) * C + c];
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int t = 2 * m + h;
                    const float e = ev[h];
                    float g = 3.f * kerr * e * e * gp[h] + (h ? r2.y : r2.x);
                    dred_part = fmaf(gp[h] * ngc * e * e, e, dred_part);
                    if (ion) {
                        const float gl = h ? l2.y : l2.x;
                        const float Sv = h ? s2.y : s2.x;
                        const float wv_t = soft_window(t, Nt, tp.wcut, tp.wwid);
                        const float ne = ngc * one_minus_exp_neg(Sv) * wv_t;
                        const float a = ngc * wv_t * expf(-Sv);
                        g = fmaf(ne, gl, g);
                        ffloat P = Pprev;
                        acc_add(P, gl * e * a, tp.plain);
                        if (t <= Nt - 2) {
                            const float r = ion_rate(tp, e);
                            const float gr = tp.hdt * (ff_value(P) + ff_value(Pprev));
                            g = fmaf(gr, ion_rate_deriv(tp, e, r), g);
                        }
                        Pprev = P;
                    }
                    ge[h] = g;
                }
                Ze[sw(m) * C + c] = make_float2(ge[0], ge[1]);
            }
        }
        // block reduction of the chi3 derivative (a block of fewer than 32 threads reduces through shared memory)
        double dsum = (double)dred_part;
        if (T >= 32) {
            for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
            if ((tid & 31) == 0) red_sh[tid >> 5] = dsum;
        } else {
            red_sh[tid] = dsum;
        }
        __syncthreads();
        if (tid == 0) {
            double b = 0.0;
            const int nred = (T >= 32) ? (T >> 5) : T;
            for (int i = 0; i < nred; ++i) b += red_sh[i];
            atomicAdd(dred, b);
        }

        // ---- 5. transpose of irfft: gE = (1/Nt) W2 rfft(ge) ----
        if constexpr (CT)
            fft_axis_ct<8, LOGM, LOGC, LOGM + 1>(Ze, TwHalfSharedCT<LOGM + 1>{twl}, false, tid);
        else
            fft_axis_tw<8>(Ze, tp.logM, logC, 1, C, tws, false, tid, T, -1, sw);
        for (int it = tid; it < (M + 1) * C; it += T) {
            const int cc = it & (C - 1);
            const int k = it >> logC;
            const int ka = k & (M - 1), kb = (M - k) & (M - 1);
            const float2 X = real_spectrum(Ze[sw(ka) * C + cc], Ze[sw(kb) * C + cc], tws.get(k));
            const float wt = (k == 0 || k == M) ? inv : 2.f * inv;
            if (tp.atc)  // the operand tiles of the Minv^T transform that follows
                tc_store_split(tp.atc, tp.atc_nwt, tp.atc_nkt, 0, k, (int)(col0 + cc), cscale(X, wt));
            else
                gE[(size_t)k * S + col0 + cc] = cscale(X, wt);
        }
        __syncthreads();  // the next group overwrites the shared arrays
    }
}

// The adjoint time-pass shapes with compile-time sizes: 2048 complex elements per block (256 threads).
#define UPPE_TIME_ADJ_CT(X) X(8, 3) X(9, 2) X(10, 1) X(11, 0)

cudaError_t uppe_configure_time_adj_kernel(size_t smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_time_adj<>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
#define UPPE_TIME_ADJ_CONF(A_, B_)                                                                              \
    if (e == cudaSuccess)                                                                                       \
        e = cudaFuncSetAttribute(k_time_adj<A_, B_>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    UPPE_TIME_ADJ_CT(UPPE_TIME_ADJ_CONF)
#undef UPPE_TIME_ADJ_CONF
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_adj<0, -1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    return e;
}

// Columns per block of the adjoint time pass: four (M + 1)-row arrays per column in shared memory,
// sized for three blocks per multiprocessor (2048 complex elements per block), 16 samples and 8
// FFT elements per thread.
static int adjoint_cols(const UppeHandle* h) {
    int c = 2048 / h->M;
    if (c < 1) c = 1;
    if (c > 16) c = 16;
    if (c > h->S) c = h->S;
    return c;
}

// The shared-memory adjoint time pass over every column group (list NULL), or over the groups
// list[1 .. list[0]] with a grid of at most nlist blocks that take them in turn.
static cudaError_t launch_time_adj_smem(UppeHandle* h, const float2* E, const float2* G, float2* gE, double* dred,
                                        const int* list, int nlist) {
    TimeParams tp = uppe_time_params(h);
    const int Ca = adjoint_cols(h);
    tp.C = Ca;
    tp.logC = ilog2_exact(Ca);
    tp.spt = 16;
    const int T = h->Nt * Ca / 16;
    const size_t smem = ((size_t)(h->M + 1) * 4 * Ca + h->Nt / 2) * sizeof(float2) + (size_t)T * sizeof(ffloat);
    int nblk = h->S / Ca;
    if (list && nlist < nblk) nblk = nlist;
    h->launches++;
    if (h->rot_pairs > 0) {  // the Raman response: 2T segment totals, Zr [M][C] (even length), the pair tables
        const size_t zr = (((size_t)h->M * Ca + 1) & ~(size_t)1) * sizeof(float2);
        const size_t smem_r = ((size_t)(h->M + 1) * 4 * Ca + h->Nt / 2) * sizeof(float2) +
                              (size_t)2 * T * sizeof(ffloat) + zr + (size_t)20 * h->rot_pairs * sizeof(float4);
        if (smem_r > 224 * 1024) return cudaErrorInvalidValue;
        k_time_adj<0, -1, 1><<<nblk, T, smem_r, h->stream>>>(E, G, gE, h->ng, h->w, h->nlfilt, h->tw, h->twLog, tp,
                                                          dred, list);
        return cudaGetLastError();
    }
#define UPPE_TIME_ADJ_CASE(A_, B_)                                                                             \
    if (tp.logM == A_ && tp.logC == B_) {                                                                      \
        k_time_adj<A_, B_><<<nblk, T, smem, h->stream>>>(E, G, gE, h->ng, h->w, h->nlfilt, h->tw, h->twLog, tp, dred, \
                                                        list);                                                 \
        return cudaGetLastError();                                                                             \
    }
    UPPE_TIME_ADJ_CT(UPPE_TIME_ADJ_CASE)
#undef UPPE_TIME_ADJ_CASE
    k_time_adj<><<<nblk, T, smem, h->stream>>>(E, G, gE, h->ng, h->w, h->nlfilt, h->tw, h->twLog, tp, dred, list);
    return cudaGetLastError();
}

// The adjoint time pass.  Where the register-resident form applies (timepass_adj_reg.cu) it takes
// the column groups without ionization and lists the others, which the shared-memory kernel then
// takes (a grid of three blocks per multiprocessor walking the list).
cudaError_t launch_time_adjoint(UppeHandle* h, const float2* E, const float2* G, float2* gE, double* dred) {
    if (time_adj_reg_ready(h) && adjoint_cols(h) == time_adj_reg_group(h->M)) {
        cudaError_t e = launch_time_adj_reg(h, E, G, gE, dred);
        if (e != cudaSuccess || h->cfg.rate_form == UPPE_RATE_NONE) return e;
        return launch_time_adj_smem(h, E, G, gE, dred, h->adj_live, 3 * h->num_sms);
    }
    return launch_time_adj_smem(h, E, G, gE, dred, nullptr, 0);
}
