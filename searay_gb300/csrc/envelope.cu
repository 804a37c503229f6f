// Time-axis pass of one paraxial (envelope) right-hand-side evaluation: update_current of SeaRay's
// paraxial solver (modules/paraxial_kernel.py:124-172) along t for every transverse point.
//
// The frequency axis holds N0 = 2^n absolute frequencies in FFT order.  One CTA takes C adjacent
// transverse points ("columns") and all N0 frequencies; 16 time samples per thread:
//   1. E(t) = ifft(i w A) and A(t) = ifft(A) (DtSpectral with sign -1, fft.cl:282-299; IFFT,
//      fft.cl:214-227) as two N0-point inverse FFTs in shared memory, left unnormalised (z = N0 E),
//   2. per time sample: the envelope rate of |E| (EnvelopeRate / EnvelopeRateSeries,
//      ionization.cl:46-69, 99-125), the electron density by the reverse trapezoid sum with
//      rate(N0-1) = 0 (ComputePlasmaDensity, ionization.cl:127-155), the rotational Raman chi
//      (AddChiParaxial, rotations.cl:30-78) when a rotator is set, then the Kerr chi
//      0.75 ng chi3/nref |E|^2 (paraxial.cl:124-138), P = chi E (paraxial.cl:140-148) and the plasma
//      current ne (|A|^2/4 - 1) A (paraxial.cl:110-122), written back in place,
//   3. two N0-point forward FFTs and J = -i w fft(P) + fft(Jpl) (DtSpectral with sign +1).  The
//      reference takes the inverse and forward transforms of -i w fft(P) around the plasma current
//      (paraxial_kernel.py:165-172); by linearity they cancel, so they are left out.
// The density sum is the blocked scan of the UPPE time pass (float-float in the mixed form).
#include <math.h>

#include "common.cuh"
#include "fft_smem.cuh"
#include "time_common.cuh"
#include "uppe_internal.h"

namespace {

constexpr int ENV_SPT = 16;  // time samples per thread

__device__ __forceinline__ float cnorm(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

// Shared layout: ZE [N0][C] (E, then P or chi), ZA [N0][C] (A, then Jpl or ne), the half twiddle
// table [N0/2], segment totals [2T], then with RAMAN the Raman chi [N0][C] (float) and the
// transition tables (20 float4 per pair).
template <bool RAMAN>
__global__ void __launch_bounds__(512) k_time_env(int mode, const float2* __restrict__ A, float2* __restrict__ out0,
                                                  float2* __restrict__ out1, const float* __restrict__ ng,
                                                  const float* __restrict__ wv, const float2* __restrict__ tw,
                                                  int twLog, TimeParams tp) {
    extern __shared__ float2 sm_env[];
    const int C = tp.C, logC = tp.logC, S = tp.S, N0 = tp.Nt, logN0 = tp.logNt;
    const int T = (int)blockDim.x, tid = threadIdx.x;
    const int R = N0 * C;
    float2* ZE = sm_env;
    float2* ZA = ZE + R;
    float2* twl = ZA + R;
    ffloat* tot = reinterpret_cast<ffloat*>(twl + (N0 >> 1));
    float* Zr = reinterpret_cast<float*>(tot + 2 * T);
    float4* Rs = reinterpret_cast<float4*>(Zr + R);
    const size_t col0 = (size_t)blockIdx.x * C;
    const bool ionize = tp.rate_form != UPPE_RATE_NONE;
    const TwHalfShared tws{twl, logN0};

    // ---- 1. stage A[k][c] (asynchronous copies), then i w A and the two inverse FFTs ----
    if (C >= 2) {
        const int hC = C >> 1;
        for (int it = tid; it < N0 * hC; it += T) {
            const int c2 = it & (hC - 1);
            const int k = it >> (logC - 1);
            cp_async16_time(&ZA[k * C + 2 * c2], &A[(size_t)k * S + col0 + 2 * c2]);
        }
    } else {
        for (int k = tid; k < N0; k += T) cp_async8(&ZA[k], &A[(size_t)k * S + col0]);
    }
    if constexpr (RAMAN)
        for (int i = tid; i < 20 * tp.rot_pairs; i += T) cp_async16_time(&Rs[i], &tp.rot_tab[i]);
    asm volatile("cp.async.commit_group;\n" ::);
    for (int j = tid; j < (N0 >> 1); j += T) twl[j] = __ldg(&tw[j << (twLog - logN0)]);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
    for (int it = tid; it < R; it += T) ZE[it] = cmul_i(cscale(ZA[it], __ldg(&wv[it >> logC])));
    __syncthreads();
    fft_axis_tw<16>(ZE, logN0, logC, 1, C, tws, true, tid, T);
    fft_axis_tw<16>(ZA, logN0, logC, 1, C, tws, true, tid, T);

    // ---- 2. sources over this thread's segment t0 .. t0 + 15 of column c ----
    const int c = tid & (C - 1);
    const int seg = tid >> logC;
    const int t0 = seg * ENV_SPT;
    const float inv = tp.inv_nt;
    const float ngc = ng[col0 + c];
    const float kerr = 0.75f * ngc * tp.redchi3;
    if constexpr (RAMAN) {  // F = |z|^2 (the scale (dalpha/hbar)/4/N0^2 is folded into cq)
        raman_pass<ENV_SPT, false>(
            tp, Rs, tot, C, logC, T, tid, seg, ngc,
            [&](int k) { return make_float2(cnorm(ZE[(t0 + 2 * k) * C + c]), cnorm(ZE[(t0 + 2 * k + 1) * C + c])); },
            [&](int k, float chi0, float chi1) {
                Zr[(t0 + 2 * k) * C + c] = chi0;
                Zr[(t0 + 2 * k + 1) * C + c] = chi1;
            });
    }
    float r[ENV_SPT];
    float r_next = 0.f;
    ffloat Sacc = {0.f, 0.f};
    if (ionize) {
        if (t0 + ENV_SPT <= N0 - 2) r_next = ion_rate(tp, sqrtf(cnorm(ZE[(t0 + ENV_SPT) * C + c])) * inv);
        ffloat part = {0.f, 0.f};
#pragma unroll
        for (int i = ENV_SPT - 1; i >= 0; --i) {
            const int t = t0 + i;
            r[i] = (t == N0 - 1) ? 0.f : ion_rate(tp, sqrtf(cnorm(ZE[t * C + c])) * inv);
            const float rn = (i == ENV_SPT - 1) ? r_next : r[i + 1];
            if (t <= N0 - 2) acc_add(part, tp.hdt * (r[i] + rn), tp.plain);
        }
        const int plain = tp.plain;
        Sacc = later_segments_sum(part, ffloat{0.f, 0.f}, tot, C, logC, T, tid, [plain](ffloat x, ffloat y) {
            if (plain) return ffloat{x.hi + y.hi, 0.f};
            return ff_add(x, y);
        });
    }
    __syncthreads();  // every read of the next segment's first sample (r_next) precedes the writes below
#pragma unroll
    for (int i = ENV_SPT - 1; i >= 0; --i) {
        const int t = t0 + i;
        const float2 e = cscale(ZE[t * C + c], inv), a = cscale(ZA[t * C + c], inv);
        float ne = 0.f;
        if (ionize) {
            const float rn = (i == ENV_SPT - 1) ? r_next : r[i + 1];
            if (t <= N0 - 2) acc_add(Sacc, tp.hdt * (r[i] + rn), tp.plain);
            ne = ngc * one_minus_exp_neg(ff_value(Sacc));
        }
        float chi = kerr * cnorm(e);
        if constexpr (RAMAN) chi = Zr[t * C + c] + chi;  // Raman first, then Kerr (paraxial_kernel.py:155-158)
        if (mode == TIME_J) {
            ZE[t * C + c] = cscale(e, chi);
            ZA[t * C + c] = cscale(a, ne * fmaf(0.25f, cnorm(a), -1.f));
        } else {
            ZE[t * C + c] = make_float2(chi, 0.f);
            ZA[t * C + c] = make_float2(ne, 0.f);
        }
    }
    __syncthreads();

    // ---- 3. forward FFTs and J = -i w P + Jpl (or the spectra of chi and ne) ----
    const bool two = ionize || mode == TIME_CHI_NE;
    fft_axis_tw<16>(ZE, logN0, logC, 1, C, tws, false, tid, T);
    if (two) fft_axis_tw<16>(ZA, logN0, logC, 1, C, tws, false, tid, T);
    for (int it = tid; it < R; it += T) {
        const int k = it >> logC;
        const size_t o = (size_t)k * S + col0 + (it & (C - 1));
        if (mode == TIME_J) {
            float2 J = cmul_mi(cscale(ZE[it], __ldg(&wv[k])));
            if (ionize) J = cadd(J, ZA[it]);
            out0[o] = J;
        } else {
            if (out0) out0[o] = ZE[it];
            if (out1) out1[o] = ionize ? ZA[it] : make_float2(0.f, 0.f);
        }
    }
}

}  // namespace

cudaError_t uppe_configure_env_kernel(size_t smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_time_env<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_env<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    return e;
}

size_t uppe_env_smem_bytes(const UppeHandle* h) {
    const size_t R = (size_t)h->Nt * h->time_cols, T = R / 16;
    size_t b = (2 * R + h->Nt / 2) * sizeof(float2) + 2 * T * sizeof(ffloat);
    if (h->rot_pairs > 0) b += R * sizeof(float) + (size_t)20 * h->rot_pairs * sizeof(float4);
    return b;
}

cudaError_t launch_time_env(UppeHandle* h, int mode, const float2* A, float2* out0, float2* out1) {
    const TimeParams tp = uppe_time_params(h);
    const int T = h->Nt * h->time_cols / 16;
    const size_t smem = uppe_env_smem_bytes(h);
    h->launches++;
    if (h->rot_pairs > 0)
        k_time_env<true><<<h->S / h->time_cols, T, smem, h->stream>>>(mode, A, out0, out1, h->ng, h->w, h->tw, h->twLog, tp);
    else
        k_time_env<false><<<h->S / h->time_cols, T, smem, h->stream>>>(mode, A, out0, out1, h->ng, h->w, h->tw, h->twLog, tp);
    return cudaGetLastError();
}
