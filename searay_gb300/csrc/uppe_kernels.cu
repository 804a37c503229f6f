// Kernels of the UPPE z-step on GB300: linear operator build, Cartesian transverse passes fused
// with the propagator phase and the RK4 stage update, the time-axis pass fused with the
// nonlinear sources, and the adaptive step-size reductions.
//
// Reference behaviour (SeaRay): modules/uppe_kernel.py:139-232 and the kernels it enqueues,
// kernels/uppe.cl:22-165, kernels/fft.cl:229-355,387-441, kernels/ionization.cl:22-155,
// kernels/paraxial.cl:27-58.
#include <math.h>
#include <stdio.h>

#include "common.cuh"
#include "fft_smem.cuh"
#include "uppe_internal.h"

// =============================================================================================
// Linear operator: kz = sqrt(w^2 (1 + chi0) - kr^2) with Im kz >= 0 and Re kz == 0 -> 1
// (uppe_kernel.py:81-84), stored per point as {hi(K), lo(K), Re kz, Im kz}, K = Re kz + kg.
// FP64 here: it runs once per material update, not per step.
// =============================================================================================
__device__ __forceinline__ void csqrt_principal(double ar, double ai, double* zr, double* zi) {
    if (ar == 0.0 && ai == 0.0) {
        *zr = 0.0;
        *zi = ai;
        return;
    }
    double t = sqrt(0.5 * (fabs(ar) + hypot(ar, ai)));
    if (ar >= 0.0) {
        *zr = t;
        *zi = ai / (2.0 * t);
    } else {
        *zr = fabs(ai) / (2.0 * t);
        *zi = copysign(t, ai);
    }
}

__global__ void k_build_operator(const double* __restrict__ w2n2, const double* __restrict__ kg,
                                 const double* __restrict__ kr2, float4* __restrict__ op, int N0, int S) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)N0 * S) return;
    int iw = (int)(idx / S);
    int s = (int)(idx - (size_t)iw * S);
    double ar = w2n2[2 * iw] - kr2[s];
    double ai = w2n2[2 * iw + 1];
    double zr, zi;
    csqrt_principal(ar, ai, &zr, &zi);
    if (zi < 0.0) {
        zr = -zr;
        zi = -zi;
    }
    if (zr == 0.0) {
        zr = 1.0;
        zi = 0.0;
    }
    double K = zr + kg[iw];
    float hi = (float)K;
    float lo = (float)(K - (double)hi);
    op[idx] = make_float4(hi, lo, (float)zr, (float)zi);
}

cudaError_t launch_build_operator(UppeHandle* h) {
    size_t n = h->P;
    int threads = 256;
    unsigned blocks = (unsigned)((n + threads - 1) / threads);
    h->launches++;
    k_build_operator<<<blocks, threads, 0, h->stream>>>(h->w2n2_d, h->kg_d, h->kr2_d, h->op, h->N0, h->S);
    return cudaGetLastError();
}

__global__ void k_operator_bounds(const float4* __restrict__ op, size_t n, float* red) {
    float mk = 0.f, mi = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float4 o = op[i];
        mk = fmaxf(mk, fabsf(o.x));
        mi = fmaxf(mi, o.w);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mk = fmaxf(mk, __shfl_xor_sync(0xffffffffu, mk, o));
        mi = fmaxf(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(reinterpret_cast<int*>(&red[0]), __float_as_int(mk));
        atomicMax(reinterpret_cast<int*>(&red[1]), __float_as_int(mi));
    }
}

cudaError_t launch_operator_bounds(UppeHandle* h) {
    size_t b = (h->P + 255) / 256;
    h->launches++;
    k_operator_bounds<<<(unsigned)(b < 1216 ? b : 1216), 256, 0, h->stream>>>(h->op, h->P, h->red);
    return cudaGetLastError();
}

// =============================================================================================
// Cartesian transverse passes: one CTA per frequency slice, the N1 x N2 slice held in shared
// memory and transformed in place (fft_smem.cuh).
// =============================================================================================
#define SLICE_ET 16

// E = IFFT2( i kz exp(i(kz+kg)z) q )   (uppe_kernel.py:210-213; uppe.cl:54-71,94-108; fft.cl:415-441)
// finish: A = IFFT2( exp(i(kz+kg)z) q ), E = i kz A   (uppe_kernel.py:250-253)
__global__ void __launch_bounds__(1024) k_real_cart(int mode, const float2* __restrict__ src,
                                                    const float4* __restrict__ op, float2* __restrict__ E,
                                                    float2* __restrict__ A_out, int logN1, int logN2,
                                                    const float2* __restrict__ tw, int twLog, StepArgs z) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int N2 = 1 << logN2;
    const size_t base = (size_t)blockIdx.x * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    for (int e = tid; e < S; e += nthr) {
        float4 o = op[base + e];
        float2 v = cmul(propagator_factor(o, pa, 1.f), src[base + e]);
        if (mode == REAL_E) v = cmul(make_float2(-o.w, o.z), v);
        sm[e] = v;
    }
    __syncthreads();
    fft_axis<SLICE_ET>(sm, logN2, logN1, N2, 1, tw, twLog, true, tid, nthr);  // along y
    fft_axis<SLICE_ET>(sm, logN1, logN2, 1, N2, tw, twLog, true, tid, nthr);  // along x
    const float scale = 1.0f / (float)S;
    for (int e = tid; e < S; e += nthr) {
        float2 v = cscale(sm[e], scale);
        if (mode == REAL_E) {
            E[base + e] = v;
        } else {
            if (A_out) A_out[base + e] = v;
            float4 o = op[base + e];
            E[base + e] = cmul(make_float2(-o.w, o.z), v);
        }
    }
}

// Forward transverse FFT of one slice of J (fft.cl:387-413), then the ODE right-hand side
// S = (i/2) exp(-i(kz+kg)z) J / Re kz (uppe.cl:73-91) and the RK4 bookkeeping of RKStage/RKFinish
// (uppe.cl:22-52) with the DC conditioner (uppe_kernel.py:127-137) on the stage estimate.
__device__ __forceinline__ void spec_update(int mode, size_t idx, float2 v, float4 o, float cond,
                                            float2* __restrict__ q_out, float2* __restrict__ qf,
                                            const float2* __restrict__ qi, float Cs, float Ce,
                                            const PhaseArgs& pa) {
    if (mode == SPEC_LOAD) {
        q_out[idx] = v;
        return;
    }
    float2 f = propagator_factor(o, pa, -1.f);
    float2 s = cscale(cmul_i(cmul(f, v)), 0.5f / o.z);
    switch (mode) {
        case SPEC_STORE_K:
            q_out[idx] = s;
            break;
        case SPEC_STAGE1: {
            float2 a = qi[idx];
            qf[idx] = cadd(a, cscale(s, Cs));
            q_out[idx] = cscale(cadd(a, cscale(s, Ce)), cond);
        } break;
        case SPEC_STAGE23: {
            float2 a = qi[idx];
            float2 b = qf[idx];
            qf[idx] = cadd(b, cscale(s, Cs));
            q_out[idx] = cscale(cadd(a, cscale(s, Ce)), cond);
        } break;
        default: {  // SPEC_FINISH
            float2 b = qf[idx];
            q_out[idx] = cscale(cadd(b, cscale(s, Cs)), cond);
        } break;
    }
}

__global__ void __launch_bounds__(1024) k_spec_cart(int mode, const float2* __restrict__ src,
                                                    const float4* __restrict__ op, float2* __restrict__ q_out,
                                                    float2* __restrict__ qf, const float2* __restrict__ qi,
                                                    float Cs, float Ce, int logN1, int logN2,
                                                    const float2* __restrict__ tw, int twLog, StepArgs z) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int N2 = 1 << logN2;
    const size_t base = (size_t)blockIdx.x * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int e = tid; e < S; e += nthr) sm[e] = src[base + e];
    __syncthreads();
    fft_axis<SLICE_ET>(sm, logN1, logN2, 1, N2, tw, twLog, false, tid, nthr);  // along x
    fft_axis<SLICE_ET>(sm, logN2, logN1, N2, 1, tw, twLog, false, tid, nthr);  // along y
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float cond = (blockIdx.x < 4) ? 0.f : 1.f;
    for (int e = tid; e < S; e += nthr) {
        const size_t idx = base + e;
        float4 o = (mode == SPEC_LOAD) ? make_float4(0, 0, 1, 0) : op[idx];
        spec_update(mode, idx, sm[e], o, cond, q_out, qf, qi, Cs, Ce, pa);
    }
}

static int slice_threads(const UppeHandle* h) { return h->S / SLICE_ET; }

cudaError_t uppe_configure_slice_kernels(size_t smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_real_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_spec_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    return e;
}

cudaError_t launch_real_cart(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z) {
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    size_t smem = (size_t)h->S * sizeof(float2);
    h->launches++;
    k_real_cart<<<h->N0, slice_threads(h), smem, h->stream>>>(mode, src, h->op, h->E, A_out, logN1, logN2, h->tw,
                                                               h->twLog, z);
    return cudaGetLastError();
}

cudaError_t launch_spec_cart(UppeHandle* h, int mode, const float2* src_real, float2* q_out, float2* qf_io,
                             const float2* qi, float Cs, float Ce, StepArgs z) {
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    size_t smem = (size_t)h->S * sizeof(float2);
    h->launches++;
    k_spec_cart<<<h->N0, slice_threads(h), smem, h->stream>>>(mode, src_real, h->op, q_out, qf_io, qi, Cs, Ce,
                                                               logN1, logN2, h->tw, h->twLog, z);
    return cudaGetLastError();
}

// =============================================================================================
// Time-axis pass.  One CTA takes C adjacent transverse points (columns) and all N0 frequencies:
//   1. irfft along w (fft.cl:257-280) via an M = Nt/2 point complex inverse FFT,
//   2. sources per time sample: Kerr chi = ng chi3/nref E^2 (uppe.cl:132-151), rate
//      (ionization.cl:22-44 / 71-97), electron density by a reverse trapezoid scan
//      (ionization.cl:127-155) in float-float, SoftTimeWindow (fft.cl:331-355), plasma current
//      ne E and polarisation chi E (uppe.cl:153-165),
//   3. one Nt point forward FFT of P + i Jpl, split into the two real spectra, and
//      J = -i w P + Jpl / (0.1 - i w) times the NL filter (uppe_kernel.py:169-186, fft.cl:282-329).
// Thread layout of the source phase: thread g handles column g mod C, time samples
// [32 s, 32 s + 32) with s = g / C, so every thread holds 32 consecutive samples.
// =============================================================================================
struct TimeParams {
    int Nt, logNt, M, logM, C, logC, S;
    float inv_nt, dt, redchi3, damping;
    int rate_form;
    float fconv, cutoff, lnpre, cpow, cexp, lnrc;
    float clog[6];
    int wcut, wwid;
    int plain;
};

__device__ __forceinline__ float ion_rate(const TimeParams& tp, float e) {
    if (tp.rate_form == UPPE_RATE_EXPLICIT) {
        float em = fmaf(tp.fconv, fabsf(e), tp.cutoff);
        return expf(tp.lnpre + tp.cpow * logf(em) + tp.cexp / em);
    } else {
        float L = logf(fmaf(tp.fconv, fabsf(e), tp.cutoff));
        float p = tp.clog[5];
        p = fmaf(p, L, tp.clog[4]);
        p = fmaf(p, L, tp.clog[3]);
        p = fmaf(p, L, tp.clog[2]);
        p = fmaf(p, L, tp.clog[1]);
        p = fmaf(p, L, tp.clog[0]);
        return expf(tp.lnrc + p);
    }
}

__device__ __forceinline__ float smooth5(float q) { return q * q * q * (10.f - 15.f * q + 6.f * q * q); }

__device__ __forceinline__ float soft_window(int i, int Ni, int cut, int wid) {
    float f = 1.f;
    if (i < cut || i > Ni - cut - 1) f = 0.f;
    if (i >= cut && i < cut + wid) f *= smooth5((float)(i - cut) / (float)wid);
    if (i <= Ni - cut - 1 && i > Ni - cut - wid - 1) f *= smooth5((float)(Ni - cut - 1 - i) / (float)wid);
    return f;
}

#define TIME_SPT 32  // time samples per thread in the source phase

__global__ void __launch_bounds__(256) k_time(int mode, const float2* __restrict__ E, float2* __restrict__ out0,
                                               float2* __restrict__ out1, const float* __restrict__ ng,
                                               const float* __restrict__ wv, const float* __restrict__ filt,
                                               const float2* __restrict__ tw, int twLog, TimeParams tp) {
    extern __shared__ float2 Y[];  // Nt * C complex; the first M * C hold Z during the irfft
    const int C = tp.C, logC = tp.logC, Nt = tp.Nt, M = tp.M, S = tp.S;
    ffloat* tot = reinterpret_cast<ffloat*>(Y + (size_t)Nt * C);
    const int tid = threadIdx.x, T = blockDim.x;
    const size_t col0 = (size_t)blockIdx.x * C;

    // ---- 1. Z[k] = (X[k] + conj X[M-k]) + i e^{2 pi i k/Nt} (X[k] - conj X[M-k]) ----
    const int npairs = (M / 2 + 1) * C;
    for (int it = tid; it < npairs; it += T) {
        const int c = it & (C - 1);
        const int k = it >> logC;
        float2 Xa = E[(size_t)k * S + col0 + c];
        float2 Xm = E[(size_t)(M - k) * S + col0 + c];
        if (k == 0) {
            Xa.y = 0.f;
            Xm.y = 0.f;
        }
        float2 t = __ldg(&tw[k << (twLog - tp.logNt)]);
        t.y = -t.y;  // e^{+2 pi i k / Nt}
        float2 b = cconj(Xm);
        Y[k * C + c] = cadd(cadd(Xa, b), cmul_i(cmul(t, csub(Xa, b))));
        if (k != 0 && 2 * k != M) {
            float2 t2 = make_float2(-t.x, t.y);  // e^{2 pi i (M-k)/Nt}
            float2 b2 = cconj(Xa);
            Y[(M - k) * C + c] = cadd(cadd(Xm, b2), cmul_i(cmul(t2, csub(Xm, b2))));
        }
    }
    __syncthreads();
    fft_axis<16>(Y, tp.logM, logC, 1, C, tw, twLog, true, tid, T);

    // ---- 2. sources ----
    const int c = tid & (C - 1);
    const int seg = tid >> logC;
    const int t0 = seg * TIME_SPT;
    float ev[TIME_SPT];
#pragma unroll
    for (int j = 0; j < TIME_SPT / 2; ++j) {
        float2 zv = Y[(t0 / 2 + j) * C + c];
        ev[2 * j] = zv.x * tp.inv_nt;
        ev[2 * j + 1] = zv.y * tp.inv_nt;
    }
    const float e_next = (t0 + TIME_SPT < Nt) ? Y[((t0 + TIME_SPT) / 2) * C + c].x * tp.inv_nt : 0.f;
    const float ngc = ng[col0 + c];
    const bool ionize = tp.rate_form != UPPE_RATE_NONE;
    const float hdt = 0.5f * tp.dt;
    ffloat carry = {0.f, 0.f};
    float r_next = 0.f;  // rate at t0 + 32 (zero at Nt - 1 and beyond)
    if (ionize) {
        r_next = (t0 + TIME_SPT <= Nt - 2) ? ion_rate(tp, e_next) : 0.f;
        ffloat part = {0.f, 0.f};
        float rn = r_next;
#pragma unroll
        for (int j = TIME_SPT - 1; j >= 0; --j) {
            const int t = t0 + j;
            const float r = (t == Nt - 1) ? 0.f : ion_rate(tp, ev[j]);
            if (t <= Nt - 2) {
                const float p = hdt * (r + rn);
                if (tp.plain)
                    part.hi += p;
                else
                    part = ff_add_f(part, p);
            }
            rn = r;
        }
        tot[tid] = part;
    }
    __syncthreads();  // every thread has read its Z samples; Y may now be overwritten
    if (ionize) {
        const int nseg = T >> logC;
        for (int s2 = seg + 1; s2 < nseg; ++s2) {
            ffloat v = tot[(s2 << logC) + c];
            if (tp.plain)
                carry.hi += v.hi;
            else
                carry = ff_add(carry, v);
        }
    }
    {
        ffloat Sacc = carry;
        float rn = r_next;
        const float kerr = ngc * tp.redchi3;
#pragma unroll
        for (int j = TIME_SPT - 1; j >= 0; --j) {
            const int t = t0 + j;
            const float e = ev[j];
            float ne = 0.f;
            if (ionize) {
                const float r = (t == Nt - 1) ? 0.f : ion_rate(tp, e);
                if (t <= Nt - 2) {
                    const float p = hdt * (r + rn);
                    if (tp.plain)
                        Sacc.hi += p;
                    else
                        Sacc = ff_add_f(Sacc, p);
                }
                rn = r;
                ne = -ngc * expm1f(-ff_value(Sacc)) * soft_window(t, Nt, tp.wcut, tp.wwid);
            }
            const float chi = kerr * e * e;
            float2 y;
            if (mode == TIME_J)
                y = make_float2(chi * e, ne * e);
            else
                y = make_float2(chi, ne);
            Y[t * C + c] = y;
        }
    }
    __syncthreads();
    fft_axis<32>(Y, tp.logNt, logC, 1, C, tw, twLog, false, tid, T);

    // ---- 3. split the packed spectra and form the current ----
    for (int it = tid; it < (M + 1) * C; it += T) {
        const int cc = it & (C - 1);
        const int k = it >> logC;
        float2 Ck = Y[k * C + cc];
        float2 Cm = cconj(Y[((Nt - k) & (Nt - 1)) * C + cc]);
        float2 P = cscale(cadd(Ck, Cm), 0.5f);
        // without a rate model the imaginary channel holds only rounding: keep it exactly zero
        float2 Q = (tp.rate_form != UPPE_RATE_NONE) ? cscale(cmul_mi(csub(Ck, Cm)), 0.5f) : make_float2(0.f, 0.f);
        const size_t o = (size_t)k * S + col0 + cc;
        if (mode == TIME_J) {
            const float wk = wv[k];
            float2 J = cmul_mi(cscale(P, wk));  // -i w P
            J = cadd(J, cdiv(Q, make_float2(tp.damping, -wk)));
            out0[o] = cscale(J, filt[k]);
        } else {
            if (out0) out0[o] = P;
            if (out1) out1[o] = Q;
        }
    }
}

cudaError_t uppe_configure_time_kernel(size_t smem_bytes) {
    return cudaFuncSetAttribute(k_time, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
}

cudaError_t launch_time_pass(UppeHandle* h, int mode, const float2* E, float2* out0, float2* out1) {
    const UppeConfig& c = h->cfg;
    TimeParams tp;
    tp.Nt = h->Nt;
    tp.logNt = ilog2_exact(h->Nt);
    tp.M = h->M;
    tp.logM = ilog2_exact(h->M);
    tp.C = h->time_cols;
    tp.logC = ilog2_exact(h->time_cols);
    tp.S = h->S;
    tp.inv_nt = (float)(1.0 / (double)h->Nt);
    tp.dt = (float)c.dt;
    tp.redchi3 = (float)c.chi3_over_nref;
    tp.damping = (float)c.damping;
    tp.rate_form = c.rate_form;
    tp.fconv = (float)c.field_conv;
    tp.cutoff = (float)c.field_cutoff;
    tp.lnpre = (c.rate_form == UPPE_RATE_EXPLICIT) ? (float)log(c.rate_conv * c.c_pre) : 0.f;
    tp.cpow = (float)c.c_pow;
    tp.cexp = (float)c.c_exp;
    tp.lnrc = (c.rate_conv > 0) ? (float)log(c.rate_conv) : 0.f;
    for (int i = 0; i < 6; ++i) tp.clog[i] = (float)c.clog[i];
    tp.wcut = c.window_cutoff;
    tp.wwid = c.window_width;
    tp.plain = (c.precision == UPPE_PREC_FP32);
    const int T = h->Nt * h->time_cols / TIME_SPT;
    const size_t smem = (size_t)h->Nt * h->time_cols * sizeof(float2) + (size_t)T * sizeof(ffloat);
    h->launches++;
    k_time<<<h->S / h->time_cols, T, smem, h->stream>>>(mode, E, out0, out1, h->ng, h->w, h->nlfilt, h->tw, h->twLog,
                                                         tp);
    return cudaGetLastError();
}

// =============================================================================================
// Adaptive step size (uppe_kernel.py:217-232, paraxial.cl:27-58): amin = 1e-2 max|q|, then
// dz = min over the grid of dphi / (0.5 dphi/L + |Im(S q*)|/(|q|^2+amin^2) - min(Re(S q*)/(..),0)).
// =============================================================================================
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void k_absmax(const float2* __restrict__ q, size_t n, float* red) {
    __shared__ float sred[32];
    float m = 0.f;
    int bad = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float2 v = q[i];
        float a = sqrtf(v.x * v.x + v.y * v.y);
        if (!isfinite(a)) bad = 1;
        m = fmaxf(m, a);
    }
    m = warp_max(m);
    bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = (threadIdx.x < (blockDim.x >> 5)) ? sred[threadIdx.x] : 0.f;
        v = warp_max(v);
        if (threadIdx.x == 0) atomicMax(reinterpret_cast<int*>(&red[0]), __float_as_int(v));
    }
    if (bad && (threadIdx.x & 31) == 0) atomicExch(reinterpret_cast<int*>(&red[2]), 1);
}

__global__ void k_step_size(const float2* __restrict__ q, const float2* __restrict__ k, size_t n, float* red,
                            float minRate, float dphi, float rel_amin) {
    __shared__ float sred[32];
    const float amin = rel_amin * red[0];
    const float amin2 = amin * amin;
    float m = INFINITY;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float2 Q = q[i], Sv = k[i];
        float den = Q.x * Q.x + Q.y * Q.y + amin2;
        float alpha = (Q.x * Sv.x + Q.y * Sv.y) / den;
        float keff = (Q.x * Sv.y - Q.y * Sv.x) / den;
        float K = minRate + fabsf(keff) - (alpha < 0.f ? alpha : 0.f);
        m = fminf(m, dphi / K);
    }
    m = warp_min(m);
    if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = (threadIdx.x < (blockDim.x >> 5)) ? sred[threadIdx.x] : INFINITY;
        v = warp_min(v);
        if (threadIdx.x == 0) atomicMin(reinterpret_cast<int*>(&red[1]), __float_as_int(v));
    }
}

static unsigned reduce_blocks(size_t n) {
    size_t b = (n + 255) / 256;
    return (unsigned)(b < 152 * 8 ? b : 152 * 8);
}

cudaError_t launch_absmax(UppeHandle* h, const float2* q) {
    h->launches++;
    k_absmax<<<reduce_blocks(h->P), 256, 0, h->stream>>>(q, h->P, h->red);
    return cudaGetLastError();
}

cudaError_t launch_step_size(UppeHandle* h, const float2* q, const float2* k, double L, double dphi,
                             double rel_amin) {
    float minRate = (float)(0.5 * dphi / L);
    h->launches++;
    k_step_size<<<reduce_blocks(h->P), 256, 0, h->stream>>>(q, k, h->P, h->red, minRate, (float)dphi,
                                                             (float)rel_amin);
    return cudaGetLastError();
}

// First RK stage once dz is known: q = cond(qi + Ce k1), qf = qi + Cs k1 (uppe.cl:22-39).
__global__ void k_apply_stage1(const float2* __restrict__ qi, const float2* __restrict__ k1, float2* __restrict__ q,
                               float2* __restrict__ qf, size_t n, int S, float Cs, float Ce) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float2 a = qi[i], s = k1[i];
        float cond = (i < (size_t)4 * S) ? 0.f : 1.f;
        qf[i] = cadd(a, cscale(s, Cs));
        q[i] = cscale(cadd(a, cscale(s, Ce)), cond);
    }
}

cudaError_t launch_apply_stage1(UppeHandle* h, float Cs, float Ce) {
    h->launches++;
    k_apply_stage1<<<reduce_blocks(h->P) * 2, 256, 0, h->stream>>>(h->qi, h->k1, h->q, h->qf, h->P, h->S, Cs, Ce);
    return cudaGetLastError();
}

// E = i kz A, applied point by point on a real-space array (uppe_kernel.py:252-253).
__global__ void k_ikz(const float2* __restrict__ A, const float4* __restrict__ op, float2* __restrict__ E, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float4 o = op[i];
        E[i] = cmul(make_float2(-o.w, o.z), A[i]);
    }
}

cudaError_t launch_ikz(UppeHandle* h, const float2* A, float2* E) {
    h->launches++;
    k_ikz<<<reduce_blocks(h->P) * 2, 256, 0, h->stream>>>(A, h->op, E, h->P);
    return cudaGetLastError();
}
