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
#include "hankel_tc.cuh"
#include "rk_stage.cuh"
#include "uppe_internal.h"

// =============================================================================================
// Linear operator: kz = sqrt(w^2 (1 + chi0) - kr^2) with Im kz >= 0 and Re kz == 0 -> 1
// (uppe_kernel.py:81-84), stored per point as K = Re kz + kg in float-float (and Im kz when the
// medium absorbs).  FP64 here: it runs once per material update, not per step.
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
                                 const double* __restrict__ kr2, float2* __restrict__ opK, float* __restrict__ opKi,
                                 int N0, int S) {
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
    opK[idx] = make_float2(hi, lo);
    opKi[idx] = (float)zi;
}

// Paraxial envelope operator kz = (f(w) - kperp^2) / (2 k0(w)) (paraxial_kernel.py:79-88), FP64;
// K holds Re kz (no Galilean term).
__global__ void k_build_operator_env(const double* __restrict__ fw, const double* __restrict__ k0,
                                     const double* __restrict__ kr2, float2* __restrict__ opK, float* __restrict__ opKi,
                                     int N0, int S) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)N0 * S) return;
    int iw = (int)(idx / S);
    int s = (int)(idx - (size_t)iw * S);
    const double r = 0.5 / k0[iw];
    const double K = (fw[2 * iw] - kr2[s]) * r;
    const float hi = (float)K;
    opK[idx] = make_float2(hi, (float)(K - (double)hi));
    opKi[idx] = (float)(fw[2 * iw + 1] * r);
}

// The same operator for a real medium (Im w^2 (1 + chi0) = 0 at every w), mostly on the FP32 units:
// a = w^2 n^2 - kperp^2 in FP64, kz = sqrt(a) as float-float (the FP32 root plus one Newton step from
// the residual a - r^2 taken in FP64, about 2^-48 relative, the rounding of the FP64 form), K = kz + kg.
// The reference's guards for a real argument: a <= 0 gives Re kz = 0, replaced by kz = 1
// (uppe_kernel.py:83-84); Im kz = 0.
__global__ void k_build_operator_real(const double* __restrict__ w2n2, const float2* __restrict__ kg2,
                                      const double* __restrict__ kr2, float2* __restrict__ opK,
                                      float* __restrict__ opKi, int N0, int S) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)N0 * S) return;
    int iw = (int)(idx / S);
    int s = (int)(idx - (size_t)iw * S);
    const double a = w2n2[2 * iw] - kr2[s];
    ffloat kz;
    if (a > 0.0) {
        const float r = sqrtf((float)a);
        // the residual a - r^2 in FP64 (r^2 of an FP32 r is exact in FP64), then one Newton step
        const double res = a - (double)r * (double)r;
        kz = ff_two_sum(r, (float)res / (2.f * r));
    } else {
        kz = ffloat{1.f, 0.f};
    }
    const float2 kg = kg2[iw];
    const ffloat K = ff_add(kz, ffloat{kg.x, kg.y});
    opK[idx] = make_float2(K.hi, K.lo);
    opKi[idx] = 0.f;
}

cudaError_t launch_build_operator(UppeHandle* h) {
    size_t n = h->P;
    int threads = 256;
    unsigned blocks = (unsigned)((n + threads - 1) / threads);
    h->launches++;
    if (!h->cfg.envelope && !h->complex_medium) {
        k_build_operator_real<<<blocks, threads, 0, h->stream>>>(h->w2n2_d, h->kg2, h->kr2_d, h->opK, h->opKi, h->N0,
                                                                  h->S);
        return cudaGetLastError();
    }
    if (h->cfg.envelope)
        k_build_operator_env<<<blocks, threads, 0, h->stream>>>(h->w2n2_d, h->kg_d, h->kr2_d, h->opK, h->opKi, h->N0,
                                                                h->S);
    else
        k_build_operator<<<blocks, threads, 0, h->stream>>>(h->w2n2_d, h->kg_d, h->kr2_d, h->opK, h->opKi, h->N0, h->S);
    return cudaGetLastError();
}

__global__ void k_operator_bounds(const float2* __restrict__ opK, const float* __restrict__ opKi, size_t n, float* red) {
    float mk = 0.f, mi = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        mk = fmaxf(mk, fabsf(opK[i].x));
        mi = fmaxf(mi, fabsf(opKi[i]));  // |Im kz|: the envelope operator has no sign guard
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
    k_operator_bounds<<<(unsigned)(b < 1216 ? b : 1216), 256, 0, h->stream>>>(h->opK, h->opKi, h->P, h->red);
    return cudaGetLastError();
}

static unsigned reduce_blocks_host(size_t n) {
    size_t b = (n + 255) / 256;
    return (unsigned)(b < 152 * 8 ? b : 152 * 8);
}

OpView uppe_op_view(const UppeHandle* h) {
    OpView v;
    v.K = h->opK;
    v.ki = h->complex_medium ? h->opKi : nullptr;
    v.kg = h->kg2;
    v.envelope = h->cfg.envelope;
    v.ncond = h->cfg.envelope ? 0 : 4;
    return v;
}

// =============================================================================================
// Cartesian transverse passes: one CTA per frequency slice, the N1 x N2 slice held in shared
// memory and transformed in place (fft_smem.cuh).
// =============================================================================================
#define SLICE_ET 16

// Shared-memory slice layout: row x of the N1 x N2 slice starts at x * (N2 + 1), so that 32 lanes
// walking down a column (stride N2 + 1 float2) hit distinct banks.  Both FFT axes map consecutive
// lanes to consecutive transforms (rows for the y transform, columns for the x transform).
__device__ __forceinline__ int slice_pad(int e, int logN2) { return e + (e >> logN2); }

__device__ __forceinline__ void cp_async8_slice(void* smem_dst, const void* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc));
}

__device__ __forceinline__ void slice_load_async(float2* sm, const float2* __restrict__ src, int S, int logN2, int tid,
                                                 int nthr) {
    for (int e = tid; e < S; e += nthr) cp_async8_slice(&sm[slice_pad(e, logN2)], &src[e]);
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
}

__device__ __forceinline__ void slice_inverse(float2* sm, int logN1, int logN2, const float2* __restrict__ tw,
                                              int twLog, int tid, int nthr) {
    const int PS = (1 << logN2) + 1;
    fft_axis_tw<SLICE_ET>(sm, logN2, logN1, PS, 1, TwGlobal{tw, twLog}, true, tid, nthr, 1);  // along y
    fft_axis_tw<SLICE_ET>(sm, logN1, logN2, 1, PS, TwGlobal{tw, twLog}, true, tid, nthr, 1);  // along x
}

__device__ __forceinline__ void slice_forward(float2* sm, int logN1, int logN2, const float2* __restrict__ tw,
                                              int twLog, int tid, int nthr) {
    const int PS = (1 << logN2) + 1;
    fft_axis_tw<SLICE_ET>(sm, logN1, logN2, 1, PS, TwGlobal{tw, twLog}, false, tid, nthr, 1);  // along x
    fft_axis_tw<SLICE_ET>(sm, logN2, logN1, PS, 1, TwGlobal{tw, twLog}, false, tid, nthr, 1);  // along y
}

// E = IFFT2( i kz exp(i(kz+kg)z) q )   (uppe_kernel.py:210-213; uppe.cl:54-71,94-108; fft.cl:415-441)
// finish: A = IFFT2( exp(i(kz+kg)z) q ), E = i kz A   (uppe_kernel.py:250-253)
// apply1: q = cond(qi + Ce k1), qf = qi + Cs k1 (uppe.cl:22-39), then E from q.
__global__ void __launch_bounds__(1024) k_real_cart(int mode, const float2* __restrict__ src, OpView opv,
                                                    float2* __restrict__ E, float2* __restrict__ A_out,
                                                    const float2* __restrict__ k1, float2* __restrict__ qf,
                                                    float Cs, float Ce, int logN1, int logN2,
                                                    const float2* __restrict__ tw, int twLog, StepArgs z) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int iw = blockIdx.x;
    const size_t base = (size_t)iw * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float2 kgw = opv.kg[iw];
    const float cond = (iw < opv.ncond) ? 0.f : 1.f;
    if (mode != REAL_APPLY1) slice_load_async(sm, src + base, S, logN2, tid, nthr);
#pragma unroll 4
    for (int e = tid; e < S; e += nthr) {
        const OpPoint o = op_at(opv, base + e, kgw);
        const int pe = slice_pad(e, logN2);
        float2 v;
        if (mode == REAL_APPLY1) {
            const float2 a = src[base + e], s = k1[base + e];
            qf[base + e] = cadd(a, cscale(s, Cs));
            v = cscale(cadd(a, cscale(s, Ce)), cond);
        } else {
            v = sm[pe];
        }
        v = cmul(propagator_factor(o, pa, 1.f), v);
        if (mode != REAL_FINISH) v = op_field(opv, o, v);
        sm[pe] = v;
    }
    __syncthreads();
    slice_inverse(sm, logN1, logN2, tw, twLog, tid, nthr);
    const float scale = 1.0f / (float)S;
#pragma unroll 4
    for (int e = tid; e < S; e += nthr) {
        const float2 v = cscale(sm[slice_pad(e, logN2)], scale);
        if (mode != REAL_FINISH) {
            E[base + e] = v;
        } else {
            if (A_out) A_out[base + e] = v;
            const OpPoint o = op_at(opv, base + e, kgw);
            E[base + e] = op_field(opv, o, v);
        }
    }
}

__global__ void __launch_bounds__(1024) k_spec_cart(int mode, const float2* __restrict__ src, OpView opv,
                                                    float2* __restrict__ q_out, float2* __restrict__ qf,
                                                    const float2* __restrict__ qi, float Cs, float Ce, int logN1,
                                                    int logN2, const float2* __restrict__ tw, int twLog, StepArgs z) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int iw = blockIdx.x;
    const size_t base = (size_t)iw * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    slice_load_async(sm, src + base, S, logN2, tid, nthr);
    slice_forward(sm, logN1, logN2, tw, twLog, tid, nthr);
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float cond = (iw < opv.ncond) ? 0.f : 1.f;
    const float2 kgw = (mode == SPEC_LOAD) ? make_float2(0.f, 0.f) : opv.kg[iw];
#pragma unroll 4
    for (int e = tid; e < S; e += nthr) {
        const size_t idx = base + e;
        OpPoint o;
        if (mode != SPEC_LOAD) o = op_at(opv, idx, kgw);
        spec_update(mode, idx, sm[slice_pad(e, logN2)], o, cond, q_out, qf, qi, Cs, Ce, pa, true);
    }
}

// Fused evaluation tail: forward 2D FFT of J, S and the RK stage, then E for the next evaluation
// from the new stage estimate: E = IFFT2(i kz exp(i(kz+kg) z_next) qw).  qw itself is written only
// by the last stage (as the next step's qi); the other stages keep it in shared memory.
__global__ void __launch_bounds__(1024) k_fused_cart(int mode, const float2* __restrict__ J, OpView opv,
                                                     float2* __restrict__ qi_out, float2* __restrict__ qf,
                                                     const float2* __restrict__ qi, float2* __restrict__ E, float Cs,
                                                     float Ce, int logN1, int logN2, const float2* __restrict__ tw,
                                                     int twLog, StepArgs z_rhs, StepArgs z_next, int next_wave) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int iw = blockIdx.x;
    const size_t base = (size_t)iw * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (tid == 0) {
        // operator and RK state of this slice are read after the forward FFT: fetch them into L2 now;
        // also the current of the slice a CTA of the next wave will take
        const size_t fb = (size_t)S * sizeof(float2);
        prefetch_l2(opv.K + base, fb);
        if (mode != SPEC_FINISH) prefetch_l2(qi + base, fb);
        if (mode != SPEC_STAGE1) prefetch_l2(qf + base, fb);
        if ((int)(iw + next_wave) < (int)gridDim.x) prefetch_l2(J + base + (size_t)next_wave * S, fb);
    }
    slice_load_async(sm, J + base, S, logN2, tid, nthr);
    slice_forward(sm, logN1, logN2, tw, twLog, tid, nthr);
    const PhaseArgs pr{z_rhs.zhi, z_rhs.zlo, z_rhs.plain};
    const PhaseArgs pn{z_next.zhi, z_next.zlo, z_next.plain};
    const float cond = (iw < opv.ncond) ? 0.f : 1.f;
    const float2 kgw = opv.kg[iw];
    const bool last = (mode == SPEC_FINISH);
#pragma unroll 2
    for (int e = tid; e < S; e += nthr) {
        const size_t idx = base + e;
        const int pe = slice_pad(e, logN2);
        const OpPoint o = op_at(opv, idx, kgw);
        const float2 qw = spec_update(mode, idx, sm[pe], o, cond, qi_out, qf, qi, Cs, Ce, pr, last);
        sm[pe] = op_field(opv, o, cmul(propagator_factor(o, pn, 1.f), qw));
    }
    __syncthreads();
    slice_inverse(sm, logN1, logN2, tw, twLog, tid, nthr);
    const float scale = 1.0f / (float)S;
#pragma unroll 4
    for (int e = tid; e < S; e += nthr) E[base + e] = cscale(sm[slice_pad(e, logN2)], scale);
}

// ---- adjoint (vector-Jacobian products) of the Cartesian slice passes ----
// ADJ_S:    out = F^H( conj(D2) in ),  D2 = (i/2) exp(-i(kz+kg)z) / Re kz   (cotangent of the RHS
//           S -> cotangent of the current J before the forward transform; F^H = unnormalised inverse FFT)
// ADJ_LOAD: out = F^H in                                                     (transpose of the load kspacex)
// ADJ_E:    out = conj(D0) (1/N) F in,  D0 = i kz exp(i(kz+kg)z)           (cotangent of E -> of q)
// ADJ_FIN:  out = conj(exp(i(kz+kg)z)) (1/N) F in                           (cotangent of the finish A -> of q)
__global__ void __launch_bounds__(1024) k_adj_cart(int mode, const float2* __restrict__ in, OpView opv,
                                                   float2* __restrict__ out, int logN1, int logN2,
                                                   const float2* __restrict__ tw, int twLog, StepArgs z) {
    extern __shared__ float2 sm[];
    const int S = 1 << (logN1 + logN2);
    const int iw = blockIdx.x;
    const size_t base = (size_t)iw * S;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const float2 kgw = opv.kg[iw];
    slice_load_async(sm, in + base, S, logN2, tid, nthr);
    if (mode == ADJ_S || mode == ADJ_LOAD) {
        if (mode == ADJ_S) {
            for (int e = tid; e < S; e += nthr) {
                const OpPoint o = op_at(opv, base + e, kgw);
                const int pe = slice_pad(e, logN2);
                // conj(D2) = (-i/2) conj(exp(-iKz) exp(Ki z)) / Re kz
                const float2 f = cconj(propagator_factor(o, pa, -1.f));
                sm[pe] = cscale(cmul_mi(cmul(f, sm[pe])), 0.5f / o.kzr);
            }
            __syncthreads();
        }
        slice_inverse(sm, logN1, logN2, tw, twLog, tid, nthr);
        for (int e = tid; e < S; e += nthr) out[base + e] = sm[slice_pad(e, logN2)];
    } else {
        slice_forward(sm, logN1, logN2, tw, twLog, tid, nthr);
        const float scale = 1.0f / (float)S;
        for (int e = tid; e < S; e += nthr) {
            const OpPoint o = op_at(opv, base + e, kgw);
            float2 v = cmul(cconj(propagator_factor(o, pa, 1.f)), cscale(sm[slice_pad(e, logN2)], scale));
            if (mode == ADJ_E) v = cmul(cconj(op_ikz(o)), v);
            out[base + e] = v;
        }
    }
}

cudaError_t launch_adj_cart(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
    if (h->slice_big) return launch_adj_big(h, mode, in, out, z);
    if (h->slice_reg) return launch_adj_reg(h, mode, in, out, z);
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    h->launches++;
    k_adj_cart<<<h->N0, h->S / SLICE_ET, (size_t)(h->S + h->N1) * sizeof(float2), h->stream>>>(
        mode, in, uppe_op_view(h), out, logN1, logN2, h->tw, h->twLog, z);
    return cudaGetLastError();
}

// RK4 adjoint bookkeeping, point by point (the conditioner C zeroes w-bins 0-3):
//   init:    lam_f = C lam_out, acc = lam_f, lam_k = a_f lam_f
//   combine: acc += C mu, lam_k = a_f lam_f + a_mu C mu
//   final:   lam_in = acc + mu
__global__ void k_adj_rk(int mode, const float2* __restrict__ lam_out, float2* __restrict__ lam_f,
                         float2* __restrict__ acc, float2* __restrict__ lam_k, const float2* __restrict__ mu,
                         float2* __restrict__ lam_in, float a_f, float a_mu, size_t n, int S) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float cond = (i < (size_t)4 * S) ? 0.f : 1.f;
        if (mode == 0) {
            const float2 lf = cscale(lam_out[i], cond);
            lam_f[i] = lf;
            acc[i] = lf;
            lam_k[i] = cscale(lf, a_f);
        } else if (mode == 1) {
            const float2 cm = cscale(mu[i], cond);
            acc[i] = cadd(acc[i], cm);
            lam_k[i] = cadd(cscale(lam_f[i], a_f), cscale(cm, a_mu));
        } else {
            lam_in[i] = cadd(acc[i], mu[i]);
        }
    }
}

// The spectral update of every point from the transformed current C (the ODE right-hand side and the
// RK stage of spec_update), as a separate pass after a tensor-core transform that stored C: many
// warps per multiprocessor hide the latency of its operand reads, which the GEMM's own epilogue,
// with one block per multiprocessor, does not.  With nx.Atc set (one azimuthal node) it also writes
// the operand of the next inverse transform, i kz exp(i (kz + kg) z_next) qw of the new stage
// estimate qw, split into the transform's bf16 tiles (zero beyond the Nk radial modes), which
// k_hankel_tc_prep would otherwise form from qw.
__global__ void k_spec_point(int mode, const float2* __restrict__ C, OpView opv, float2* __restrict__ q_out,
                             float2* __restrict__ qf, const float2* __restrict__ qi, float Cs, float Ce, StepArgs z,
                             size_t n, int S, TcNext nx) {
    pdl_begin();
    const PhaseArgs pa{z.zhi, z.zlo, z.plain};
    const PhaseArgs pn{nx.z.zhi, nx.z.zlo, nx.z.plain};
    // idx = w S + k: (w, k) advance with the grid stride (one division per thread, not per point)
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t idx0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int dw = (int)(stride / (size_t)S), dk = (int)(stride - (size_t)dw * S);
    int w = (int)(idx0 / (size_t)S), k = (int)(idx0 - (size_t)w * S);
    for (size_t idx = idx0; idx < n; idx += stride) {
        const float cond = (w < opv.ncond) ? 0.f : 1.f;
        const OpPoint o = op_at(opv, idx, opv.kg[w]);
        const float2 qw = spec_update(mode, idx, C[idx], o, cond, q_out, qf, qi, Cs, Ce, pa, true);
        if (nx.Atc) {
            float2 a = make_float2(0.f, 0.f);
            if (k < nx.Nk) a = op_field(opv, o, cmul(propagator_factor(o, pn, 1.f), qw));
            tc_store_split(nx.Atc, nx.nwt, nx.nkt, 0, w, k, a);
        }
        w += dw;
        k += dk;
        if (k >= S) {
            k -= S;
            ++w;
        }
    }
}

cudaError_t launch_spec_point(UppeHandle* h, int mode, const float2* C, float2* q_out, float2* qf, const float2* qi,
                              float Cs, float Ce, StepArgs z, const StepArgs* z_next) {
    TcNext nx{};
    if (z_next) nx = hankel_tc_next(h, *z_next);
    h->launches++;
    launch_pdl(k_spec_point, dim3(reduce_blocks_host(h->P)), dim3(256), 0, h->stream, mode, C, uppe_op_view(h), q_out,
               qf, qi, Cs, Ce, z, h->P, h->S, nx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && z_next) {
        h->atc_next = 1;
        h->atc_next_src = q_out;
        h->atc_next_z = *z_next;
        h->atc_next_mat = h->mat_version;
    }
    return e;
}

cudaError_t launch_adj_rk(UppeHandle* h, int mode, const float2* lam_out, float2* lam_in, float a_f, float a_mu) {
    h->launches++;
    k_adj_rk<<<reduce_blocks_host(h->P), 256, 0, h->stream>>>(mode, lam_out, h->adj_lf, h->adj_acc, h->adj_lk,
                                                               h->adj_mu, lam_in, a_f, a_mu, h->P, h->S);
    return cudaGetLastError();
}

static int slice_threads(const UppeHandle* h) { return h->S / SLICE_ET; }

cudaError_t uppe_configure_slice_kernels(size_t smem_bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_real_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_spec_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fused_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_adj_cart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e == cudaSuccess) e = configure_fused_reg();
    if (e == cudaSuccess) e = configure_real_reg();
    if (e == cudaSuccess) e = configure_spec_reg();
    if (e == cudaSuccess) e = configure_adj_reg();
    return e;
}

static size_t slice_smem(const UppeHandle* h) { return (size_t)(h->S + h->N1) * sizeof(float2); }

cudaError_t launch_real_cart(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z) {
    if (h->slice_big) return launch_real_big(h, mode, src, A_out, nullptr, nullptr, 0.f, 0.f, z);
    if (h->slice_reg) return launch_real_reg(h, mode, src, A_out, nullptr, nullptr, 0.f, 0.f, z);
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    h->launches++;
    k_real_cart<<<h->N0, slice_threads(h), slice_smem(h), h->stream>>>(mode, src, uppe_op_view(h), h->E, A_out,
                                                                        nullptr, nullptr, 0.f, 0.f, logN1, logN2,
                                                                        h->tw, h->twLog, z);
    return cudaGetLastError();
}

cudaError_t launch_apply1_cart(UppeHandle* h, float Cs, float Ce, StepArgs z) {
    if (h->slice_big) return launch_real_big(h, REAL_APPLY1, h->qi, nullptr, h->k1, h->qf, Cs, Ce, z);
    if (h->slice_reg) return launch_real_reg(h, REAL_APPLY1, h->qi, nullptr, h->k1, h->qf, Cs, Ce, z);
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    h->launches++;
    k_real_cart<<<h->N0, slice_threads(h), slice_smem(h), h->stream>>>(REAL_APPLY1, h->qi, uppe_op_view(h), h->E,
                                                                        nullptr, h->k1, h->qf, Cs, Ce, logN1, logN2,
                                                                        h->tw, h->twLog, z);
    return cudaGetLastError();
}

cudaError_t launch_spec_cart(UppeHandle* h, int mode, const float2* src_real, float2* q_out, float2* qf_io,
                             const float2* qi, float Cs, float Ce, StepArgs z) {
    if (h->slice_big) return launch_spec_big(h, mode, src_real, q_out, qf_io, qi, Cs, Ce, z);
    if (h->slice_reg) return launch_spec_reg(h, mode, src_real, q_out, qf_io, qi, Cs, Ce, z);
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    h->launches++;
    k_spec_cart<<<h->N0, slice_threads(h), slice_smem(h), h->stream>>>(mode, src_real, uppe_op_view(h), q_out, qf_io,
                                                                        qi, Cs, Ce, logN1, logN2, h->tw, h->twLog, z);
    return cudaGetLastError();
}

cudaError_t launch_fused_cart(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                              bool zs_current) {
    if (h->slice_big) return launch_fused_big(h, mode, Cs, Ce, z_rhs, z_next, zs_current);
    if (h->slice_reg) {
        // The NL filter leaves the slices w >= nl_cut_off without current (J = 0, so S = 0): the fused
        // pass walks the others, and one block per such slice applies the stage with S = 0 and forms
        // E, so that no persistent block takes a fourth slice for them (513 slices on 152 blocks).
        const int jhi = h->cfg.nl_cut_off;
        if (!h->cfg.envelope && h->cfg.nl_cut_on <= 0 && jhi > 0 && jhi < h->N0) {
            cudaError_t e = launch_fused_reg(h, mode, Cs, Ce, z_rhs, z_next, jhi);
            if (e != cudaSuccess) return e;
            // With S = 0 there, those slices keep q = cond qi through the step (qf = qi after stage 1),
            // so stage 2 would rewrite stage 1's E and the finish stage 3's E, and the finish would
            // write q = qi back (cond = 1 above the conditioned bins): both are left out, except
            // when the stage estimates are being stored (stage_q)
            if (zs_current && jhi >= 4 && !h->stage_q) return cudaSuccess;
            if (mode == SPEC_STAGE1)
                return launch_real_reg_range(h, REAL_ZS1, h->qi, nullptr, nullptr, h->qf, 0.f, 0.f, z_next, jhi,
                                             h->N0 - jhi);
            if (mode == SPEC_STAGE23)
                return launch_real_reg_range(h, REAL_ZS23, h->qi, nullptr, nullptr, nullptr, 0.f, 0.f, z_next, jhi,
                                             h->N0 - jhi);
            return launch_real_reg_range(h, REAL_ZSF, h->qf, nullptr, nullptr, h->qi, 0.f, 0.f, z_next, jhi,
                                         h->N0 - jhi);
        }
        return launch_fused_reg(h, mode, Cs, Ce, z_rhs, z_next, h->N0);
    }
    int logN1 = ilog2_exact(h->N1), logN2 = ilog2_exact(h->N2);
    h->launches++;
    k_fused_cart<<<h->N0, slice_threads(h), slice_smem(h), h->stream>>>(mode, h->J, uppe_op_view(h), h->qi, h->qf,
                                                                         h->qi, h->E, Cs, Ce, logN1, logN2, h->tw,
                                                                         h->twLog, z_rhs, z_next, h->num_sms);
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
                               float2* __restrict__ qf, size_t n, int S, float Cs, float Ce, int ncond) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float2 a = qi[i], s = k1[i];
        float cond = (i < (size_t)ncond * S) ? 0.f : 1.f;
        qf[i] = cadd(a, cscale(s, Cs));
        q[i] = cscale(cadd(a, cscale(s, Ce)), cond);
    }
}

cudaError_t launch_apply_stage1(UppeHandle* h, float Cs, float Ce) {
    h->launches++;
    k_apply_stage1<<<reduce_blocks(h->P) * 2, 256, 0, h->stream>>>(h->qi, h->k1, h->q, h->qf, h->P, h->S, Cs, Ce,
                                                                   h->cfg.envelope ? 0 : 4);
    return cudaGetLastError();
}

// E = i kz A, applied point by point on a real-space array (uppe_kernel.py:252-253).
__global__ void k_ikz(const float2* __restrict__ A, OpView opv, float2* __restrict__ E, size_t n, int S) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const OpPoint o = op_at(opv, i, opv.kg[i / S]);
        E[i] = op_field(opv, o, A[i]);
    }
}

cudaError_t launch_ikz(UppeHandle* h, const float2* A, float2* E) {
    h->launches++;
    k_ikz<<<reduce_blocks(h->P) * 2, 256, 0, h->stream>>>(A, uppe_op_view(h), E, h->P, h->S);
    return cudaGetLastError();
}
