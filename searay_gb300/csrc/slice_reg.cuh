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
//   mixed -> natural (m2n):  the same steps in reverse order.
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
#include "fft_smem.cuh"
#include "rk_stage.cuh"
#include "uppe_internal.h"

#define UPPE_COS_PI8 0.92387953251128675613f
#define UPPE_SIN_PI8 0.38268343236508977173f

// v * W16^E, W16 = exp(-2 pi i / 16); conjugated twiddle for the inverse transform
template <int E, bool INV>
UPPE_DEV float2 mul_w16(float2 v) {
    float2 w;
    if constexpr (E == 4) {
        return INV ? cmul_i(v) : cmul_mi(v);
    } else {
        if constexpr (E == 1) w = make_float2(UPPE_COS_PI8, -UPPE_SIN_PI8);
        else if constexpr (E == 2) w = make_float2(UPPE_SQRT1_2, -UPPE_SQRT1_2);
        else if constexpr (E == 3) w = make_float2(UPPE_SIN_PI8, -UPPE_COS_PI8);
        else if constexpr (E == 6) w = make_float2(-UPPE_SQRT1_2, -UPPE_SQRT1_2);
        else w = make_float2(-UPPE_COS_PI8, UPPE_SIN_PI8);  // E == 9
        if (INV) w.y = -w.y;
        return cmul(v, w);
    }
}

// In-register 16-point DFT, natural order in and out: 4 x 4 with W16 twiddles between the halves.
template <bool INV>
UPPE_DEV void dft16(float2 (&v)[16]) {
    float2 t[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
        float2 u[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
        dft_small<4>(u, INV);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) t[n1][k1] = u[k1];
    }
    t[1][1] = mul_w16<1, INV>(t[1][1]);
    t[1][2] = mul_w16<2, INV>(t[1][2]);
    t[1][3] = mul_w16<3, INV>(t[1][3]);
    t[2][1] = mul_w16<2, INV>(t[2][1]);
    t[2][2] = mul_w16<4, INV>(t[2][2]);
    t[2][3] = mul_w16<6, INV>(t[2][3]);
    t[3][1] = mul_w16<3, INV>(t[3][1]);
    t[3][2] = mul_w16<6, INV>(t[3][2]);
    t[3][3] = mul_w16<9, INV>(t[3][3]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        float2 u[4] = {t[0][k1], t[1][k1], t[2][k1], t[3][k1]};
        dft_small<4>(u, INV);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = u[k2];
    }
}

template <bool INV>
UPPE_DEV float2 tw_at(const TwGlobal& tw, int k, int sh) {
    float2 t = tw.get(k << sh);
    if (INV) t.y = -t.y;
    return t;
}

// natural -> mixed along one axis of length 16 R; `ex` is this line's exchange region, j the
// thread's index within the line.  v[m] = x[j + R m]  ->  w[s R + b] = X[j + R s + 16 b].
template <int R, int LOGN, bool INV>
UPPE_DEV void reg_n2m(float2 (&v)[16], float2 (&w)[16], float2* ex, int j, const TwGlobal& tw) {
    dft16<INV>(v);
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) w[a] = v[a];
    } else {
        const int sh = tw.log - LOGN;
#pragma unroll
        for (int a = 1; a < 16; ++a) v[a] = cmul(v[a], tw_at<INV>(tw, j * a, sh));
#pragma unroll
        for (int a = 0; a < 16; ++a) ex[j * 17 + a] = v[a];
        __syncwarp();
#pragma unroll
        for (int s = 0; s < 16 / R; ++s) {
            float2 u[R];
#pragma unroll
            for (int jj = 0; jj < R; ++jj) u[jj] = ex[jj * 17 + j + R * s];
            dft_small<R>(u, INV);
#pragma unroll
            for (int b = 0; b < R; ++b) w[s * R + b] = u[b];
        }
    }
}

// mixed -> natural along one axis: w[s R + b] = X[j + R s + 16 b]  ->  v[m] = x[j + R m].
template <int R, int LOGN, bool INV>
UPPE_DEV void reg_m2n(float2 (&w)[16], float2 (&v)[16], float2* ex, int j, const TwGlobal& tw) {
    if constexpr (R == 1) {
#pragma unroll
        for (int a = 0; a < 16; ++a) v[a] = w[a];
    } else {
        const int sh = tw.log - LOGN;
        __syncwarp();  // the line's last reads of this region are done
#pragma unroll
        for (int s = 0; s < 16 / R; ++s) {
            float2 u[R];
#pragma unroll
            for (int b = 0; b < R; ++b) u[b] = w[s * R + b];
            dft_small<R>(u, INV);
            const int a = j + R * s;
            ex[a] = u[0];
#pragma unroll
            for (int jj = 1; jj < R; ++jj) ex[jj * 17 + a] = cmul(u[jj], tw_at<INV>(tw, jj * a, sh));
        }
        __syncwarp();
#pragma unroll
        for (int a = 0; a < 16; ++a) v[a] = ex[j * 17 + a];
    }
    dft16<INV>(v);
}

template <int LN1, int LN2>
struct RegSlice {
    static constexpr int N1 = 1 << LN1, N2 = 1 << LN2, S = N1 * N2, T = S / 16;
    static constexpr int R1 = N1 / 16, R2 = N2 / 16;
    static constexpr int P = N2 + 2;
    static constexpr int EXW = 544;
    static constexpr int NWARP = (T + 31) / 32;
    static constexpr int SMEM = (N1 * P > NWARP * EXW ? N1 * P : NWARP * EXW) * (int)sizeof(float2);
};

// Thread coordinates of both layouts.  Row layout: line x (row), lane jr; column layout: line ky
// (column), lane ic.  exr / exc: the thread's line region for the exchanges.
template <class RS>
struct RegCoords {
    int x, jr, ky, ic;
    float2 *exr, *exc;
    UPPE_DEV RegCoords(float2* sm, int tid) {
        x = tid / RS::R2;
        jr = tid % RS::R2;
        ky = tid / RS::R1;
        ic = tid % RS::R1;
        exr = sm + (tid >> 5) * RS::EXW + ((tid & 31) / RS::R2) * 17 * RS::R2;
        exc = sm + (tid >> 5) * RS::EXW + ((tid & 31) / RS::R1) * 17 * RS::R1;
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
    reg_n2m<RS::R2, LN2, INV>(v, w, c.exr, c.jr, tw);
    rows_to_cols<RS>(w, v, sm, c);
    reg_n2m<RS::R1, LN1, INV>(v, w, c.exc, c.ic, tw);
}

// Inverse 2D transform: w in the column layout, mixed order -> v in the row layout, natural order
// (v[m] at (x, jr + R2 m)).
template <class RS, int LN1, int LN2, bool INV>
UPPE_DEV void slice_inv_to_rows(float2 (&w)[16], float2 (&v)[16], float2* sm, const RegCoords<RS>& c,
                                const TwGlobal& tw) {
    reg_m2n<RS::R1, LN1, INV>(w, v, c.exc, c.ic, tw);
    cols_to_rows<RS>(v, w, sm, c);
    reg_m2n<RS::R2, LN2, INV>(w, v, c.exr, c.jr, tw);
}

// linear index (within the slice) of register r of the column layout
template <class RS>
UPPE_DEV int col_elem(const RegCoords<RS>& c, int r) {
    const int s = r / RS::R1, b = r % RS::R1;
    return (c.ic + RS::R1 * s + 16 * b) * RS::N2 + c.ky;
}

// ---------------------------------------------------------------------------------------------
// Fused evaluation tail (the same contract as the generic k_fused_cart): forward 2D FFT of J,
// S = (i/2) exp(-i(kz+kg) z) J / Re kz and the RK stage, then E for the next evaluation,
// E = IFFT2(i kz exp(i(kz+kg) z_next) qw)  (uppe.cl:22-52,73-108; uppe_kernel.py:210-213).
// ---------------------------------------------------------------------------------------------
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_fused_reg(int mode, const float2* __restrict__ J, OpView opv, float2* __restrict__ qi_out,
                float2* __restrict__ qf, const float2* __restrict__ qi, float2* __restrict__ E, float Cs, float Ce,
                const float2* __restrict__ tw, int twLog, StepArgs z_rhs, StepArgs z_next, int next_wave) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x;
    const size_t base = (size_t)iw * RS::S;
    if (tid == 0) {
        // operator and RK state of this slice are read after the forward FFT: fetch them into L2 now;
        // also the current of the slice a CTA of the next wave will take
        constexpr size_t fb = (size_t)RS::S * sizeof(float2);
        prefetch_l2(opv.K + base, fb);
        if (mode != SPEC_FINISH) prefetch_l2(qi + base, fb);
        if (mode != SPEC_STAGE1) prefetch_l2(qf + base, fb);
        if ((int)(iw + next_wave) < (int)gridDim.x) prefetch_l2(J + base + (size_t)next_wave * RS::S, fb);
    }
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid);
    float2 w[16], v[16];
    slice_fwd_from_global<RS, LN1, LN2, false>(J + base, w, sm, c, twg);

    const PhaseArgs pr{z_rhs.zhi, z_rhs.zlo, z_rhs.plain};
    const PhaseArgs pn{z_next.zhi, z_next.zlo, z_next.plain};
    const float cond = (iw < 4) ? 0.f : 1.f;
    const float2 kgw = opv.kg[iw];
    const bool last = (mode == SPEC_FINISH);
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const size_t idx = base + col_elem(c, r);
        const OpPoint o = op_at(opv, idx, kgw);
        const float2 qw = spec_update(mode, idx, w[r], o, cond, qi_out, qf, qi, Cs, Ce, pr, last);
        w[r] = cmul(op_ikz(o), cmul(propagator_factor(o, pn, 1.f), qw));
    }
    slice_inv_to_rows<RS, LN1, LN2, true>(w, v, sm, c, twg);
    float2* dst = E + base + (size_t)c.x * RS::N2 + c.jr;
    constexpr float scale = 1.0f / (float)RS::S;
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[RS::R2 * m] = cscale(v[m], scale);
}

// Inverse transverse transform (modes of k_real_cart): E = IFFT2(i kz e^{..} q), the finish form
// A = IFFT2(e^{..} q), E = i kz A, or the first RK stage from k1 followed by E.
template <int LN1, int LN2>
__global__ void __launch_bounds__(RegSlice<LN1, LN2>::T, 1)
    k_real_reg(int mode, const float2* __restrict__ src, OpView opv, float2* __restrict__ E,
               float2* __restrict__ A_out, const float2* __restrict__ k1, float2* __restrict__ qf, float Cs, float Ce,
               const float2* __restrict__ tw, int twLog, StepArgs z) {
    using RS = RegSlice<LN1, LN2>;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x, iw = blockIdx.x;
    const size_t base = (size_t)iw * RS::S;
    const TwGlobal twg{tw, twLog};
    const RegCoords<RS> c(sm, tid);
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
    const RegCoords<RS> c(sm, tid);
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
    const RegCoords<RS> c(sm, tid);
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

