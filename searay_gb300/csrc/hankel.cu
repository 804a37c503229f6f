// Cylindrical transverse transform: the radial Hankel transform of SeaRay's HankelTransformTool
// (modules/grid_tools.py:252-325; kernels fft.cl:363-385 RootVolumeMultiply/Divide, :443-477
// RadialTransform/InverseRadialTransform) as a batched complex x real GEMM per azimuthal mode,
// with the root-volume weights folded into the matrices:
//     forward  J_k = sum_r Mfwd[k][r] J_r,  Mfwd[k][r] = H[k][r] Lambda_r / Lambda_k  (k < Nk, else 0)
//     inverse  E_r = sum_k Minv[r][k] E_k,  Minv[r][k] = H[k][r] Lambda_k / Lambda_r
// The spectral-side operations are fused into the GEMM: the A-operand loader applies the propagator
// phase and i kz, the epilogue forms the ODE right-hand side and the RK4 stage update.
// The azimuthal FFT (FFT_axis2/IFFT_axis2, fft.cl:401-441) of grids with N2 > 1 runs as a separate
// DFT pass around the GEMM.
#include "common.cuh"
#include "uppe_internal.h"

#define GBM 32
#define GBN 64
#define GBK 16

enum { A_PLAIN = 0, A_QPHASE_IKZ = 1, A_QPHASE = 2, A_SADJ = 3 };
enum { C_STORE = 0, C_FINISH1 = 1, C_SPEC = 2, C_QADJ = 3, C_FADJ = 4 };

struct GemmArgs {
    const float2* A;  // operand source ([w][r|k][m] layout, row length N1, N2 azimuthal nodes)
    const float* B;   // [N2][NI][NK]
    OpView op;
    float2* C0;       // store target / q_out / A_out
    float2* C1;       // E (finish) / qf
    const float2* qi;
    int N0, N1, N2, NI, NK;
    int spec_mode;
    float Cs, Ce;
    StepArgs z;
};

template <int AMODE, int CMODE>
__global__ void __launch_bounds__(256) k_hankel_gemm(GemmArgs g) {
    __shared__ float2 As[GBK][GBM + 1];
    __shared__ __align__(16) float Bs[GBK][GBN + 4];
    const int m = blockIdx.z;
    const int w0 = blockIdx.y * GBM;
    const int i0 = blockIdx.x * GBN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const PhaseArgs pa{g.z.zhi, g.z.zlo, g.z.plain};
    float2 acc[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[r][j] = make_float2(0.f, 0.f);
    const float* Bm = g.B + (size_t)m * g.NI * g.NK;
    for (int k0 = 0; k0 < g.NK; k0 += GBK) {
        for (int e = threadIdx.x; e < GBK * GBM; e += 256) {
            const int kk = e % GBK, ww = e / GBK;
            const int w = w0 + ww, k = k0 + kk;
            float2 v = make_float2(0.f, 0.f);
            if (w < g.N0 && k < g.NK) {
                const size_t idx = ((size_t)w * g.N1 + k) * g.N2 + m;
                v = g.A[idx];
                if (AMODE == A_SADJ) {
                    // conj(D2) v, D2 = (i/2) exp(-i(kz+kg)z) / Re kz
                    const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
                    const float2 f = cconj(propagator_factor(o, pa, -1.f));
                    v = cscale(cmul_mi(cmul(f, v)), 0.5f / o.kzr);
                } else if (AMODE != A_PLAIN) {
                    const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
                    v = cmul(propagator_factor(o, pa, 1.f), v);
                    if (AMODE == A_QPHASE_IKZ) v = op_field(g.op, o, v);
                }
            }
            As[kk][ww] = v;
        }
        for (int e = threadIdx.x; e < GBK * GBN; e += 256) {
            const int kk = e % GBK, ii = e / GBK;
            const int i = i0 + ii, k = k0 + kk;
            Bs[kk][ii] = (i < g.NI && k < g.NK) ? Bm[(size_t)i * g.NK + k] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GBK; ++kk) {
            const float2 a0 = As[kk][ty * 2], a1 = As[kk][ty * 2 + 1];
            const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
            const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[0][j].x = fmaf(a0.x, bb[j], acc[0][j].x);
                acc[0][j].y = fmaf(a0.y, bb[j], acc[0][j].y);
                acc[1][j].x = fmaf(a1.x, bb[j], acc[1][j].x);
                acc[1][j].y = fmaf(a1.y, bb[j], acc[1][j].y);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int w = w0 + ty * 2 + r;
        if (w >= g.N0) continue;
        const float cond = (w < g.op.ncond) ? 0.f : 1.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int i = i0 + tx * 4 + j;
            if (i >= g.NI) continue;
            const size_t idx = ((size_t)w * g.N1 + i) * g.N2 + m;
            const float2 v = acc[r][j];
            if (CMODE == C_STORE) {
                g.C0[idx] = v;
            } else if (CMODE == C_QADJ || CMODE == C_FADJ) {
                const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
                float2 r = cmul(cconj(propagator_factor(o, pa, 1.f)), v);
                if (CMODE == C_QADJ) r = cmul(cconj(op_ikz(o)), r);
                g.C0[idx] = r;
            } else if (CMODE == C_FINISH1) {
                const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
                if (g.C0) g.C0[idx] = v;
                g.C1[idx] = op_field(g.op, o, v);
            } else {
                const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
                float2 f = propagator_factor(o, pa, -1.f);
                float2 s = cscale(cmul_i(cmul(f, v)), 0.5f / o.kzr);
                switch (g.spec_mode) {
                    case SPEC_STORE_K:
                        g.C0[idx] = s;
                        break;
                    case SPEC_STAGE1: {
                        float2 a = g.qi[idx];
                        g.C1[idx] = cadd(a, cscale(s, g.Cs));
                        g.C0[idx] = cscale(cadd(a, cscale(s, g.Ce)), cond);
                    } break;
                    case SPEC_STAGE23: {
                        float2 a = g.qi[idx];
                        float2 b = g.C1[idx];
                        g.C1[idx] = cadd(b, cscale(s, g.Cs));
                        g.C0[idx] = cscale(cadd(a, cscale(s, g.Ce)), cond);
                    } break;
                    default: {
                        float2 b = g.C1[idx];
                        g.C0[idx] = cscale(cadd(b, cscale(s, g.Cs)), cond);
                    } break;
                }
            }
        }
    }
}

// Azimuthal DFT along the contiguous last axis (length N2): out[row][j] = scale * sum_m in[row][m] W^{jm},
// W = exp(-+2 pi i / N2) (numpy fft / ifft conventions, fft.cl:401-441).
__global__ void k_azimuth_dft(const float2* __restrict__ in, float2* __restrict__ out, size_t rows, int N2,
                              int logN2, bool inv, float scale, const float2* __restrict__ tw, int twLog) {
    const size_t n = rows * (size_t)N2;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i >> logN2;
        const int j = (int)(i & (N2 - 1));
        const float2* src = in + row * N2;
        float2 acc = make_float2(0.f, 0.f);
        for (int mm = 0; mm < N2; ++mm) {
            float2 w = __ldg(&tw[((j * mm) & (N2 - 1)) << (twLog - logN2)]);
            if (inv) w.y = -w.y;
            acc = cadd(acc, cmul(src[mm], w));
        }
        out[i] = cscale(acc, scale);
    }
}

static cudaError_t launch_azimuth(UppeHandle* h, const float2* in, float2* out, bool inv) {
    const int logN2 = ilog2_exact(h->N2);
    const size_t rows = (size_t)h->N0 * h->N1;
    const size_t n = rows * h->N2;
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    h->launches++;
    k_azimuth_dft<<<blocks, 256, 0, h->stream>>>(in, out, rows, h->N2, logN2, inv, inv ? 1.f / h->N2 : 1.f, h->tw,
                                                  h->twLog);
    return cudaGetLastError();
}

cudaError_t launch_hankel_tc(UppeHandle* h, int amode, int cmode, const float2* A, int which, float2* C0,
                             float2* C1, const float2* qi, int NI, int NK, int spec_mode, float Cs, float Ce,
                             StepArgs z);

// Mixed-precision form: tensor-core GEMM (hankel_tc.cu); plain FP32 form: the FP32 SIMT GEMM below.
template <int AMODE, int CMODE>
static cudaError_t run_gemm(UppeHandle* h, GemmArgs& g) {
    if (h->cfg.precision == UPPE_PREC_MIXED)
        return launch_hankel_tc(h, AMODE, CMODE, g.A, g.B == h->Minv ? 1 : 0, g.C0, g.C1, g.qi, g.NI, g.NK,
                                g.spec_mode, g.Cs, g.Ce, g.z);
    dim3 grid((g.NI + GBN - 1) / GBN, (g.N0 + GBM - 1) / GBM, g.N2);
    h->launches++;
    k_hankel_gemm<AMODE, CMODE><<<grid, 256, 0, h->stream>>>(g);
    return cudaGetLastError();
}

static GemmArgs base_args(UppeHandle* h, StepArgs z) {
    GemmArgs g{};
    g.op = uppe_op_view(h);
    g.N0 = h->N0;
    g.N1 = h->N1;
    g.N2 = h->N2;
    g.z = z;
    return g;
}

// Inverse transform: E = T^-1(i kz exp(..) q) or, for finish, A = T^-1(exp(..) q) and E = i kz A.
cudaError_t launch_real_cyl(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z) {
    GemmArgs g = base_args(h, z);
    g.A = src;
    g.B = h->Minv;
    g.NI = h->N1;
    g.NK = h->Nk;
    cudaError_t err;
    if (h->N2 == 1) {
        if (mode == REAL_E) {
            g.C0 = h->E;
            err = run_gemm<A_QPHASE_IKZ, C_STORE>(h, g);
        } else {
            g.C0 = A_out;
            g.C1 = h->E;
            err = run_gemm<A_QPHASE, C_FINISH1>(h, g);
        }
        return err;
    }
    g.C0 = h->scratch;
    if (mode == REAL_E) {
        err = run_gemm<A_QPHASE_IKZ, C_STORE>(h, g);
        if (err != cudaSuccess) return err;
        return launch_azimuth(h, h->scratch, h->E, true);
    }
    err = run_gemm<A_QPHASE, C_STORE>(h, g);
    if (err != cudaSuccess) return err;
    float2* A = A_out ? A_out : h->k1;  // k1 is free at finish time
    err = launch_azimuth(h, h->scratch, A, true);
    if (err != cudaSuccess) return err;
    return launch_ikz(h, A, h->E);
}

// Forward transform of J (or of the incoming field for SPEC_LOAD) and the spectral update: fused
// into the GEMM's epilogue in the SIMT form and on azimuthal grids (N2 > 1, the operand is the
// azimuthal DFT in scratch); a separate elementwise pass after the tensor-core GEMM otherwise.
// z_next (stages whose estimate the next evaluation transforms at z_next): the tensor-core form's
// spectral update also writes that inverse transform's operand tiles (k_spec_point).
cudaError_t launch_spec_cyl(UppeHandle* h, int mode, const float2* src_real, float2* q_out, float2* qf_io,
                            const float2* qi, float Cs, float Ce, StepArgs z, const StepArgs* z_next) {
    GemmArgs g = base_args(h, z);
    g.B = h->Mfwd;
    g.NI = h->N1;
    g.NK = h->N1;
    g.A = src_real;
    if (h->N2 > 1) {
        cudaError_t err = launch_azimuth(h, src_real, h->scratch, false);
        if (err != cudaSuccess) return err;
        g.A = h->scratch;
    }
    g.C0 = q_out;
    g.C1 = qf_io;
    g.qi = qi;
    g.Cs = Cs;
    g.Ce = Ce;
    g.spec_mode = mode;
    if (mode == SPEC_LOAD) return run_gemm<A_PLAIN, C_STORE>(h, g);
    if (h->cfg.precision == UPPE_PREC_MIXED && g.A == h->J) {
        // the tensor-core transform stores its product over J (its pre-pass has already read J into
        // the operand tiles), then a separate pass applies S and the RK stage
        g.C0 = h->J;
        cudaError_t err = run_gemm<A_PLAIN, C_STORE>(h, g);
        if (err != cudaSuccess) return err;
        return launch_spec_point(h, mode, h->J, q_out, qf_io, qi, Cs, Ce, z, h->N2 == 1 ? z_next : nullptr);
    }
    return run_gemm<A_PLAIN, C_SPEC>(h, g);
}

// Adjoint transverse transforms on cylindrical grids (one azimuthal node) with the transposed folded
// matrices: ADJ_S / ADJ_LOAD apply Mfwd^T, ADJ_E / ADJ_FIN apply Minv^T; the tensor-core GEMM in the
// mixed-precision form, the FP32 SIMT GEMM in the plain form.
template <int AMODE, int CMODE>
static cudaError_t run_gemm_adj(UppeHandle* h, GemmArgs& g) {
    if (h->cfg.precision == UPPE_PREC_MIXED)
        return launch_hankel_tc(h, AMODE, CMODE, g.A, g.B == h->MfwdT ? 2 : 3, g.C0, g.C1, g.qi, g.NI, g.NK,
                                g.spec_mode, g.Cs, g.Ce, g.z);
    dim3 grid((g.NI + GBN - 1) / GBN, (g.N0 + GBM - 1) / GBM, g.N2);
    h->launches++;
    k_hankel_gemm<AMODE, CMODE><<<grid, 256, 0, h->stream>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_adj_cyl(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
    GemmArgs g = base_args(h, z);
    g.A = in;
    g.C0 = out;
    g.NI = h->N1;
    g.NK = h->N1;
    switch (mode) {
        case ADJ_S:
            g.B = h->MfwdT;
            return run_gemm_adj<A_SADJ, C_STORE>(h, g);
        case ADJ_LOAD:
            g.B = h->MfwdT;
            return run_gemm_adj<A_PLAIN, C_STORE>(h, g);
        case ADJ_E:
            g.B = h->MinvT;
            return run_gemm_adj<A_PLAIN, C_QADJ>(h, g);
        default:
            g.B = h->MinvT;
            return run_gemm_adj<A_PLAIN, C_FADJ>(h, g);
    }
}
