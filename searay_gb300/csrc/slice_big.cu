// Cartesian passes for slices larger than one CTA's shared memory holds (more than 128 x 128 points,
// up to 256 x 256): the 2D transform is split into a row pass and a column pass through HBM.
//
//   row pass:    batched 1D FFT of every row (N2 points, the contiguous axis) of every slice,
//                forward (natural -> natural) or inverse (+ optional 1/S scale and the finish outputs);
//   column pass: one CTA per (slice, tile of 16 columns): the column FFT (N1 points) of each column
//                of the tile, the pointwise work of the pass (RK stage, propagator phase, i kz, the
//                adjoint factors), and/or the inverse column FFT.
//
// Both use the register-resident line transforms of slice_reg.cuh (16 values per thread, a 16-point
// DFT in registers, the line's R = N/16 threads exchange through shared memory).  In the column
// pass a warp holds 16 consecutive columns and two line lanes, so its global accesses are 128-byte
// row segments; a column's lines span several warps and meet at the CTA barrier.
//
// Sources and destinations may be the same buffer (each CTA owns its rows or columns whole).
// A fused evaluation tail is rows(J -> J), columns(J -> J, RK stage), rows^-1(J -> E): three
// launches in place in J (J is consumed by the evaluation).  The same contracts as the one-kernel
// slice passes (uppe_kernels.cu, slice_reg.cuh) hold for every mode.
#include <math.h>

#include "slice_reg.cuh"

template <int LN2, bool INV>
__global__ void __launch_bounds__(256)
    k_rows_big(const float2* src, float2* dst, float scale, int finish, float2* __restrict__ A_out, OpView opv,
               int N1, const float2* __restrict__ tw, int twLog, int ahead) {
    constexpr int N2 = 1 << LN2, R2 = N2 / 16, ROWS = 256 / R2;
    __shared__ float2 xb[8 * 544];
    const int tid = threadIdx.x;
    // the rows of the block `ahead` places on (about one wave later) into L2: one 128-byte line per
    // thread (ROWS N2 complex values = 32 KB)
    if (blockIdx.x + ahead < gridDim.x)
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(src + (size_t)(blockIdx.x + ahead) * ROWS * N2 + 16 * tid));
    const size_t row = (size_t)blockIdx.x * ROWS + tid / R2;
    const int j = tid % R2;
    float2* ex = xb + (tid >> 5) * 544 + ((tid & 31) / R2) * 17 * R2;
    const LineSync<false> sync{0, 0};
    const TwGlobal twg{tw, twLog};
    const float2* s = src + row * N2;
    float2* d = dst + row * N2;
    float2 v[16], w[16];
    if constexpr (!INV) {
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = s[j + R2 * m];
        reg_n2m<R2, LN2, false>(v, w, ex, j, twg, sync);
#pragma unroll
        for (int r = 0; r < 16; ++r) d[j + R2 * (r / R2) + 16 * (r % R2)] = cscale(w[r], scale);
    } else {
#pragma unroll
        for (int r = 0; r < 16; ++r) w[r] = s[j + R2 * (r / R2) + 16 * (r % R2)];
        reg_m2n<R2, LN2, true>(w, v, ex, j, twg, sync);
        if (!finish) {
#pragma unroll
            for (int m = 0; m < 16; ++m) d[j + R2 * m] = cscale(v[m], scale);
        } else {
            // finish: A = IFFT2(e^{..} q), E = i kz A at the same point (uppe_kernel.py:250-253)
            const float2 kgw = opv.kg[row / N1];
#pragma unroll
            for (int m = 0; m < 16; ++m) {
                const size_t idx = row * N2 + j + R2 * m;
                const float2 val = cscale(v[m], scale);
                if (A_out) A_out[idx] = val;
                d[j + R2 * m] = cmul(op_ikz(op_at(opv, idx, kgw)), val);
            }
        }
    }
}

// The pass kind is a template parameter (one body per kind keeps each kernel's code small).  The
// adjoint stage kind runs three blocks per multiprocessor (80 registers: more warps hide its operand
// loads better than the registers it gives up); the forward fused kind keeps 128 registers, two blocks.  In the
// kinds that update the RK or adjoint state (BC_FUSED, BC_ADJ_STAGE) the pointwise operands of eight
// points are loaded before any store of those points: the stores could alias the loads as far as
// the compiler knows, which otherwise serialises every point behind a full memory latency.
template <int LN1, int LN2, int KIND>
__global__ void __launch_bounds__(16 << (LN1 - 4), KIND == BC_ADJ_STAGE ? 3 : 2) k_cols_big(BigColArgs a, OpView opv, const float2* __restrict__ tw,
                                                              int twLog, int ahead) {
    constexpr int N1 = 1 << LN1, N2 = 1 << LN2, R1 = N1 / 16, T = 16 * R1, TILES = N2 / 16;
    constexpr int QC = 17 * R1 + 1;
    __shared__ float2 xb[16 * QC];
    const int tid = threadIdx.x;
    const int iw = blockIdx.x / TILES;
    const int c = tid & 15, i = tid >> 4;
    const int ky = (blockIdx.x % TILES) * 16 + c;
    const size_t base = (size_t)iw * N1 * N2;
    float2* ex = xb + c * QC;
    const LineSync<true> sync{0, T};
    const TwGlobal twg{tw, twLog};
    const PhaseArgs p0{a.z0.zhi, a.z0.zlo, a.z0.plain};
    const PhaseArgs p1{a.z1.zhi, a.z1.zlo, a.z1.plain};
    const float cond = (iw < 4) ? 0.f : 1.f;
    const float2 kgw = opv.kg[iw];
    const int mode = a.mode;
    float2 v[16], w[16];
    const auto idx_of = [&](int r) {
        const int kx = i + R1 * (r / R1) + 16 * (r % R1);
        return base + (size_t)kx * N2 + ky;
    };

    if constexpr (KIND == BC_FUSED || KIND == BC_SPEC || KIND == BC_ADJ_FWD || KIND == BC_ADJ_STAGE) {
        // the source columns of the block `ahead` places on (about one wave later) into L2: one
        // 128-byte line (16 columns) of one of its N1 = T rows per thread
        const unsigned fb = blockIdx.x + (unsigned)ahead;
        if (fb < gridDim.x) {
            const size_t fbase = (size_t)(fb / TILES) * N1 * N2 + (size_t)(fb % TILES) * 16;
            asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.src + fbase + (size_t)tid * N2));
        }
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = a.src[base + (size_t)(i + R1 * m) * N2 + ky];
        if constexpr (KIND == BC_FUSED || KIND == BC_ADJ_STAGE) {
            // the pointwise operands of this thread's 16 points are asked into L2 while the column
            // transform runs, so that their loads after it find them there
            const bool pa = (KIND == BC_ADJ_STAGE) || mode != SPEC_FINISH;
            const bool pb = (KIND == BC_ADJ_STAGE) || mode != SPEC_STAGE1;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const size_t idx = idx_of(r);
                asm volatile("prefetch.global.L2 [%0];\n" ::"l"(opv.K + idx));
                if (pa) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.qi + idx));
                if (pb) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.qf + idx));
            }
        }
        reg_n2m<R1, LN1, false>(v, w, ex, i, twg, sync);
    }
    if constexpr (KIND == BC_FUSED || KIND == BC_ADJ_STAGE) {
        // BC_FUSED: S and the RK stage (spec_update), E of the next evaluation;
        // BC_ADJ_STAGE: the cotangent of q, the reverse RK bookkeeping and conj(D2) (k_adj_fused_reg)
        const bool need_a = (KIND == BC_ADJ_STAGE) || mode != SPEC_FINISH;   // qi (fused) / lam_f
        const bool need_b = (KIND == BC_ADJ_STAGE) || mode != SPEC_STAGE1;   // qf (fused) / acc
#pragma unroll
        for (int h8 = 0; h8 < 16; h8 += 8) {
            float2 K8[8], A8[8], B8[8];
            float ki8[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const size_t idx = idx_of(h8 + j);
                K8[j] = opv.K[idx];
                ki8[j] = opv.ki ? opv.ki[idx] : 0.f;
                A8[j] = need_a ? a.qi[idx] : make_float2(0.f, 0.f);
                B8[j] = need_b ? a.qf[idx] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int r = h8 + j;
                const size_t idx = idx_of(r);
                OpPoint o;
                o.Khi = K8[j].x;
                o.Klo = K8[j].y;
                o.kzr = opv.envelope ? kgw.x : (K8[j].x - kgw.x) + (K8[j].y - kgw.y);
                o.kzi = ki8[j];
                if constexpr (KIND == BC_FUSED) {
                    const float2 f = propagator_factor(o, p0, -1.f);
                    const float2 sv = cscale(cmul_i(cmul(f, w[r])), 0.5f / o.kzr);
                    float2 qw;
                    if (mode == SPEC_STAGE1) {
                        a.qf[idx] = cadd(A8[j], cscale(sv, a.Cs));
                        qw = cscale(cadd(A8[j], cscale(sv, a.Ce)), cond);
                    } else if (mode == SPEC_STAGE23) {
                        a.qf[idx] = cadd(B8[j], cscale(sv, a.Cs));
                        qw = cscale(cadd(A8[j], cscale(sv, a.Ce)), cond);
                    } else {
                        qw = cscale(cadd(B8[j], cscale(sv, a.Cs)), cond);
                        a.q_out[idx] = qw;
                    }
                    if (a.q_store && mode != SPEC_FINISH) a.q_store[idx] = qw;
                    w[r] = cmul(op_ikz(o), cmul(propagator_factor(o, p1, 1.f), qw));
                } else {
                    const float2 mu = cmul(cconj(op_ikz(o)), cmul(cconj(propagator_factor(o, p0, 1.f)),
                                                                  cscale(w[r], 1.0f / (float)(N1 * N2))));
                    if (mode == 2) {
                        a.dst[idx] = cadd(B8[j], mu);
                    } else {
                        const float2 cm = cscale(mu, cond);
                        a.qf[idx] = cadd(B8[j], cm);
                        const float2 lk = cadd(cscale(A8[j], a.Cs), cscale(cm, a.Ce));
                        const float2 f = cconj(propagator_factor(o, p1, -1.f));
                        w[r] = cscale(cmul_mi(cmul(f, lk)), 0.5f / o.kzr);
                    }
                }
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const size_t idx = idx_of(r);
            if constexpr (KIND == BC_SPEC) {
                OpPoint o;
                if (mode != SPEC_LOAD) o = op_at(opv, idx, kgw);
                spec_update(mode, idx, w[r], o, cond, a.q_out, a.qf, a.qi, a.Cs, a.Ce, p0, true);
            } else if constexpr (KIND == BC_REAL) {
                const OpPoint o = op_at(opv, idx, kgw);
                float2 val;
                if (mode == REAL_APPLY1) {
                    const float2 q0 = a.qi[idx], s = a.k1[idx];
                    a.qf[idx] = cadd(q0, cscale(s, a.Cs));
                    val = cscale(cadd(q0, cscale(s, a.Ce)), cond);
                } else {
                    val = a.src[idx];
                }
                val = cmul(propagator_factor(o, p0, 1.f), val);
                if (mode != REAL_FINISH) val = cmul(op_ikz(o), val);
                w[r] = val;
            } else if constexpr (KIND == BC_ADJ_IN) {
                float2 val = a.src[idx];
                if (mode == ADJ_S) {
                    const OpPoint o = op_at(opv, idx, kgw);
                    const float2 f = cconj(propagator_factor(o, p0, -1.f));
                    val = cscale(cmul_mi(cmul(f, val)), 0.5f / o.kzr);
                }
                w[r] = val;
            } else {  // BC_ADJ_FWD
                const OpPoint o = op_at(opv, idx, kgw);
                float2 val = cmul(cconj(propagator_factor(o, p0, 1.f)), cscale(w[r], 1.0f / (float)(N1 * N2)));
                if (mode == ADJ_E) val = cmul(cconj(op_ikz(o)), val);
                a.dst[idx] = val;
            }
        }
    }
    const bool inverse = (KIND == BC_FUSED || KIND == BC_REAL || KIND == BC_ADJ_IN) ||
                         (KIND == BC_ADJ_STAGE && mode == 1);
    if (inverse) {
        reg_m2n<R1, LN1, true>(w, v, ex, i, twg, sync);
#pragma unroll
        for (int m = 0; m < 16; ++m) a.dst[base + (size_t)(i + R1 * m) * N2 + ky] = v[m];
    }
}

// ---------------------------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------------------------
bool big_slice_supported(int N1, int N2) {
    auto ok = [](int n) { return n == 128 || n == 256; };
    return ok(N1) && ok(N2) && N1 * N2 > 16384;
}

// Row transforms of the slices [0, nslices) (every slice when nslices < 0).
template <bool INV>
static cudaError_t rows(UppeHandle* h, const float2* src, float2* dst, float scale, int finish, float2* A_out,
                        int nslices = -1) {
    const size_t nrows = (size_t)(nslices < 0 ? h->N0 : nslices) * h->N1;
    h->launches++;
    const OpView opv = uppe_op_view(h);
    if (h->N2 == 256) {
        k_rows_big<8, INV><<<(unsigned)(nrows / 16), 256, 0, h->stream>>>(src, dst, scale, finish, A_out, opv, h->N1,
                                                                         h->tw, h->twLog, 2 * h->num_sms);
    } else {
        k_rows_big<7, INV><<<(unsigned)(nrows / 32), 256, 0, h->stream>>>(src, dst, scale, finish, A_out, opv, h->N1,
                                                                         h->tw, h->twLog, 2 * h->num_sms);
    }
    return cudaGetLastError();
}

template <int KIND>
static void cols_kind(UppeHandle* h, const BigColArgs& a, const OpView& opv, unsigned grid) {
    if (h->N1 == 256 && h->N2 == 256)
        k_cols_big<8, 8, KIND><<<grid, 256, 0, h->stream>>>(a, opv, h->tw, h->twLog, 2 * h->num_sms);
    else if (h->N1 == 256)
        k_cols_big<8, 7, KIND><<<grid, 256, 0, h->stream>>>(a, opv, h->tw, h->twLog, 2 * h->num_sms);
    else
        k_cols_big<7, 8, KIND><<<grid, 128, 0, h->stream>>>(a, opv, h->tw, h->twLog, 2 * h->num_sms);
}

// Column passes of the slices [0, nslices) (every slice when nslices < 0).
static cudaError_t cols(UppeHandle* h, const BigColArgs& a, int nslices = -1) {
    h->launches++;
    const OpView opv = uppe_op_view(h);
    const unsigned grid = (unsigned)((nslices < 0 ? h->N0 : nslices) * (h->N2 / 16));
    switch (a.kind) {
        case BC_FUSED: cols_kind<BC_FUSED>(h, a, opv, grid); break;
        case BC_SPEC: cols_kind<BC_SPEC>(h, a, opv, grid); break;
        case BC_REAL: cols_kind<BC_REAL>(h, a, opv, grid); break;
        case BC_ADJ_IN: cols_kind<BC_ADJ_IN>(h, a, opv, grid); break;
        case BC_ADJ_FWD: cols_kind<BC_ADJ_FWD>(h, a, opv, grid); break;
        case BC_ADJ_STAGE: cols_kind<BC_ADJ_STAGE>(h, a, opv, grid); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_fused_big(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                             bool zs_current) {
    // The time pass's NL filter leaves J = 0 on the slices w >= nl_cut_off: their forward row
    // transforms are left out (the column pass then reads those zeros, and S = 0 there exactly).
    // In stage 2 and the finish those slices already hold their q and E (launch_fused_cart): the
    // column and inverse row passes leave them out as well.
    const int jhi = h->cfg.nl_cut_off;
    const int nfwd = (!h->cfg.envelope && h->cfg.nl_cut_on <= 0 && jhi > 0 && jhi < h->N0) ? jhi : h->N0;
    const int nall = (zs_current && nfwd < h->N0 && jhi >= 4 && !h->stage_q) ? nfwd : h->N0;
    BigColArgs a{};
    a.kind = BC_FUSED;
    a.mode = mode;
    a.src = h->J;
    a.dst = h->J;
    a.q_out = h->qi;
    a.qf = h->qf;
    a.qi = h->qi;
    a.Cs = Cs;
    a.Ce = Ce;
    a.z0 = z_rhs;
    a.z1 = z_next;
    a.q_store = h->stage_q;
    // 256 x 256 slices with SEARAY_UPPE_CLUSTER=1: the three passes in one launch, the slice held by a
    // cluster of CTAs (slice_cluster.cu); the three-pass form otherwise or where that cannot run
    if (h->slice_cluster) {
        cudaError_t ec = launch_fused_cluster(h, a, nfwd, nall);
        if (ec != cudaErrorNotSupported) return ec;
        h->slice_cluster = 0;
    }
    cudaError_t e = rows<false>(h, h->J, h->J, 1.f, 0, nullptr, nfwd);
    if (e == cudaSuccess) e = cols(h, a, nall);
    if (e == cudaSuccess) e = rows<true>(h, h->J, h->E, 1.0f / (float)h->S, 0, nullptr, nall);
    return e;
}

// One stage boundary of the reverse RK4 sweep (the contract of k_adj_fused_reg): rows of the
// cotangent g of E into J, the column pass, and (mode 1) the inverse rows into J; mode 2 writes the
// cotangent of the step's input to out from the column pass.  J is free here (the adjoint time
// pass has consumed it).
cudaError_t launch_adj_fused_big(UppeHandle* h, int mode, const float2* g, float2* out, float a_f, float a_mu,
                                 StepArgs z_e, StepArgs z_s) {
    cudaError_t e = rows<false>(h, g, h->J, 1.f, 0, nullptr);
    BigColArgs a{};
    a.kind = BC_ADJ_STAGE;
    a.mode = mode;
    a.src = h->J;
    a.dst = (mode == 2) ? out : h->J;
    a.qf = h->adj_acc;
    a.qi = h->adj_lf;
    a.Cs = a_f;
    a.Ce = a_mu;
    a.z0 = z_e;
    a.z1 = z_s;
    if (e == cudaSuccess) e = cols(h, a);
    if (mode == 1 && e == cudaSuccess) e = rows<true>(h, h->J, out, 1.f, 0, nullptr);
    return e;
}

cudaError_t launch_real_big(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1, float2* qf,
                            float Cs, float Ce, StepArgs z) {
    BigColArgs a{};
    a.kind = BC_REAL;
    a.mode = mode;
    a.src = src;
    a.dst = h->E;
    a.qi = src;
    a.k1 = k1;
    a.qf = qf;
    a.Cs = Cs;
    a.Ce = Ce;
    a.z0 = z;
    cudaError_t e = cols(h, a);
    if (e == cudaSuccess) e = rows<true>(h, h->E, h->E, 1.0f / (float)h->S, mode == REAL_FINISH, A_out);
    return e;
}

cudaError_t launch_spec_big(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                            float Cs, float Ce, StepArgs z) {
    // the row transform goes to J when the source is J (consumed), else to E (then stale)
    float2* tmp = (src == h->J) ? h->J : h->E;
    if (tmp == h->E) h->E_valid = 0;
    cudaError_t e = rows<false>(h, src, tmp, 1.f, 0, nullptr);
    BigColArgs a{};
    a.kind = BC_SPEC;
    a.mode = mode;
    a.src = tmp;
    a.q_out = q_out;
    a.qf = qf;
    a.qi = qi;
    a.Cs = Cs;
    a.Ce = Ce;
    a.z0 = z;
    if (e == cudaSuccess) e = cols(h, a);
    return e;
}

cudaError_t launch_adj_big(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
    BigColArgs a{};
    a.mode = mode;
    a.z0 = z;
    if (mode == ADJ_S || mode == ADJ_LOAD) {
        a.kind = BC_ADJ_IN;
        a.src = in;
        a.dst = out;
        cudaError_t e = cols(h, a);
        if (e == cudaSuccess) e = rows<true>(h, out, out, 1.f, 0, nullptr);
        return e;
    }
    a.kind = BC_ADJ_FWD;
    cudaError_t e = rows<false>(h, in, out, 1.f, 0, nullptr);
    a.src = out;
    a.dst = out;
    if (e == cudaSuccess) e = cols(h, a);
    return e;
}
