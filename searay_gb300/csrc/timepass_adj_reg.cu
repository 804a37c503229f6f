// Register-resident adjoint time pass (the vector-Jacobian product of k_time_reg) for M = Nt/2 =
// 256, 512 and 1024 without a rotator, on the column layout of timepass_reg.cuh.
//
// For a column with the stage field E(w) and the cotangent G(w) of its current J(w) (the
// transposes of SeaRay's update_current, modules/uppe_kernel.py:139-186, and of the real-FFT
// steps of fft.cl:257-329, as in k_time_adj):
//   e(t)  = irfft(E)                                   (the forward's field, recomputed)
//   gp(t) = irfft-transposed of G i w W filt            (W = 1 at k = 0 and M, 1/2 inside)
//   ge(t) = 3 (ng chi3 / nref) e^2 gp                   (transpose of P = chi e, chi = ng chi3/nref e^2)
//   gE(w) = (1/Nt) W2 rfft(ge)                          (W2 = 1 at k = 0 and M, 2 inside)
// and d(loss)/d(chi3/nref) += sum_t gp ng e^3 (one double atomic per block).
//
// Columns with a nonzero ionization rate need the density, the transposed density scan and a
// third transform; they stay with the shared-memory kernel k_time_adj.  This pass decides per
// column, from e, whether any sample reaches the rate threshold (the forward's warp vote), and
// skips whole groups of k_time_adj's width (CA = 2048 / M adjacent columns) that hold such a
// column: it appends the group to a list (count in list[0]) that k_time_adj then walks.  A skipped
// group is neither read beyond E nor written here, so every column's gE and its share of the chi3
// derivative come from exactly one of the two kernels.
//
// Per column: stage E (rows of NC columns, cp.async), pack and inverse-transform it in registers,
// park e (time order, column-contiguous) in a global scratch array, stage G, pack and inverse-
// transform it, form ge against the parked e, forward-transform ge and write gE.  Same block shape,
// shared-memory column buffers and register budget as k_time_reg.
#include <math.h>

#include "hankel_tc.cuh"
#include "time_common.cuh"
#include "timepass_reg.cuh"
#include "uppe_internal.h"

template <int LOGM>
__global__ void __launch_bounds__(256, TReg<LOGM>::MINB)
    k_time_adj_reg(const float2* __restrict__ E, const float2* __restrict__ Gc, float2* __restrict__ gE,
                   const float* __restrict__ ng, const float* __restrict__ wv, const float2* __restrict__ twt,
                   float2* __restrict__ park_all, int* __restrict__ list, TimeParams tp,
                   double* __restrict__ dred) {
    using G = TReg<LOGM>;
    constexpr int M = G::M, TC = G::TC, R1 = G::R1, NC = G::NC, LD = G::LD;
    constexpr int CA = 2048 / M, NG = NC / CA;  // k_time_adj's group width; groups per block
    static_assert(NG * CA == NC && NG >= 1 && (TC == 32 || CA >= 2), "groups hold whole warps");
    extern __shared__ float2 sm[];
    __shared__ int col_live[NC];
    __shared__ int grp_live[NG];
    __shared__ double red_sh[G::THREADS / 32];
    const int tid = threadIdx.x;
    const size_t S = (size_t)tp.S;
    const size_t col0 = (size_t)blockIdx.x * NC;

    // ---- stage the NC half spectra of E into the column buffers ----
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

    // ---- e(t): irfft of E, T layout (v = Nt (e(2m) + i e(2m+1))) ----
    float2 v[R1];
    tr_pack_inverse<LOGM>(v, buf, twI, twP, t, [&](int k) { return buf[k]; });
    const float inv = tp.inv_nt;
    const float ngc = ng[col];
    const float kerr = ngc * tp.redchi3;
    bool live = false;
    if (tp.rate_form != UPPE_RATE_NONE) {
        // any sample with Em = fconv |e| + cutoff >= em_min: Em grows with |e| (fconv > 0), so the
        // largest |e| of the lane decides (the same roundings as per sample)
        float mx = 0.f;
#pragma unroll
        for (int r = 0; r < R1; ++r) mx = fmaxf(mx, fmaxf(fabsf(v[r].x), fabsf(v[r].y)));
        const bool any = fmaf(tp.fconv, mx * inv, tp.cutoff) >= tp.em_min;
        live = __any_sync(0xffffffffu, any);  // both columns of a warp when TC = 16: one group
    }
    if (t == 0) col_live[cl] = live ? 1 : 0;
    __syncthreads();
    if (tid < NG) {
        int any = 0;
#pragma unroll
        for (int i = 0; i < CA; ++i) any |= col_live[tid * CA + i];
        grp_live[tid] = any;
        if (any) {
            const int slot = atomicAdd(list, 1);
            list[1 + slot] = (int)blockIdx.x * NG + tid;
        }
    }
    __syncthreads();
    const bool skip = grp_live[cl / CA] != 0;  // warp-uniform
    float2* park = park_all + col * (size_t)M;
    if (!skip) {
#pragma unroll
        for (int r = 0; r < R1; ++r) park[G::tm(t, r)] = v[r];
    }
    __syncthreads();  // every column's exchange reads of its buffer are done

    // ---- stage G of the columns this pass takes ----
    for (int i = tid; i < (M + 1) * NC; i += G::THREADS) {
        const int c = i & (NC - 1), k = i / NC;
        if (!grp_live[c / CA]) cp_async8(&sm[c * LD + k], &Gc[(size_t)k * S + col0 + c]);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();

    float dpart = 0.f;
    if (!skip) {
        // gp(t): the packed inverse of G i w W filt (the NL filter is 1 on [cut_on, cut_off))
        tr_pack_inverse<LOGM>(v, buf, twI, twP, t, [&](int k) {
            if (k < tp.cut_on || k >= tp.cut_off) return make_float2(0.f, 0.f);
            const float wt = (k == 0 || k == M) ? 1.f : 0.5f;
            return cscale(cmul_i(buf[k]), __ldg(&wv[k]) * wt);
        });
        // ge = 3 kerr e^2 gp against the parked e (this lane's own entries)
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const float2 z = park[G::tm(t, r)];
            const float2 gp = v[r];
            const float e0 = z.x * inv, e1 = z.y * inv;
            dpart = fmaf(gp.x * ngc * e0 * e0, e0, dpart);
            dpart = fmaf(gp.y * ngc * e1 * e1, e1, dpart);
            v[r] = make_float2(3.f * kerr * e0 * e0 * gp.x, 3.f * kerr * e1 * e1 * gp.y);
        }
        // gE = (1/Nt) W2 rfft(ge)
        tr_forward<LOGM>(v, buf, twF, t);
        __syncwarp();  // the exchange reads of buf are done before the output staging
        tr_unpack<LOGM>(v, twP, t, lane, [&](int k, float2 X) {
            buf[k] = cscale(X, (k == 0 || k == M) ? inv : 2.f * inv);
        });
    }

    // ---- the chi3 derivative of the block, then gE rows of the columns this pass took ----
    double ds = (double)dpart;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ds += __shfl_xor_sync(0xffffffffu, ds, o);
    if (lane == 0) red_sh[warp] = ds;
    __syncthreads();
    if (tid == 0) {
        double b = 0.0;
#pragma unroll
        for (int i = 0; i < G::THREADS / 32; ++i) b += red_sh[i];
        if (b != 0.0) atomicAdd(dred, b);
    }
    for (int i = tid; i < (M + 1) * NC; i += G::THREADS) {
        const int c = i & (NC - 1), k = i / NC;
        if (grp_live[c / CA]) continue;
        if (tp.atc)  // the operand tiles of the Minv^T transform that follows
            tc_store_split(tp.atc, tp.atc_nwt, tp.atc_nkt, 0, k, (int)(col0 + c), sm[c * LD + k]);
        else
            gE[(size_t)k * S + col0 + c] = sm[c * LD + k];
    }
}

// ---- host side ----

int time_adj_reg_group(int M) { return 2048 / M; }

size_t time_adj_reg_list_len(const UppeHandle* h) { return 1 + (size_t)h->S / (2048 / h->M); }

// The register pass takes a grid only when its blocks (NC columns each) fill the multiprocessors:
// on small transverse grids (256 radial points: 32 blocks at M = 1024) the shared-memory kernel's
// narrower blocks (2048 / M columns) spread the work wider and ran faster (forward+adjoint at
// 1025 x 256: 6.97e8 grid-pt steps/s with it, 6.42e8 with the register pass).
bool time_adj_reg_ready(const UppeHandle* h) {
    const int nc = h->M == 1024 ? TReg<10>::NC : h->M == 512 ? TReg<9>::NC : TReg<8>::NC;
    return h->time_reg && h->tw_reg && h->adj_live && (h->tscr || h->adj_park) && time_reg_supported(h) &&
           h->S / nc >= h->num_sms;
}

cudaError_t uppe_configure_time_adj_reg() {
    cudaError_t e =
        cudaFuncSetAttribute(k_time_adj_reg<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TReg<8>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_adj_reg<9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TReg<9>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_time_adj_reg<10>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)TReg<10>::SMEM);
    return e;
}

// The register pass over every column; the groups it leaves are listed in h->adj_live (count
// first, reset here).  The park is the forward's scratch when the handle has one ([S][2 (M + 1)]
// complex), else h->adj_park ([S][M]).
cudaError_t launch_time_adj_reg(UppeHandle* h, const float2* E, const float2* G, float2* gE, double* dred) {
    const TimeParams tp = uppe_time_params(h);
    float2* park = h->tscr ? h->tscr : h->adj_park;
    cudaError_t e = cudaMemsetAsync(h->adj_live, 0, sizeof(int), h->stream);
    if (e != cudaSuccess) return e;
    h->launches++;
    switch (h->M) {
        case 256:
            k_time_adj_reg<8><<<h->S / TReg<8>::NC, TReg<8>::THREADS, TReg<8>::SMEM, h->stream>>>(
                E, G, gE, h->ng, h->w, h->tw_reg, park, h->adj_live, tp, dred);
            break;
        case 512:
            k_time_adj_reg<9><<<h->S / TReg<9>::NC, TReg<9>::THREADS, TReg<9>::SMEM, h->stream>>>(
                E, G, gE, h->ng, h->w, h->tw_reg, park, h->adj_live, tp, dred);
            break;
        default:
            k_time_adj_reg<10><<<h->S / TReg<10>::NC, TReg<10>::THREADS, TReg<10>::SMEM, h->stream>>>(
                E, G, gE, h->ng, h->w, h->tw_reg, park, h->adj_live, tp, dred);
            break;
    }
    return cudaGetLastError();
}
