// Radial Hankel transform on the 5th-generation tensor cores (tcgen05), split-BF16x3.
//
// Same contraction as hankel.cu, C[w][i] = sum_k A(w,k) B[i][k] with complex A and real B (the
// folded Hankel matrices of modules/grid_tools.py:252-325), but as a real GEMM on the tensor core:
//   * a tile of 64 frequencies becomes 128 MMA rows, row 2j = Re A(w0+j, .), row 2j+1 = Im A(w0+j, .);
//   * every FP32 operand x is split into bf16 x_hi + x_lo and the product is accumulated as
//     A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32 (the dropped A_lo B_lo is ~2^-18 of the product);
//   * one elected thread issues tcgen05.mma (M=128, N=128, K=16) from shared-memory operands in the
//     no-swizzle K-major core-matrix layout; the accumulator lives in tensor memory (TMEM) and is
//     read back with tcgen05.ld for the fused epilogue (store, finish, or ODE RHS + RK stage);
//   * the A operand (the field with its propagator phase and i kz where the mode asks) is formed and
//     split once per transform by k_hankel_tc_prep into tiles in that same layout, so every K step
//     of an output tile is two contiguous 32 KB blocks (A and B), fetched by bulk copies into a ring
//     of three shared-memory stages.
// Every wait on an mbarrier is bounded; on expiry the kernel records an error flag and skips ahead.
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "hankel_tc.cuh"
#include "uppe_internal.h"

#define TC_WAIT_LIMIT (1 << 24)

// operand modes (TA_SADJ: the cotangent of S times conj(D2), the A operand of the adjoint ADJ_S)
enum { TA_PLAIN = 0, TA_QPHASE_IKZ = 1, TA_QPHASE = 2, TA_PRESPLIT = 3, TA_SADJ = 4 };
// epilogues (TC_QADJ / TC_FADJ: conj(D0) C and conj(exp(i(kz+kg)z)) C of the adjoint ADJ_E / ADJ_FIN)
enum { TC_STORE = 0, TC_FINISH1 = 1, TC_SPEC = 2, TC_QADJ = 3, TC_FADJ = 4 };

struct TcArgs {
    const float2* A;
    const uint8_t* Btc;  // split matrix tiles [N2][nit][nkt][hi 16 KB | lo 16 KB]
    const uint8_t* Atc;  // split field tiles [N2][nwt][nkt][hi 16 KB | lo 16 KB] (TA_PRESPLIT)
    int nit, nkt, nwt;
    OpView op;
    float2* C0;
    float2* C1;
    const float2* qi;
    int N0, N1, N2, NI, NK;
    int spec_mode;
    float Cs, Ce;
    StepArgs z;
    int* err;
};

// Shared-memory matrix descriptor of tcgen05 (start address, LBO, SBO in 16-byte units; version 1;
// no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M = 128, N = TN.
template <int TN>
__device__ __forceinline__ uint32_t instr_desc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TC_ROWS >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, int* err) {
    for (int i = 0; i < TC_WAIT_LIMIT; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    if (err) atomicExch(err, 1);
    return false;
}

// Output-tile shapes of the GEMM: TN = 128 columns per tile, 512 threads, three 64 KB stages, one
// block per multiprocessor (the shape in use); TN = 64, 256 threads, two 48 KB stages, two blocks
// per multiprocessor, gave the same results bit for bit but ran slower (18.7 against 15.7 us per
// inverse transform at 2049 x 512: every A tile is fetched by twice as many blocks).  A stage is
// [A_hi | A_lo | B_hi | B_lo]; a B tile of TN rows is the upper or lower half (contiguous 8 KB) of the
// 128-row split matrix tiles.
template <int TN>
struct TcShape {
    static constexpr int THREADS = TN == 128 ? 512 : 256;
    static constexpr int NSTAGE = TN == 128 ? 3 : 2;
    static constexpr int MINB = TN == 128 ? 1 : 2;
    static constexpr uint32_t BTILE = (uint32_t)TN * TC_K * 2;  // bytes of one B operand (hi or lo)
    static constexpr uint32_t STAGE = 2 * TC_TILE_BYTES + 2 * BTILE;
    static constexpr int LD = TN + 1;  // padded row of the epilogue staging tile (float2)
};

// One 16-byte-aligned block of global memory (a multiple of 16 bytes) into this CTA's shared memory
// by the bulk-copy engine; completion is counted in transaction bytes on the mbarrier.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

template <int TN>
__device__ __forceinline__ void tc_issue(uint32_t tmem_d, uint32_t st_a, uint32_t idesc, bool first, uint32_t mbar) {
    constexpr uint32_t BT = TcShape<TN>::BTILE;
    asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
    for (int ks = 0; ks < TC_K / 16; ++ks) {
        const uint32_t koff = (uint32_t)ks * 256u;  // two core matrices along K per K=16 step
        const uint64_t ahi = smem_desc(st_a + koff);
        const uint64_t alo = smem_desc(st_a + TC_TILE_BYTES + koff);
        const uint64_t bhi = smem_desc(st_a + 2 * TC_TILE_BYTES + koff);
        const uint64_t blo = smem_desc(st_a + 2 * TC_TILE_BYTES + BT + koff);
        const uint32_t acc0 = (!first || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(ahi), "l"(bhi), "r"(idesc), "r"(acc0));
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(ahi), "l"(blo), "r"(idesc), "r"(1u));
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(alo), "l"(bhi), "r"(idesc), "r"(1u));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

// The A operand tiles of one transform: element (w, k) of azimuthal mode m, with the propagator phase
// and i kz as AMODE asks, split into bf16 hi/lo at rows 2(w - w0)
// and 2(w - w0) + 1 of its tile, zero outside [N0) x [NK).  One thread per element of the padded
// [nwt * 64][nkt * 64] grid; consecutive threads take consecutive k.
template <int AMODE>
__global__ void __launch_bounds__(256) k_hankel_tc_prep(TcArgs g, uint8_t* __restrict__ Atc) {
    pdl_begin();
    const int m = blockIdx.y;
    const int KP = g.nkt * TC_K;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)g.nwt * TC_W * KP) return;
    const int k = (int)(e % KP), w = (int)(e / KP);
    const PhaseArgs pa{g.z.zhi, g.z.zlo, g.z.plain};
    float2 v = make_float2(0.f, 0.f);
    if (w < g.N0 && k < g.NK) {
        const size_t idx = ((size_t)w * g.N1 + k) * g.N2 + m;
        v = g.A[idx];
        if (AMODE == TA_SADJ) {
            // conj(D2) v, D2 = (i/2) exp(-i(kz+kg)z) / Re kz
            const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
            const float2 f = cconj(propagator_factor(o, pa, -1.f));
            v = cscale(cmul_mi(cmul(f, v)), 0.5f / o.kzr);
        } else if (AMODE != TA_PLAIN) {
            const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
            v = cmul(propagator_factor(o, pa, 1.f), v);
            if (AMODE == TA_QPHASE_IKZ) v = op_field(g.op, o, v);
        }
    }
    tc_store_split(Atc, g.nwt, g.nkt, m, w, k, v);
}

// The GEMM of one output tile (64 frequencies x TN columns) on pre-split operand tiles (AMODE =
// TA_PRESPLIT).  Thread 0 drives a ring of NSTAGE stages: it issues the A and B tiles of a K step
// as bulk copies that complete on the stage's `full` mbarrier, waits for them, issues the MMAs of the
// step (committed to the stage's `done` mbarrier), and refills the stage of the previous step once
// its MMAs have completed, so the copies run NSTAGE - 1 steps ahead of the tensor core.
template <int AMODE, int CMODE, int TN>
__global__ void __launch_bounds__(TcShape<TN>::THREADS, TcShape<TN>::MINB) k_hankel_tc(TcArgs g) {
    using SH = TcShape<TN>;
    constexpr int NST = SH::NSTAGE, TT = SH::THREADS, LD = SH::LD;
    pdl_begin();
    static_assert(AMODE == TA_PRESPLIT, "the GEMM reads pre-split operand tiles");
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // NST pipeline stages of [A_hi | A_lo | B_hi | B_lo] (1024-byte aligned), reused afterwards
    // as the epilogue staging tile
    const uint32_t raw_a = (uint32_t)__cvta_generic_to_shared(smem_raw);
    uint8_t* tiles = smem_raw + (((raw_a + 1023u) & ~1023u) - raw_a);
    float2* stage = reinterpret_cast<float2*>(tiles);
    __shared__ uint64_t full[NST], done[NST];
    __shared__ uint32_t tmem_slot;
    __shared__ int aborted;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m = blockIdx.z;
    const int w0 = blockIdx.y * TC_W;
    const int it = blockIdx.x;
    const int i0 = it * TN;
    const PhaseArgs pa{g.z.zhi, g.z.zlo, g.z.plain};
    const uint32_t tiles_a = smem_u32(tiles);
    const uint32_t full0 = smem_u32(&full[0]), done0 = smem_u32(&done[0]);  // stage s at + 8 s

    if (tid == 0) {
        aborted = 0;
        for (int s2 = 0; s2 < NST; ++s2) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full0 + 8u * s2));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(done0 + 8u * s2));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem_d = tmem_slot;
    const int nkt = g.nkt;
    const uint32_t idesc = instr_desc<TN>();
    // B: the 128-row split tile of this output tile, and the TN-row half of it (TN = 64)
    const int it128 = (it * TN) / 128;
    const uint32_t bhalf = (uint32_t)(((it * TN) & 127) / TN) * SH::BTILE;
    const uint8_t* Bbase = g.Btc + ((size_t)(m * g.nit + it128) * nkt) * (2 * TC_TILE_BYTES);
    const uint8_t* Abase = g.Atc + ((size_t)m * g.nwt + w0 / TC_W) * nkt * (size_t)(2 * TC_TILE_BYTES);

    if (tid == 0) {
        const auto load = [&](int kt, int s2) {
            const uint32_t st = tiles_a + (uint32_t)s2 * SH::STAGE, fb = full0 + 8u * s2;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(SH::STAGE)
                         : "memory");
            bulk_g2s(st, Abase + (size_t)kt * (2 * TC_TILE_BYTES), 2 * TC_TILE_BYTES, fb);
            const uint8_t* bk = Bbase + (size_t)kt * (2 * TC_TILE_BYTES);
            if constexpr (TN == 128) {
                bulk_g2s(st + 2 * TC_TILE_BYTES, bk, 2 * TC_TILE_BYTES, fb);
            } else {
                bulk_g2s(st + 2 * TC_TILE_BYTES, bk + bhalf, SH::BTILE, fb);
                bulk_g2s(st + 2 * TC_TILE_BYTES + SH::BTILE, bk + TC_TILE_BYTES + bhalf, SH::BTILE, fb);
            }
        };
        int issued = 0;  // K steps whose copies are issued
        int landed = 0;  // K steps whose copies have been waited for
        int mmas = 0;    // K steps whose MMAs are issued
        bool ok = true;
        for (; issued < nkt && issued < NST; ++issued) load(issued, issued);
        for (int kt = 0; kt < nkt && ok; ++kt) {
            const int s2 = kt % NST;
            ok = mbar_wait(full0 + 8u * s2, (uint32_t)((kt / NST) & 1), g.err);
            if (!ok) break;
            landed = kt + 1;
            tc_issue<TN>(tmem_d, tiles_a + (uint32_t)s2 * SH::STAGE, idesc, kt == 0, done0 + 8u * s2);
            mmas = kt + 1;
            if (kt >= 1 && issued < nkt) {
                const int sp = (kt - 1) % NST;  // == issued % NST
                ok = mbar_wait(done0 + 8u * sp, (uint32_t)(((kt - 1) / NST) & 1), g.err);
                if (!ok) break;
                load(issued, sp);
                ++issued;
            }
        }
        // all MMAs are complete once the last commit has arrived (commits track all earlier MMAs)
        if (ok) ok = mbar_wait(done0 + 8u * ((nkt - 1) % NST), (uint32_t)(((nkt - 1) / NST) & 1), g.err);
        if (!ok) {
            // drain: the copies still in flight into this CTA's shared memory, then the issued MMAs
            for (int t = landed; t < issued; ++t)
                mbar_wait(full0 + 8u * (t % NST), (uint32_t)((t / NST) & 1), nullptr);
            if (mmas > 0)
                mbar_wait(done0 + 8u * ((mmas - 1) % NST), (uint32_t)(((mmas - 1) / NST) & 1), nullptr);
            aborted = 1;
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    __syncthreads();

    // ---- epilogue: TMEM -> registers -> padded staging tile [64][129] complex ----
    // warp w reads accumulator lanes 32 (w % 4) .. + 31 (the lane quarter a warp may access); the
    // warps of one quarter take different 32-column chunks
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;  // accumulator lane = MMA row
    const int wl = row >> 1;
    const int part = row & 1;
#pragma unroll 1
    for (int c0 = (warp >> 2) * 32; c0 < TN; c0 += (TT / 128) * 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem_d + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        float* st = reinterpret_cast<float*>(stage + wl * LD + c0) + part;
#pragma unroll
        for (int j = 0; j < 32; ++j) st[2 * j] = __uint_as_float(r[j]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_d), "r"(TN));
    if (aborted) return;

    // ---- fused epilogue, coalesced along the output columns ----
    for (int e = tid; e < TC_W * TN; e += TT) {
        const int col = e & (TN - 1), wle = e / TN;
        const int w = w0 + wle, i = i0 + col;
        if (w >= g.N0 || i >= g.NI) continue;
        const float2 v = stage[wle * LD + col];
        const size_t idx = ((size_t)w * g.N1 + i) * g.N2 + m;
        if (CMODE == TC_STORE) {
            g.C0[idx] = v;
        } else if (CMODE == TC_QADJ || CMODE == TC_FADJ) {
            const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
            float2 r = cmul(cconj(propagator_factor(o, pa, 1.f)), v);
            if (CMODE == TC_QADJ) r = cmul(cconj(op_ikz(o)), r);
            g.C0[idx] = r;
        } else if (CMODE == TC_FINISH1) {
            const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
            if (g.C0) g.C0[idx] = v;
            g.C1[idx] = op_field(g.op, o, v);
        } else {
            const float cond = (w < g.op.ncond) ? 0.f : 1.f;
            const OpPoint o = op_at(g.op, idx, g.op.kg[w]);
            const float2 f = propagator_factor(o, pa, -1.f);
            const float2 s = cscale(cmul_i(cmul(f, v)), 0.5f / o.kzr);
            switch (g.spec_mode) {
                case SPEC_STORE_K:
                    g.C0[idx] = s;
                    break;
                case SPEC_STAGE1: {
                    const float2 a = g.qi[idx];
                    g.C1[idx] = cadd(a, cscale(s, g.Cs));
                    g.C0[idx] = cscale(cadd(a, cscale(s, g.Ce)), cond);
                } break;
                case SPEC_STAGE23: {
                    const float2 a = g.qi[idx];
                    const float2 b = g.C1[idx];
                    g.C1[idx] = cadd(b, cscale(s, g.Cs));
                    g.C0[idx] = cscale(cadd(a, cscale(s, g.Ce)), cond);
                } break;
                default: {
                    const float2 b = g.C1[idx];
                    g.C0[idx] = cscale(cadd(b, cscale(s, g.Cs)), cond);
                } break;
            }
        }
    }
}

template <int TN>
static size_t tc_smem_bytes() {
    const size_t ops = TcShape<TN>::NSTAGE * (size_t)TcShape<TN>::STAGE;
    const size_t stage = (size_t)TC_W * TcShape<TN>::LD * sizeof(float2);
    return (ops > stage ? ops : stage) + 1024;  // + alignment slack
}

template <int AMODE, int CMODE, int TN>
static cudaError_t run_tc_shape(UppeHandle* h, TcArgs& a) {
    static bool configured = false;
    const size_t smem = tc_smem_bytes<TN>();
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_hankel_tc<AMODE, CMODE, TN>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((a.NI + TN - 1) / TN, (a.N0 + TC_W - 1) / TC_W, a.N2);
    h->launches++;
    launch_pdl(k_hankel_tc<AMODE, CMODE, TN>, grid, dim3(TcShape<TN>::THREADS), smem, h->stream, a);
    return cudaGetLastError();
}

template <int AMODE, int CMODE>
static cudaError_t run_tc(UppeHandle* h, TcArgs& a) {
    return run_tc_shape<AMODE, CMODE, 128>(h, a);
}

// Entry used by hankel.cu in the mixed-precision form.  amode/cmode follow hankel.cu's A_*/C_* codes
// (its A_SADJ = 3 is TA_SADJ here); `which` selects the split matrix tiles: 0 Mfwd, 1 Minv,
// 2 Mfwd^T, 3 Minv^T (the last two for the adjoint transforms).
cudaError_t launch_hankel_tc(UppeHandle* h, int amode, int cmode, const float2* A, int which, float2* C0,
                             float2* C1, const float2* qi, int NI, int NK, int spec_mode, float Cs, float Ce,
                             StepArgs z) {
    TcArgs a{};
    a.A = A;
    const uint8_t* const tiles[4] = {h->Mfwd_tc, h->Minv_tc, h->MfwdT_tc, h->MinvT_tc};
    if (which < 0 || which > 3 || !tiles[which]) return cudaErrorInvalidValue;
    if (amode == 3) amode = TA_SADJ;
    a.Btc = tiles[which];
    a.nit = (NI + TC_N - 1) / TC_N;
    a.nkt = (NK + TC_K - 1) / TC_K;
    a.op = uppe_op_view(h);
    a.C0 = C0;
    a.C1 = C1;
    a.qi = qi;
    a.N0 = h->N0;
    a.N1 = h->N1;
    a.N2 = h->N2;
    a.NI = NI;
    a.NK = NK;
    a.spec_mode = spec_mode;
    a.Cs = Cs;
    a.Ce = Ce;
    a.z = z;
    a.err = h->dev_err;
    a.nwt = (h->N0 + TC_W - 1) / TC_W;
    a.Atc = h->Atc;
    // the A operand once per transform (k_hankel_tc_prep), then the GEMM on pre-split tiles.  The
    // inverse transform of a stage estimate finds its operand already written when the spectral
    // update that produced the estimate was asked for it (k_spec_point with a TcNext): same source,
    // same z, same material, no transform in between (atc_next is cleared by every other use of the
    // tiles and by every entry point other than uppe_rk4_step).
    if (!h->Atc || (size_t)h->N2 * a.nwt * a.nkt * 2 * TC_TILE_BYTES > h->Atc_bytes) return cudaErrorInvalidValue;
    // Likewise the forward transform of J, and the adjoint's Minv^T transform of the cotangent of E,
    // find their operand written by the time pass that formed it.
    const bool ready_inv = amode == TA_QPHASE_IKZ && which == 1 && h->atc_next && h->atc_next_src == A &&
                           h->atc_next_z.zhi == z.zhi && h->atc_next_z.zlo == z.zlo &&
                           h->atc_next_z.plain == z.plain && h->atc_next_mat == h->mat_version;
    const bool ready_fwd = amode == TA_PLAIN && h->atc_fwd && which == h->atc_fwd_which && A == h->atc_fwd_src;
    const bool ready = ready_inv || ready_fwd;
    h->atc_next = 0;
    h->atc_fwd = 0;
    if (!ready) {
        const size_t n = (size_t)a.nwt * TC_W * a.nkt * TC_K;
        dim3 grid((unsigned)((n + 255) / 256), h->N2);
        h->launches++;
        if (amode == TA_PLAIN)
            launch_pdl(k_hankel_tc_prep<TA_PLAIN>, grid, dim3(256), 0, h->stream, a, h->Atc);
        else if (amode == TA_QPHASE_IKZ)
            launch_pdl(k_hankel_tc_prep<TA_QPHASE_IKZ>, grid, dim3(256), 0, h->stream, a, h->Atc);
        else if (amode == TA_SADJ)
            launch_pdl(k_hankel_tc_prep<TA_SADJ>, grid, dim3(256), 0, h->stream, a, h->Atc);
        else
            launch_pdl(k_hankel_tc_prep<TA_QPHASE>, grid, dim3(256), 0, h->stream, a, h->Atc);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (cmode == TC_STORE) return run_tc<TA_PRESPLIT, TC_STORE>(h, a);
    if (cmode == TC_SPEC) return run_tc<TA_PRESPLIT, TC_SPEC>(h, a);
    if (cmode == TC_FINISH1) return run_tc<TA_PRESPLIT, TC_FINISH1>(h, a);
    if (cmode == TC_QADJ) return run_tc<TA_PRESPLIT, TC_QADJ>(h, a);
    if (cmode == TC_FADJ) return run_tc<TA_PRESPLIT, TC_FADJ>(h, a);
    return cudaErrorInvalidValue;
}

// The operand of the next inverse transform, for the spectral update that writes it (N2 = 1): the
// tile counts of the Minv transform and its z.
TcNext hankel_tc_next(const UppeHandle* h, StepArgs z_next) {
    TcNext nx;
    nx.Atc = h->Atc;
    nx.nwt = (h->N0 + TC_W - 1) / TC_W;
    nx.nkt = (h->Nk + TC_K - 1) / TC_K;
    nx.Nk = h->Nk;
    nx.z = z_next;
    return nx;
}

// Bytes of the pre-split A tiles for the transforms of a handle (reduction length up to N1).
size_t uppe_hankel_tc_atile_bytes(int N0, int N1, int N2) {
    const size_t nwt = (N0 + TC_W - 1) / TC_W, nkt = (N1 + TC_K - 1) / TC_K;
    return (size_t)N2 * nwt * nkt * 2 * TC_TILE_BYTES;
}

// Host: round to the nearest bf16 (ties to even) and back, for the split of the matrices.
static inline uint16_t host_bf16_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);  // inf / nan
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static inline float host_bf16_value(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Split an FP32 matrix B[N2][NI][NK] into bf16 hi/lo tiles in the core-matrix order of the kernel.
void uppe_split_matrix_tiles(const float* B, int N2, int NI, int NK, std::vector<uint8_t>& out) {
    const int nit = (NI + TC_N - 1) / TC_N, nkt = (NK + TC_K - 1) / TC_K;
    out.assign((size_t)N2 * nit * nkt * 2 * TC_TILE_BYTES, 0);
    for (int m = 0; m < N2; ++m)
        for (int it = 0; it < nit; ++it)
            for (int kt = 0; kt < nkt; ++kt) {
                uint8_t* tile = out.data() + ((size_t)(m * nit + it) * nkt + kt) * 2 * TC_TILE_BYTES;
                for (int r = 0; r < TC_N; ++r)
                    for (int kk = 0; kk < TC_K; ++kk) {
                        const int i = it * TC_N + r, k = kt * TC_K + kk;
                        const float b = (i < NI && k < NK) ? B[((size_t)m * NI + i) * NK + k] : 0.f;
                        const uint16_t hb = host_bf16_bits(b);
                        const uint16_t lb = host_bf16_bits(b - host_bf16_value(hb));
                        const uint32_t o = (uint32_t)((r >> 3) * 1024 + (kk >> 3) * 128 + (r & 7) * 16 + (kk & 7) * 2);
                        memcpy(tile + o, &hb, 2);
                        memcpy(tile + TC_TILE_BYTES + o, &lb, 2);
                    }
            }
}
