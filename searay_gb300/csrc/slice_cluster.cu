// Fused evaluation tail for 256 x 256 Cartesian slices in one launch: a cluster of 8 CTAs holds one
// frequency slice (512 KB of complex64) in its distributed shared memory.
//
// The three-pass form (slice_big.cu: rows, columns with the RK stage, inverse rows) moves every point
// through HBM three times (about 80 bytes per point and evaluation against the 40-48 of the
// evaluation itself), only because a 256 x 256 slice does not fit one CTA's shared memory.  Here CTA r
// of the cluster:
//   1. loads rows [32 r, 32 r + 32) of J and transforms them along y in registers (16 lanes per row,
//      16 values per lane; slice_reg.cuh's line transforms), into its own shared memory T[row][ky];
//   2. after a cluster barrier gathers its 32 columns ky in [32 r, 32 r + 32) from the 8 CTAs' T
//      (ld.shared::cluster), transforms them along x, applies S = (i/2) e^{-i(kz+kg)z} J / Re kz, the
//      RK stage and the propagator of the next evaluation (uppe.cl:22-108, as k_cols_big's BC_FUSED
//      kind), and transforms back along x;
//   3. once every CTA has read its T (a split cluster barrier), writes the columns into T, and after
//      a cluster barrier gathers its rows back, transforms them along y and stores E.
// HBM traffic per point: J 8, K 8, qi and/or qf 8-16, qf or qi 8, E 8: 40-48 bytes.
//
// 512 threads and about 133 KB of shared memory per CTA: one CTA per multiprocessor, a cluster on 8
// multiprocessors.  Measured on 1025 x 256 x 256 it takes 1.86 ms per evaluation against 0.90 ms
// for the three passes (one CTA per multiprocessor leaves each phase's memory latency exposed), so
// it is selected only on request (SEARAY_UPPE_CLUSTER=1); it gives the three-pass results bit for bit.
// Every CTA of a cluster runs the same barrier sequence; there are no waits on flags.  The slices without current (w >= nl_cut_off, J = 0 from the NL filter) skip the load and
// the forward row transform and run the rest on zeros (S = 0 exactly).
#include <cooperative_groups.h>

#include "slice_reg.cuh"

namespace cg = cooperative_groups;

#define SC_CL 8                  // CTAs per cluster (one slice)
#define SC_N 256                 // slice side
#define SC_ROWS (SC_N / SC_CL)   // rows (and columns) per CTA
#define SC_THREADS 512
#define SC_PT 257                // pitch of T (float2): conflict-free row writes and column reads
#define SC_T (SC_ROWS * SC_PT)   // T: [32][257]
#define SC_EXR (16 * 544)        // row exchange: 16 warps x two 16-lane lines x 17 x 16
#define SC_EXC (32 * (17 * 16 + 1))  // column exchange: 32 columns x (17 R1 + 1)
#define SC_EX (SC_EXR > SC_EXC ? SC_EXR : SC_EXC)
#define SC_SMEM ((SC_T + SC_EX) * (int)sizeof(float2))

__device__ __forceinline__ void sc_cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void sc_cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

__global__ void __cluster_dims__(SC_CL, 1, 1) __launch_bounds__(SC_THREADS, 1)
    k_slice_cluster(BigColArgs a, OpView opv, const float2* __restrict__ tw, int twLog, int nfwd, float inv_s,
                    float2* __restrict__ E_out) {
    extern __shared__ float2 scm[];
    float2* T = scm;
    float2* EX = scm + SC_T;
    cg::cluster_group cluster = cg::this_cluster();
    const int r = (int)cluster.block_rank();
    const int iw = blockIdx.x / SC_CL;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const size_t base = (size_t)iw * SC_N * SC_N;
    const TwGlobal twg{tw, twLog};
    float2 v[16], w[16];

    // ---- 1. rows x = 32 r + xl: forward transform along y ----
    const int xl = tid >> 4, j = tid & 15;
    float2* exr = EX + warp * 544 + (lane >> 4) * 272;
    const LineSync<false> rsync{0, 0};
    if (iw < nfwd) {
        const float2* s = a.src + base + (size_t)(SC_ROWS * r + xl) * SC_N + j;
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = s[16 * m];
        reg_n2m<16, 8, false>(v, w, exr, j, twg, rsync);  // w[b] = X[x][j + 16 b]
    } else {
#pragma unroll
        for (int b = 0; b < 16; ++b) w[b] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int b = 0; b < 16; ++b) T[xl * SC_PT + j + 16 * b] = w[b];
    sc_cluster_arrive();
    sc_cluster_wait();

    // ---- 2. columns ky = 32 r + 16 tile + c: gather along x from the cluster ----
    const int c = tid & 15, i = (tid >> 4) & 15, tile = tid >> 8;
    const int kyl = 16 * tile + c, ky = SC_ROWS * r + kyl;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const int x = i + 16 * m;
        const float2* Tq = cluster.map_shared_rank(T, x / SC_ROWS);
        v[m] = Tq[(x % SC_ROWS) * SC_PT + ky];
    }
    sc_cluster_arrive();  // this CTA's reads of the cluster's T are done
    float2* exc = EX + kyl * (17 * 16 + 1);
    const LineSync<true> csync{1 + tile, 256};
    reg_n2m<16, 8, false>(v, w, exc, i, twg, csync);  // w[q] at kx = i + 16 q
    {
        const PhaseArgs p0{a.z0.zhi, a.z0.zlo, a.z0.plain};
        const PhaseArgs p1{a.z1.zhi, a.z1.zlo, a.z1.plain};
        const float cond = (iw < opv.ncond) ? 0.f : 1.f;
        const float2 kgw = opv.kg[iw];
        const int mode = a.mode;
        const bool need_a = mode != SPEC_FINISH;  // qi
        const bool need_b = mode != SPEC_STAGE1;  // qf
        // the operands of eight points are loaded before any store of those points (the pointers live
        // in structs: the compiler must assume a store may alias the next point's loads)
#pragma unroll
        for (int h8 = 0; h8 < 16; h8 += 8) {
            float2 K8[8], A8[8], B8[8];
            float ki8[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const size_t idx = base + (size_t)(i + 16 * (h8 + q)) * SC_N + ky;
                K8[q] = opv.K[idx];
                ki8[q] = opv.ki ? opv.ki[idx] : 0.f;
                A8[q] = need_a ? a.qi[idx] : make_float2(0.f, 0.f);
                B8[q] = need_b ? a.qf[idx] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int rr = h8 + q;
                const size_t idx = base + (size_t)(i + 16 * rr) * SC_N + ky;
                OpPoint o;
                o.Khi = K8[q].x;
                o.Klo = K8[q].y;
                o.kzr = (K8[q].x - kgw.x) + (K8[q].y - kgw.y);
                o.kzi = ki8[q];
                const float2 f = propagator_factor(o, p0, -1.f);
                const float2 sv = cscale(cmul_i(cmul(f, w[rr])), 0.5f / o.kzr);
                float2 qw;
                if (mode == SPEC_STAGE1) {
                    a.qf[idx] = cadd(A8[q], cscale(sv, a.Cs));
                    qw = cscale(cadd(A8[q], cscale(sv, a.Ce)), cond);
                } else if (mode == SPEC_STAGE23) {
                    a.qf[idx] = cadd(B8[q], cscale(sv, a.Cs));
                    qw = cscale(cadd(A8[q], cscale(sv, a.Ce)), cond);
                } else {
                    qw = cscale(cadd(B8[q], cscale(sv, a.Cs)), cond);
                    a.q_out[idx] = qw;
                }
                if (a.q_store && mode != SPEC_FINISH) a.q_store[idx] = qw;
                w[rr] = cmul(op_ikz(o), cmul(propagator_factor(o, p1, 1.f), qw));
            }
        }
    }
    reg_m2n<16, 8, true>(w, v, exc, i, twg, csync);  // v[m] at x = i + 16 m
    sc_cluster_wait();  // every CTA has read this CTA's T: overwrite it with the columns
#pragma unroll
    for (int m = 0; m < 16; ++m) T[kyl * SC_PT + i + 16 * m] = v[m];
    sc_cluster_arrive();
    sc_cluster_wait();

    // ---- 3. rows x = 32 r + xl again: gather along y, inverse transform, store E ----
    const int x = SC_ROWS * r + xl;
#pragma unroll
    for (int b = 0; b < 16; ++b) {
        const int kyb = j + 16 * b;
        const float2* Tq = cluster.map_shared_rank(T, kyb / SC_ROWS);
        w[b] = Tq[(kyb % SC_ROWS) * SC_PT + x];
    }
    sc_cluster_arrive();  // this CTA's reads of the cluster's T are done
    reg_m2n<16, 8, true>(w, v, exr, j, twg, rsync);
    float2* d = E_out + base + (size_t)x * SC_N + j;
#pragma unroll
    for (int m = 0; m < 16; ++m) d[16 * m] = cscale(v[m], inv_s);
    sc_cluster_wait();  // no CTA leaves while another may still read its shared memory
}

static int g_cluster_ok = -1;  // per process: -1 unknown, 0 no, 1 yes

bool cluster_slice_supported(int N1, int N2) { return N1 == SC_N && N2 == SC_N; }

// Configures the kernel once and checks that a cluster of 8 such CTAs can be resident.
static bool cluster_slice_ready() {
    if (g_cluster_ok >= 0) return g_cluster_ok == 1;
    g_cluster_ok = 0;
    if (cudaFuncSetAttribute(k_slice_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, SC_SMEM) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(SC_CL, 1, 1);
    cfg.blockDim = dim3(SC_THREADS, 1, 1);
    cfg.dynamicSmemBytes = SC_SMEM;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = SC_CL;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_slice_cluster, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    g_cluster_ok = nclusters > 0 ? 1 : 0;
    return g_cluster_ok == 1;
}

// The fused tail of launch_fused_big over the slices [0, nall), rows of the slices [0, nfwd) loaded
// (the others hold J = 0).  Returns cudaErrorNotSupported when the cluster form cannot run here.
cudaError_t launch_fused_cluster(UppeHandle* h, const BigColArgs& a, int nfwd, int nall) {
    if (!cluster_slice_supported(h->N1, h->N2) || !cluster_slice_ready()) return cudaErrorNotSupported;
    h->launches++;
    const OpView opv = uppe_op_view(h);
    k_slice_cluster<<<(unsigned)(nall * SC_CL), SC_THREADS, SC_SMEM, h->stream>>>(a, opv, h->tw, h->twLog, nfwd,
                                                                                   1.0f / (float)h->S, h->E);
    return cudaGetLastError();
}
