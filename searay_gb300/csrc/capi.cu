// C ABI of libsearay_uppe (include/searay_uppe.h): handle management and the orchestration of one
// RK4 step, one right-hand-side evaluation and the diagnostic finish.  Mirrors the control flow of
// SeaRay's modules/uppe_kernel.py:188-331 with device-resident state and no per-step host sync
// unless the adaptive step estimate is required.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>
#include <utility>
#include <complex>
#include <vector>

#include "common.cuh"
#include "uppe_internal.h"

void uppe_split_matrix_tiles(const float* B, int N2, int NI, int NK, std::vector<uint8_t>& out);
size_t uppe_hankel_tc_atile_bytes(int N0, int N1, int N2);

static char g_create_error[512] = "";

int uppe_set_error(UppeHandle* h, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    char* dst = h ? h->err : g_create_error;
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return 0;
}

#define CUDA_TRY(h, expr)                                                                         \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            uppe_set_error((h), "%s failed: %s", #expr, cudaGetErrorString(e_));                  \
            return (e_ == cudaErrorMemoryAllocation) ? UPPE_E_NOMEM : UPPE_E_CUDA;                \
        }                                                                                         \
    } while (0)

// ---- optional per-class timing with CUDA events on the handle's stream ----
struct ProfState {
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    double ms[UPPE_NCLASS];
    long long count[UPPE_NCLASS];
    size_t next;
};

static cudaEvent_t prof_event(ProfState* ps) {
    if (ps->next == ps->pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ps->pool.push_back(e);
    }
    return ps->pool[ps->next++];
}

static cudaError_t prof_resolve(UppeHandle* h) {
    ProfState* ps = (ProfState*)h->prof;
    if (!ps) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return e;
    for (auto& p : ps->pending) {
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        if (e != cudaSuccess) return e;
        ps->ms[p.first] += ms;
        ps->count[p.first] += 1;
    }
    ps->pending.clear();
    ps->next = 0;
    return cudaSuccess;
}

struct ProfScope {
    UppeHandle* h;
    int cls;
    cudaEvent_t b, e;
    ProfScope(UppeHandle* h_, int c) : h(h_), cls(c), b(nullptr), e(nullptr) {
        ProfState* ps = (ProfState*)h->prof;
        if (!ps) return;
        if (ps->pending.size() > 4096) prof_resolve(h);
        b = prof_event(ps);
        e = prof_event(ps);
        if (b) cudaEventRecord(b, h->stream);
    }
    ~ProfScope() {
        ProfState* ps = (ProfState*)h->prof;
        if (!ps || !b || !e) return;
        cudaEventRecord(e, h->stream);
        ps->pending.push_back({cls, {b, e}});
    }
};

#define PROF_TRY(h, cls, expr)      \
    do {                            \
        ProfScope ps_((h), (cls));  \
        CUDA_TRY((h), (expr));      \
    } while (0)

static bool is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

static StepArgs split_z(const UppeHandle* h, double z) {
    StepArgs s;
    s.zhi = (float)z;
    s.zlo = (float)(z - (double)s.zhi);
    s.plain = (h->cfg.precision == UPPE_PREC_FP32);
    return s;
}

static void free_buffers(UppeHandle* h) {
    void* ptrs[] = {h->q,  h->qi,   h->qf,   h->k1,   h->E,     h->J,      h->scratch, h->opK,  h->opKi, h->kg2,
                    h->ng, h->tw,   h->w,    h->nlfilt, h->Minv, h->Mfwd, h->kr2_d, h->w2n2_d, h->kg_d, h->red, h->dev_err, h->Minv_tc, h->Mfwd_tc,
                    h->MfwdT_tc, h->MinvT_tc,
                    h->adj_q1, h->adj_q2, h->adj_q3, h->adj_lf, h->adj_acc, h->adj_lk, h->adj_mu, h->MfwdT, h->MinvT,
                    h->adj_E[0], h->adj_E[1], h->adj_E[2], h->adj_E[3],
                    h->dred_d, h->rot, h->Atc, h->tw_reg, h->tscr, h->adj_live, h->adj_park};
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

extern "C" int uppe_create(const UppeConfig* cfg, UppeHandle** out) {
    if (!cfg || !out) {
        uppe_set_error(nullptr, "uppe_create: null argument");
        return UPPE_E_ARG;
    }
    *out = nullptr;
    const UppeConfig& c = *cfg;
    const bool env = c.envelope != 0;
    if (env && (c.n0 < 16 || !is_pow2(c.n0))) {
        uppe_set_error(nullptr, "Paraxial propagator requires 2**n w-nodes with n >= 4 (got %d)", c.n0);
        return UPPE_E_ARG;
    }
    if (!env && (c.n0 < 17 || !is_pow2(c.n0 - 1))) {
        uppe_set_error(nullptr, "UPPE propagator requires 2**n+1 w-nodes with n >= 4 (got %d)", c.n0);
        return UPPE_E_ARG;
    }
    if (!is_pow2(c.n1) || !is_pow2(c.n2)) {
        uppe_set_error(nullptr, "UPPE propagator requires 2**n x-nodes and y-nodes (got %d, %d)", c.n1, c.n2);
        return UPPE_E_ARG;
    }
    const int Nt = env ? c.n0 : 2 * c.n0 - 2;  // time samples (complex envelope: one per frequency)
    if (Nt > 8192) {
        uppe_set_error(nullptr, "time axis of %d samples exceeds the 8192 supported by the time pass", Nt);
        return UPPE_E_ARG;
    }
    const long S = (long)c.n1 * c.n2;
    if (env && !c.cylindrical && (S < 16 || S > 16384)) {
        uppe_set_error(nullptr, "paraxial Cartesian slice %d x %d outside the supported 16 points .. 128 x 128", c.n1,
                       c.n2);
        return UPPE_E_ARG;
    }
    if (!c.cylindrical && (S < 16 || (S > 16384 && !big_slice_supported(c.n1, c.n2)))) {
        uppe_set_error(nullptr,
                       "Cartesian slice %d x %d outside the supported 16 points .. 128 x 128, 128 x 256, 256 x 128 "
                       "and 256 x 256", c.n1, c.n2);
        return UPPE_E_ARG;
    }
    if (c.cylindrical && (c.radial_modes < 1 || c.radial_modes > c.n1)) {
        uppe_set_error(nullptr, "radial modes %d must lie in [1, %d]", c.radial_modes, c.n1);
        return UPPE_E_ARG;
    }
    if (c.precision != UPPE_PREC_MIXED && c.precision != UPPE_PREC_FP32) {
        uppe_set_error(nullptr, "unknown precision form %d", c.precision);
        return UPPE_E_ARG;
    }
    if (c.rate_form < UPPE_RATE_NONE || c.rate_form > UPPE_RATE_SERIES) {
        uppe_set_error(nullptr, "unknown rate form %d", c.rate_form);
        return UPPE_E_ARG;
    }
    UppeHandle* h = new (std::nothrow) UppeHandle();
    if (!h) {
        uppe_set_error(nullptr, "out of host memory");
        return UPPE_E_NOMEM;
    }
    memset(h, 0, sizeof(UppeHandle));
    h->cfg = c;
    h->N0 = c.n0;
    h->N1 = c.n1;
    h->N2 = c.n2;
    h->Nk = c.cylindrical ? c.radial_modes : c.n1;
    h->Nt = Nt;
    h->M = env ? c.n0 : c.n0 - 1;
    h->S = (int)S;
    h->P = (size_t)c.n0 * S;
    // transverse points per time-pass block (the envelope pass holds two complex arrays per point);
    // at most 32, so that a warp holds whole segments of its columns (later_segments_sum)
    int tc = env ? 4096 / Nt : 8192 / Nt;
    if (tc < 1) tc = 1;
    if (tc > (env ? 32 : 16)) tc = env ? 32 : 16;
    if (tc > h->S) tc = h->S;
    h->time_cols = tc;
    h->redchi3 = c.chi3_over_nref;
    // time-pass thread layout: 16 samples per thread (512 threads per 8192 samples, 2 blocks per SM)
    // where the block stays within 1024 threads, else 32; SEARAY_UPPE_TIME_SPT=32 forces the latter
    h->time_spt = (Nt * tc / 16 <= 1024) ? 16 : 32;
    if (const char* v = getenv("SEARAY_UPPE_TIME_SPT")) {
        if (atoi(v) == 32) h->time_spt = 32;
    }
    // Cartesian slices of 16..128 points per axis use the register-resident transforms;
    // SEARAY_UPPE_SLICE=generic selects the shared-memory Stockham form for them as well
    h->slice_big = !env && !c.cylindrical && big_slice_supported(c.n1, c.n2);
    h->slice_reg = !env && !c.cylindrical && reg_slice_supported(c.n1, c.n2);
    if (const char* v = getenv("SEARAY_UPPE_SLICE")) {
        if (strcmp(v, "generic") == 0) h->slice_reg = 0;
    }
    h->time_reg = 1;
    if (const char* v = getenv("SEARAY_UPPE_TIME")) {
        if (strcmp(v, "smem") == 0) h->time_reg = 0;
    }
    // tensor-core Hankel transforms: the spectral update of a stage writes the next inverse transform's
    // operand tiles (SEARAY_UPPE_TC_NEXT=0: the transform's own pre-pass forms them)
    h->tc_next = 1;
    if (const char* v = getenv("SEARAY_UPPE_TC_NEXT")) {
        if (strcmp(v, "0") == 0) h->tc_next = 0;
    }
    // 256 x 256 slices: the three-pass tail; SEARAY_UPPE_CLUSTER=1 selects the cluster-fused tail
    // (slice_cluster.cu: one launch, 40-48 bytes per point, but measured twice as slow)
    h->slice_cluster = 0;
    if (const char* v = getenv("SEARAY_UPPE_CLUSTER")) {
        if (strcmp(v, "1") == 0) h->slice_cluster = h->slice_big && cluster_slice_supported(c.n1, c.n2);
    }
    int nt = Nt;
    if (c.n1 > nt) nt = c.n1;
    if (c.n2 > nt) nt = c.n2;
    h->twLog = ilog2_exact(nt);
    h->stream = 0;
    {
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
            h->num_sms = nsm;
        if (h->num_sms <= 0) h->num_sms = 152;
        // small envelope grids: fewer transverse points per time-pass block while that leaves fewer
        // blocks than multiprocessors, keeping at least one full warp per block
        while (env && h->time_cols > 1 && h->S / h->time_cols < h->num_sms &&
               h->Nt * (h->time_cols / 2) / 16 >= 32)
            h->time_cols /= 2;
        int smsm = 0;
        if (cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess)
            h->smem_per_sm = smsm;
        if (h->smem_per_sm <= 0) h->smem_per_sm = 228 * 1024;
    }

    const size_t fbytes = h->P * sizeof(float2);
    cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes)                                           \
    if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes));
    ALLOC(h->q, fbytes);
    ALLOC(h->qi, fbytes);
    ALLOC(h->qf, fbytes);
    ALLOC(h->k1, fbytes);
    ALLOC(h->E, fbytes);
    ALLOC(h->J, fbytes);
    if (c.cylindrical && c.n2 > 1) ALLOC(h->scratch, fbytes);
    ALLOC(h->opK, h->P * sizeof(float2));
    ALLOC(h->opKi, h->P * sizeof(float));
    ALLOC(h->kg2, (size_t)c.n0 * sizeof(float2));
    ALLOC(h->ng, (size_t)S * sizeof(float));
    ALLOC(h->tw, ((size_t)1 << h->twLog) * sizeof(float2));
    ALLOC(h->w, (size_t)c.n0 * sizeof(float));
    ALLOC(h->nlfilt, (size_t)c.n0 * sizeof(float));
    if (c.cylindrical) {
        ALLOC(h->Minv, (size_t)c.n2 * c.n1 * h->Nk * sizeof(float));
        ALLOC(h->Mfwd, (size_t)c.n2 * c.n1 * c.n1 * sizeof(float));
    }
    // the register-resident time pass (M = 256, 512, 1024): its twiddle tables, and its parking
    // scratch for ionizing columns when the medium ionizes
    const bool time_reg = !env && (h->M == 256 || h->M == 512 || h->M == 1024);
    if (time_reg) ALLOC(h->tw_reg, time_reg_table_len(h->M) * sizeof(float2));
    if (time_reg && c.rate_form != UPPE_RATE_NONE) ALLOC(h->tscr, time_reg_scratch_len(h) * sizeof(float2));
    ALLOC(h->kr2_d, (size_t)S * sizeof(double));
    ALLOC(h->w2n2_d, (size_t)2 * c.n0 * sizeof(double));
    ALLOC(h->kg_d, (size_t)c.n0 * sizeof(double));
    ALLOC(h->red, 4 * sizeof(float));
    ALLOC(h->dev_err, sizeof(int));
#undef ALLOC
    if (e != cudaSuccess) {
        uppe_set_error(nullptr, "device allocation failed: %s", cudaGetErrorString(e));
        free_buffers(h);
        delete h;
        return (e == cudaErrorMemoryAllocation) ? UPPE_E_NOMEM : UPPE_E_CUDA;  // no device, no driver, ...
    }
    // twiddle table tw[j] = exp(-2 pi i j / NT), computed in FP64
    const int NT = 1 << h->twLog;
    std::vector<float2> tw(NT);
    for (int j = 0; j < NT; ++j) {
        double a = -2.0 * M_PI * (double)j / (double)NT;
        tw[j] = make_float2((float)cos(a), (float)sin(a));
    }
    e = cudaMemcpy(h->tw, tw.data(), NT * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && h->tw_reg) {
        std::vector<float2> twr(time_reg_table_len(h->M));
        time_reg_tables(h->M, twr.data());
        e = cudaMemcpy(h->tw_reg, twr.data(), twr.size() * sizeof(float2), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(h->dev_err, 0, sizeof(int));
    // Allow the kernels that stage a whole slice / time tile in shared memory the full 227 KB; each
    // launch still requests only what its grid needs.
    if (e == cudaSuccess) e = uppe_configure_slice_kernels(227 * 1024);
    if (e == cudaSuccess) e = uppe_configure_time_kernel(227 * 1024);
    if (e == cudaSuccess && h->tw_reg) e = uppe_configure_time_reg();
    if (e == cudaSuccess && h->tw_reg) e = uppe_configure_time_adj_reg();
    if (e == cudaSuccess) e = uppe_configure_time_adj_kernel(224 * 1024);  // leaves room for its static shared memory
    if (e == cudaSuccess && env) e = uppe_configure_env_kernel(227 * 1024);
    if (e != cudaSuccess) {
        uppe_set_error(nullptr, "device set-up failed: %s", cudaGetErrorString(e));
        free_buffers(h);
        delete h;
        return UPPE_E_CUDA;
    }
    *out = h;
    return UPPE_OK;
}

extern "C" int uppe_destroy(UppeHandle* h) {
    if (!h) return UPPE_OK;
    if (h->prof) {
        ProfState* ps = (ProfState*)h->prof;
        for (cudaEvent_t e : ps->pool) cudaEventDestroy(e);
        delete ps;
        h->prof = nullptr;
    }
    free_buffers(h);
    delete h;
    return UPPE_OK;
}

extern "C" int uppe_set_stream(UppeHandle* h, void* stream) {
    if (!h) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    h->stream = (cudaStream_t)stream;
    return UPPE_OK;
}

extern "C" int uppe_set_grid(UppeHandle* h, const double* w, const double* kr2, const double* H, const double* Lambda) {
    if (!h || !w || !kr2) return h ? (uppe_set_error(h, "uppe_set_grid: null table"), UPPE_E_ARG) : UPPE_E_ARG;
    const UppeConfig& c = h->cfg;
    if (!c.envelope && w[0] != 0.0) {
        uppe_set_error(h, "UPPE propagator requires frequency range [0,...]");
        return UPPE_E_ARG;
    }
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    std::vector<float> wf(h->N0), filt(h->N0);
    for (int k = 0; k < h->N0; ++k) {
        wf[k] = (float)w[k];
        filt[k] = (k < c.nl_cut_on || k >= c.nl_cut_off) ? 0.f : 1.f;
    }
    CUDA_TRY(h, cudaMemcpy(h->w, wf.data(), h->N0 * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemcpy(h->nlfilt, filt.data(), h->N0 * sizeof(float), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemcpy(h->kr2_d, kr2, (size_t)h->S * sizeof(double), cudaMemcpyHostToDevice));
    if (c.cylindrical) {
        if (!H || !Lambda) {
            uppe_set_error(h, "cylindrical grid needs the Hankel basis and root-volume weights");
            return UPPE_E_ARG;
        }
        const int Nr = h->N1, Nk = h->Nk, Nm = h->N2;
        std::vector<float> Minv((size_t)Nm * Nr * Nk), Mfwd((size_t)Nm * Nr * Nr, 0.f);
        // H layout (Nk, Nr, Nm) (grid_tools.py:294)
        for (int m = 0; m < Nm; ++m)
            for (int k = 0; k < Nk; ++k)
                for (int r = 0; r < Nr; ++r) {
                    double hv = H[((size_t)k * Nr + r) * Nm + m];
                    Minv[((size_t)m * Nr + r) * Nk + k] = (float)(hv * Lambda[k] / Lambda[r]);
                    Mfwd[((size_t)m * Nr + k) * Nr + r] = (float)(hv * Lambda[r] / Lambda[k]);
                }
        CUDA_TRY(h, cudaMemcpy(h->Minv, Minv.data(), Minv.size() * sizeof(float), cudaMemcpyHostToDevice));
        CUDA_TRY(h, cudaMemcpy(h->Mfwd, Mfwd.data(), Mfwd.size() * sizeof(float), cudaMemcpyHostToDevice));
        // transposed matrices for the adjoint transforms (one azimuthal node)
        if (Nm == 1) {
            std::vector<float> MfT((size_t)Nr * Nr, 0.f), MiT((size_t)Nr * Nr, 0.f);
            for (int r = 0; r < Nr; ++r)
                for (int k = 0; k < Nr; ++k) {
                    MfT[(size_t)r * Nr + k] = Mfwd[(size_t)k * Nr + r];
                    if (k < Nk) MiT[(size_t)k * Nr + r] = Minv[(size_t)r * Nk + k];
                }
            if (!h->MfwdT) CUDA_TRY(h, cudaMalloc((void**)&h->MfwdT, MfT.size() * sizeof(float)));
            if (!h->MinvT) CUDA_TRY(h, cudaMalloc((void**)&h->MinvT, MiT.size() * sizeof(float)));
            CUDA_TRY(h, cudaMemcpy(h->MfwdT, MfT.data(), MfT.size() * sizeof(float), cudaMemcpyHostToDevice));
            CUDA_TRY(h, cudaMemcpy(h->MinvT, MiT.data(), MiT.size() * sizeof(float), cudaMemcpyHostToDevice));
            if (c.precision == UPPE_PREC_MIXED) {  // the adjoint transforms on the tensor cores
                std::vector<uint8_t> t;
                uppe_split_matrix_tiles(MfT.data(), 1, Nr, Nr, t);
                if (!h->MfwdT_tc) CUDA_TRY(h, cudaMalloc((void**)&h->MfwdT_tc, t.size()));
                CUDA_TRY(h, cudaMemcpy(h->MfwdT_tc, t.data(), t.size(), cudaMemcpyHostToDevice));
                uppe_split_matrix_tiles(MiT.data(), 1, Nr, Nr, t);
                if (!h->MinvT_tc) CUDA_TRY(h, cudaMalloc((void**)&h->MinvT_tc, t.size()));
                CUDA_TRY(h, cudaMemcpy(h->MinvT_tc, t.data(), t.size(), cudaMemcpyHostToDevice));
            }
        }
        if (c.precision == UPPE_PREC_MIXED) {
            std::vector<uint8_t> t;
            uppe_split_matrix_tiles(Minv.data(), Nm, Nr, Nk, t);
            if (!h->Minv_tc) CUDA_TRY(h, cudaMalloc((void**)&h->Minv_tc, t.size()));
            CUDA_TRY(h, cudaMemcpy(h->Minv_tc, t.data(), t.size(), cudaMemcpyHostToDevice));
            uppe_split_matrix_tiles(Mfwd.data(), Nm, Nr, Nr, t);
            if (!h->Mfwd_tc) CUDA_TRY(h, cudaMalloc((void**)&h->Mfwd_tc, t.size()));
            CUDA_TRY(h, cudaMemcpy(h->Mfwd_tc, t.data(), t.size(), cudaMemcpyHostToDevice));
            if (!h->Atc) {
                h->Atc_bytes = uppe_hankel_tc_atile_bytes(h->N0, Nr, Nm);
                CUDA_TRY(h, cudaMalloc((void**)&h->Atc, h->Atc_bytes));
                // the padding of the tiles (w >= N0, k >= N1) stays zero: the kernels that write the
                // tiles directly (time pass, spectral update) write only inside the grid
                CUDA_TRY(h, cudaMemset(h->Atc, 0, h->Atc_bytes));
            }
        }
    }
    h->have_grid = 1;
    return UPPE_OK;
}

extern "C" int uppe_set_material(UppeHandle* h, const double* w2n2, const double* kg, const double* ng) {
    if (!h) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (!h->have_grid) {
        uppe_set_error(h, "uppe_set_material before uppe_set_grid");
        return UPPE_E_ARG;
    }
    if (!w2n2 || !kg || !ng) {
        uppe_set_error(h, "uppe_set_material: null table");
        return UPPE_E_ARG;
    }
    std::vector<float2> kg2(h->N0);
    int cplx = 0;
    for (int k = 0; k < h->N0; ++k) {
        const float hi = (float)kg[k];
        // envelope solver: kg holds k0(w), the divisor of the right-hand side
        kg2[k] = h->cfg.envelope ? make_float2(hi, 0.f) : make_float2(hi, (float)(kg[k] - (double)hi));
        if (w2n2[2 * k + 1] != 0.0) cplx = 1;
        if (h->cfg.envelope && kg[k] == 0.0) {
            uppe_set_error(h, "paraxial k0(w) = w0 dn + w ng vanishes at frequency node %d", k);
            return UPPE_E_ARG;
        }
    }
    std::vector<float> ngf(h->S);
    for (int s = 0; s < h->S; ++s) ngf[s] = (float)ng[s];
    CUDA_TRY(h, cudaMemcpyAsync(h->w2n2_d, w2n2, 2 * h->N0 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->kg_d, kg, h->N0 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ng, ngf.data(), h->S * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->kg2, kg2.data(), h->N0 * sizeof(float2), cudaMemcpyHostToDevice, h->stream));
    h->complex_medium = cplx;
    h->mat_version += 1;
    h->E_valid = 0;
    PROF_TRY(h, UPPE_CLASS_OPERATOR, launch_build_operator(h));
    // exact max |Re kz + kg| and max Im kz of the new operator, for the range checks
    const float init[4] = {0.f, 0.f, 0.f, 0.f};
    CUDA_TRY(h, cudaMemcpyAsync(h->red, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    PROF_TRY(h, UPPE_CLASS_OPERATOR, launch_operator_bounds(h));
    float red[4];
    CUDA_TRY(h, cudaMemcpyAsync(red, h->red, sizeof(red), cudaMemcpyDeviceToHost, h->stream));
    // the pageable host tables above must be consumed before returning
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->max_abs_K = red[0];
    h->max_Ki = red[1];
    h->have_material = 1;
    return UPPE_OK;
}

static int check_ready(UppeHandle* h, bool need_field) {
    if (!h->have_grid || !h->have_material) {
        uppe_set_error(h, "grid and material must be set before propagating");
        return UPPE_E_ARG;
    }
    if (need_field && !h->have_field) {
        uppe_set_error(h, "no field loaded");
        return UPPE_E_ARG;
    }
    return UPPE_OK;
}

static cudaError_t real_pass(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z) {
    return h->cfg.cylindrical ? launch_real_cyl(h, mode, src, A_out, z) : launch_real_cart(h, mode, src, A_out, z);
}

static cudaError_t spec_pass(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                             float Cs, float Ce, StepArgs z, const StepArgs* z_next = nullptr) {
    return h->cfg.cylindrical ? launch_spec_cyl(h, mode, src, q_out, qf, qi, Cs, Ce, z, z_next)
                              : launch_spec_cart(h, mode, src, q_out, qf, qi, Cs, Ce, z);
}

// One source evaluation: J = sources(T^-1(...q...)) on the real side.
static cudaError_t eval_to_J(UppeHandle* h, const float2* qsrc, StepArgs z) {
    cudaError_t e;
    {
        ProfScope ps(h, UPPE_CLASS_TRANSVERSE_INV);
        e = real_pass(h, REAL_E, qsrc, nullptr, z);
    }
    if (e != cudaSuccess) return e;
    ProfScope ps(h, UPPE_CLASS_TIME);
    // cylindrical mixed form, one azimuthal node: J goes straight into the operand tiles of the
    // forward tensor-core transform that follows (its pre-pass is then skipped)
    const bool to_tc = h->cfg.cylindrical && h->cfg.precision == UPPE_PREC_MIXED && h->N2 == 1 && h->tc_next &&
                       h->Atc && !h->cfg.envelope;
    h->time_atc = to_tc ? 1 : 0;
    e = launch_time_pass(h, TIME_J, h->E, h->J, nullptr);
    h->time_atc = 0;
    h->atc_fwd = (to_tc && e == cudaSuccess) ? 1 : 0;
    h->atc_fwd_which = 0;
    h->atc_fwd_src = h->J;
    return e;
}

extern "C" int uppe_load_field(UppeHandle* h, const void* a) {
    if (!h || !a) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (!h->have_grid) {
        uppe_set_error(h, "uppe_load_field before uppe_set_grid");
        return UPPE_E_ARG;
    }
    StepArgs z = split_z(h, 0.0);
    PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, spec_pass(h, SPEC_LOAD, (const float2*)a, h->qi, nullptr, nullptr, 0.f, 0.f, z));
    h->have_field = 1;
    return UPPE_OK;
}

// Range limits of the representation, checked on the host before work is issued:
//  - the float-float phase reduction is exact while |K z| < 2^24 rad (about 1.6e7 rad);
//  - the interaction-picture amplitude grows as exp(Im kz z), which must stay inside FP32 range.
static int check_range(UppeHandle* h, double z) {
    const double az = fabs(z);
    if (h->cfg.precision == UPPE_PREC_MIXED && h->max_abs_K * az >= 1.6e7) {
        uppe_set_error(h, "propagator phase |(kz+kg) z| = %.3g rad exceeds the 1.6e7 rad of the float-float phase",
                       h->max_abs_K * az);
        return UPPE_E_RANGE;
    }
    if (h->max_Ki * az > 80.0) {
        uppe_set_error(h, "Im(kz) z = %.3g: the interaction-picture amplitude exp(Im(kz) z) leaves FP32 range",
                       h->max_Ki * az);
        return UPPE_E_RANGE;
    }
    return UPPE_OK;
}

static bool same_z(double a, double b) { return fabs(a - b) <= 1e-12 * fmax(1.0, fabs(b)); }

// Adaptive estimate of dz from k1 (held in h->k1) and qi: one host read per step.
static int estimate_dz(UppeHandle* h, double L, double z_sub, double dzmin, double* dz) {
    const float init[4] = {0.f, INFINITY, 0.f, 0.f};
    CUDA_TRY(h, cudaMemcpyAsync(h->red, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    PROF_TRY(h, UPPE_CLASS_STEP_SIZE, launch_absmax(h, h->qi));
    PROF_TRY(h, UPPE_CLASS_STEP_SIZE, launch_step_size(h, h->qi, h->k1, L, 0.4, 1e-2));
    float red[4];
    CUDA_TRY(h, cudaMemcpyAsync(red, h->red, sizeof(red), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    double d = (double)red[1];
    if (d < dzmin) d = dzmin;
    if (z_sub + d > L) d = L - z_sub;
    *dz = d;
    return UPPE_OK;
}

// Cartesian grids: every evaluation is the time pass plus one fused slice pass that finishes the
// RK stage and already produces E for the next evaluation; the last stage leaves E for the first
// evaluation of the next step, so a step is 8 kernels.
static int rk4_step_cartesian(UppeHandle* h, double z_phase, double L, double z_sub, double dzmin, bool adaptive,
                              double* dz_out) {
    if (!(h->E_valid && h->E_mat == h->mat_version && same_z(h->E_z, z_phase))) {
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_INV, launch_real_cart(h, REAL_E, h->qi, nullptr, split_z(h, z_phase)));
    }
    h->E_valid = 0;
    PROF_TRY(h, UPPE_CLASS_TIME, launch_time_pass(h, TIME_J, h->E, h->J, nullptr));
    double dz;
    if (adaptive) {
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
                 launch_spec_cart(h, SPEC_STORE_K, h->J, h->k1, nullptr, nullptr, 0.f, 0.f, split_z(h, z_phase)));
        int rc = estimate_dz(h, L, z_sub, dzmin, &dz);
        if (rc) return rc;
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_INV,
                 launch_apply1_cart(h, (float)(dz / 6), (float)(dz / 2), split_z(h, z_phase + 0.5 * dz)));
    } else {
        dz = L - z_sub;
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
                 launch_fused_cart(h, SPEC_STAGE1, (float)(dz / 6), (float)(dz / 2), split_z(h, z_phase),
                                   split_z(h, z_phase + 0.5 * dz)));
    }
    const StepArgs zh = split_z(h, z_phase + 0.5 * dz), ze = split_z(h, z_phase + dz);
    PROF_TRY(h, UPPE_CLASS_TIME, launch_time_pass(h, TIME_J, h->E, h->J, nullptr));
    PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
             launch_fused_cart(h, SPEC_STAGE23, (float)(dz / 3), (float)(dz / 2), zh, zh, /*zs_current=*/true));
    PROF_TRY(h, UPPE_CLASS_TIME, launch_time_pass(h, TIME_J, h->E, h->J, nullptr));
    PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, launch_fused_cart(h, SPEC_STAGE23, (float)(dz / 3), (float)dz, zh, ze));
    PROF_TRY(h, UPPE_CLASS_TIME, launch_time_pass(h, TIME_J, h->E, h->J, nullptr));
    PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
             launch_fused_cart(h, SPEC_FINISH, (float)(dz / 6), 0.f, ze, ze, /*zs_current=*/true));
    h->E_valid = 1;
    h->E_z = z_phase + dz;
    h->E_mat = h->mat_version;
    *dz_out = dz;
    return UPPE_OK;
}

// Cylindrical grids: inverse transform, time pass and forward transform per evaluation.
static int rk4_step_generic(UppeHandle* h, double z_phase, double L, double z_sub, double dzmin, bool adaptive,
                            double* dz_out) {
    double dz;
    h->E_valid = 0;
    if (adaptive) {
        StepArgs z = split_z(h, z_phase);
        CUDA_TRY(h, eval_to_J(h, h->qi, z));
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, spec_pass(h, SPEC_STORE_K, h->J, h->k1, nullptr, nullptr, 0.f, 0.f, z));
        int rc = estimate_dz(h, L, z_sub, dzmin, &dz);
        if (rc) return rc;
        PROF_TRY(h, UPPE_CLASS_STEP_SIZE, launch_apply_stage1(h, (float)(dz / 6), (float)(dz / 2)));
    } else {
        dz = L - z_sub;
        StepArgs z = split_z(h, z_phase);
        const StepArgs zn = split_z(h, z_phase + 0.5 * dz);
        CUDA_TRY(h, eval_to_J(h, h->qi, z));
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, spec_pass(h, SPEC_STAGE1, h->J, h->q, h->qf, h->qi, (float)(dz / 6),
                                                         (float)(dz / 2), z, h->tc_next ? &zn : nullptr));
    }
    {
        // each stage estimate is transformed next at zn: the spectral update that forms it also forms
        // that transform's operand (mixed form, one azimuthal node)
        StepArgs z = split_z(h, z_phase + 0.5 * dz);
        const StepArgs zn = split_z(h, z_phase + dz);
        CUDA_TRY(h, eval_to_J(h, h->q, z));
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
                 spec_pass(h, SPEC_STAGE23, h->J, h->q, h->qf, h->qi, (float)(dz / 3), (float)(dz / 2), z,
                           h->tc_next ? &z : nullptr));
        CUDA_TRY(h, eval_to_J(h, h->q, z));
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD,
                 spec_pass(h, SPEC_STAGE23, h->J, h->q, h->qf, h->qi, (float)(dz / 3), (float)dz, z,
                           h->tc_next ? &zn : nullptr));
    }
    {
        // the step's result is transformed next by the following step's first evaluation, at the
        // same z (a later call checks the source, z and material before using the tiles)
        StepArgs z = split_z(h, z_phase + dz);
        CUDA_TRY(h, eval_to_J(h, h->q, z));
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, spec_pass(h, SPEC_FINISH, h->J, h->qi, h->qf, nullptr, (float)(dz / 6),
                                                         0.f, z, h->tc_next ? &z : nullptr));
    }
    *dz_out = dz;
    return UPPE_OK;
}

extern "C" int uppe_rk4_step(UppeHandle* h, double z_phase, double L, double z_sub, double dzmin, double* dz_out) {
    if (!h) return UPPE_E_ARG;
    int rc = check_ready(h, true);
    if (rc) return rc;
    if (!(L > 0.0)) {
        uppe_set_error(h, "subcycle length must be positive");
        return UPPE_E_ARG;
    }
    const bool adaptive = !(dzmin >= L - z_sub);
    rc = check_range(h, z_phase + (L - z_sub));
    if (rc) return rc;
    h->kept_valid = 0;
    double dz = 0.0;
    rc = h->cfg.cylindrical ? rk4_step_generic(h, z_phase, L, z_sub, dzmin, adaptive, &dz)
                            : rk4_step_cartesian(h, z_phase, L, z_sub, dzmin, adaptive, &dz);
    if (rc) return rc;
    if (dz_out) *dz_out = dz;
    return UPPE_OK;
}

extern "C" int uppe_finish(UppeHandle* h, double z_phase, void* A, void* J, void* chi_w, void* ne_w) {
    if (!h) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    int rc = check_ready(h, true);
    if (rc) return rc;
    rc = check_range(h, z_phase);
    if (rc) return rc;
    StepArgs z = split_z(h, z_phase);
    h->E_valid = 0;
    PROF_TRY(h, UPPE_CLASS_OTHER, real_pass(h, REAL_FINISH, h->qi, (float2*)A, z));
    PROF_TRY(h, UPPE_CLASS_OTHER, launch_time_pass(h, TIME_J, h->E, J ? (float2*)J : h->J, nullptr));
    if (chi_w || ne_w) PROF_TRY(h, UPPE_CLASS_OTHER, launch_time_pass(h, TIME_CHI_NE, h->E, (float2*)chi_w, (float2*)ne_w));
    return UPPE_OK;
}

extern "C" int uppe_eval_rhs(UppeHandle* h, const void* q_in, double z_phase, void* S_out) {
    if (!h || !q_in || !S_out) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    int rc = check_ready(h, false);
    if (rc) return rc;
    rc = check_range(h, z_phase);
    if (rc) return rc;
    StepArgs z = split_z(h, z_phase);
    h->E_valid = 0;
    CUDA_TRY(h, eval_to_J(h, (const float2*)q_in, z));
    PROF_TRY(h, UPPE_CLASS_TRANSVERSE_FWD, spec_pass(h, SPEC_STORE_K, h->J, (float2*)S_out, nullptr, nullptr, 0.f, 0.f, z));
    return UPPE_OK;
}

extern "C" int uppe_get_field(UppeHandle* h, void* q_out) {
    if (!h || !q_out) return UPPE_E_ARG;
    int rc = check_ready(h, true);
    if (rc) return rc;
    CUDA_TRY(h, cudaMemcpyAsync(q_out, h->qi, h->P * sizeof(float2), cudaMemcpyDeviceToDevice, h->stream));
    return UPPE_OK;
}

extern "C" int uppe_check_finite(UppeHandle* h, int* nonfinite) {
    if (!h || !nonfinite) return UPPE_E_ARG;
    int rc = check_ready(h, true);
    if (rc) return rc;
    const float init[4] = {0.f, INFINITY, 0.f, 0.f};
    CUDA_TRY(h, cudaMemcpyAsync(h->red, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, launch_absmax(h, h->qi));
    float red[4];
    int derr = 0;
    CUDA_TRY(h, cudaMemcpyAsync(red, h->red, sizeof(red), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(&derr, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    *nonfinite = (red[2] != 0.f) ? 1 : 0;
    if (derr) {
        uppe_set_error(h, "a tensor-core kernel's bounded wait expired; results of this handle are invalid");
        return UPPE_E_CUDA;
    }
    return UPPE_OK;
}

// =============================================================================================
// Adjoint: vector-Jacobian products of the fixed-step RK4 map, of the load transform and of the
// finish transform, for gradients through torch.autograd.
// =============================================================================================
extern "C" int uppe_set_chi3(UppeHandle* h, double chi3_over_nref) {
    if (!h) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    h->redchi3 = chi3_over_nref;
    return UPPE_OK;
}

extern "C" int uppe_set_rotator(UppeHandle* h, int nstates, const double* Tj, const double* Wj, double dalpha,
                                double hbar) {
    if (!h || nstates < 0 || (nstates > 0 && (!Tj || !Wj))) {
        if (h) uppe_set_error(h, "uppe_set_rotator: invalid arguments");
        return UPPE_E_ARG;
    }
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (nstates > 0 && !(hbar > 0.0)) {
        uppe_set_error(h, "uppe_set_rotator: hbar must be positive (got %g)", hbar);
        return UPPE_E_ARG;
    }
    // transitions j -> j-2 for j >= 2 that contribute (T_j = 0 adds exactly nothing)
    std::vector<int> js;
    for (int j = 2; j < nstates; ++j)
        if (Tj[j] != 0.0) js.push_back(j);
    if (js.size() > 128) {
        uppe_set_error(h, "uppe_set_rotator: %zu contributing transitions exceed the 128 supported", js.size());
        return UPPE_E_ARG;
    }
    if (h->cfg.envelope) {
        const int keep = h->rot_pairs;
        h->rot_pairs = ((int)js.size() + 1) / 2;
        const size_t need = uppe_env_smem_bytes(h);
        h->rot_pairs = keep;
        if (need > 227 * 1024) {
            uppe_set_error(h, "uppe_set_rotator: the envelope time pass would need %zu bytes of shared memory", need);
            return UPPE_E_ARG;
        }
    }
    if (h->rot) {
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        CUDA_TRY(h, cudaFree(h->rot));
        h->rot = nullptr;
    }
    h->rot_pairs = 0;
    h->E_valid = 0;
    if (js.empty()) return UPPE_OK;
    // transitions in pairs (A, B); an odd count gets a null partner (h2 = 1, cq = 0: adds exactly 0)
    const int npair = ((int)js.size() + 1) / 2, nseg = h->Nt / 16;
    const double dt = h->cfg.dt, Nt = (double)h->Nt;
    // per pair 20 float4: the constants (4) and the powers h2^i, i < 16; then the phasors
    std::vector<float> tab((size_t)npair * 80 + (size_t)npair * nseg * 4, 0.f);
    for (size_t s = 0; s < 2 * (size_t)npair; ++s) {
        const int pr = (int)(s / 2), lane = (int)(s % 2);
        float* t = &tab[(size_t)80 * pr];
        float* p0 = &tab[(size_t)80 * npair + (size_t)4 * nseg * pr];
        if (s >= js.size()) {
            t[0 + lane] = 1.f;  // h2 = 1
            t[6 + lane] = 1.f;  // |h2|^2 = 1
            for (int i = 0; i < 16; ++i) t[16 + 4 * i + lane] = 1.f;
            for (int seg = 0; seg < nseg; ++seg) p0[4 * seg + lane] = 1.f;
            continue;
        }
        const int j = js[s];
        const std::complex<double> I(0.0, 1.0);
        const std::complex<double> wdt = std::complex<double>(Wj[2 * j], Wj[2 * j + 1]) * dt;
        const std::complex<double> h1 = std::exp(0.5 * I * wdt), h2 = std::exp(I * wdt);
        const double S = 2.0 * j * (j - 1) / (15.0 * (2 * j - 1));
        // cq = 2 dalpha T_j S_j wdt (-i dt) conj(1/h) fF / Nt^2: the drive F = fF z^2 of the time pass's
        // unnormalised field z = Nt E, fF = dalpha / (2 hbar) for the real field (AddChiUPPE) and
        // dalpha / (4 hbar) on |z|^2 for the envelope (AddChiParaxial: the cycle average of E^2 / 2)
        const double fF = (h->cfg.envelope ? 0.25 : 0.5) * dalpha / hbar;
        const std::complex<double> cq = 2.0 * dalpha * Tj[j] * S * wdt * (-I * dt) * std::conj(1.0 / h1) * fF /
                                        (Nt * Nt);
        t[0 + lane] = (float)h2.real();
        t[2 + lane] = (float)h2.imag();
        t[4 + lane] = (float)(-h2.imag());
        t[6 + lane] = (float)std::norm(h2);
        t[8 + lane] = (float)cq.real();
        t[10 + lane] = (float)cq.imag();
        for (int i = 0; i < 16; ++i) {
            const std::complex<double> hp = std::exp(I * wdt * (double)i);
            t[16 + 4 * i + lane] = (float)hp.real();
            t[16 + 4 * i + 2 + lane] = (float)hp.imag();
        }
        // phasor p = e^{i wdt (n + 1/2)} at the first sample n = Nt - 16 (seg + 1) of each segment
        for (int seg = 0; seg < nseg; ++seg) {
            const std::complex<double> p = std::exp(I * wdt * (Nt - 16.0 * (seg + 1) + 0.5));
            p0[4 * seg + lane] = (float)p.real();
            p0[4 * seg + 2 + lane] = (float)p.imag();
        }
    }
    void* d = nullptr;
    if (cudaMalloc(&d, tab.size() * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        uppe_set_error(h, "uppe_set_rotator: device allocation of %zu bytes failed", tab.size() * sizeof(float));
        return UPPE_E_NOMEM;
    }
    h->rot = (float*)d;
    CUDA_TRY(h, cudaMemcpy(h->rot, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    h->rot_pairs = npair;
    return UPPE_OK;
}

extern "C" int uppe_set_field(UppeHandle* h, const void* q) {
    if (!h || !q) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (!h->have_grid) {
        uppe_set_error(h, "uppe_set_field before uppe_set_grid");
        return UPPE_E_ARG;
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->qi, q, h->P * sizeof(float2), cudaMemcpyDeviceToDevice, h->stream));
    h->have_field = 1;
    h->E_valid = 0;
    return UPPE_OK;
}

static int ensure_adjoint(UppeHandle* h) {
    if (h->cfg.cylindrical && h->N2 != 1) {
        uppe_set_error(h, "the adjoint supports cylindrical grids with one azimuthal node only");
        return UPPE_E_ARG;
    }
    if (h->cfg.envelope) {
        uppe_set_error(h, "the adjoint is not built for the paraxial envelope solver");
        return UPPE_E_ARG;
    }
    if (h->adj_mu) return UPPE_OK;
    // Only buffers still missing are allocated, so a call after a failed allocation neither leaks
    // nor reallocates; adj_mu, the "allocated" mark, comes last, after the scalar dred_d.
    if (!h->dred_d) CUDA_TRY(h, cudaMalloc((void**)&h->dred_d, sizeof(double)));
    // the register-resident adjoint time pass: its list of column groups with ionization, and a park
    // for e(t) where the forward has no scratch (media without ionization)
    if (h->time_reg && h->tw_reg && time_reg_supported(h)) {
        if (!h->tscr && !h->adj_park)
            CUDA_TRY(h, cudaMalloc((void**)&h->adj_park, (size_t)h->S * h->M * sizeof(float2)));
        if (!h->adj_live) CUDA_TRY(h, cudaMalloc((void**)&h->adj_live, time_adj_reg_list_len(h) * sizeof(int)));
    }
    const size_t fb = h->P * sizeof(float2);
    float2** bufs[] = {&h->adj_q1, &h->adj_q2, &h->adj_q3,   &h->adj_lf,   &h->adj_acc,
                       &h->adj_lk, &h->adj_E[0], &h->adj_E[1], &h->adj_E[2], &h->adj_E[3],
                       &h->adj_mu};
    for (float2** b : bufs)
        if (!*b) CUDA_TRY(h, cudaMalloc((void**)b, fb));
    return UPPE_OK;
}

static cudaError_t adj_pass(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
    return h->cfg.cylindrical ? launch_adj_cyl(h, mode, in, out, z) : launch_adj_cart(h, mode, in, out, z);
}

// mu = S'(qs)^H lamk at z = zs (the right-hand side of load_source, uppe_kernel.py:188-216)
// Es: E of (qs, zs) when the recompute kept it, else formed here.
static int vjp_rhs(UppeHandle* h, const float2* qs, double zs, const float2* lamk, float2* mu, const float2* Es) {
    const StepArgs z = split_z(h, zs);
    h->E_valid = 0;
    if (!Es) {
        PROF_TRY(h, UPPE_CLASS_OTHER, real_pass(h, REAL_E, qs, nullptr, z));
        Es = h->E;
    }
    PROF_TRY(h, UPPE_CLASS_OTHER, adj_pass(h, ADJ_S, lamk, h->J, z));
    // cylindrical mixed form, one azimuthal node: the cotangent of E goes straight into the operand
    // tiles of the Minv^T transform that follows
    const bool to_tc = h->cfg.cylindrical && h->cfg.precision == UPPE_PREC_MIXED && h->N2 == 1 && h->tc_next &&
                       h->Atc && !h->cfg.envelope;
    {
        ProfScope ps(h, UPPE_CLASS_OTHER);
        h->time_atc = to_tc ? 1 : 0;
        const cudaError_t et = launch_time_adjoint(h, Es, h->J, h->k1, h->dred_d);
        h->time_atc = 0;
        CUDA_TRY(h, et);
    }
    h->atc_fwd = to_tc ? 1 : 0;
    h->atc_fwd_which = 3;
    h->atc_fwd_src = h->k1;
    PROF_TRY(h, UPPE_CLASS_OTHER, adj_pass(h, ADJ_E, h->k1, mu, z));
    return UPPE_OK;
}

// The reverse RK4 sweep on Cartesian grids (register-resident or big slices), from the E of the four
// stage states in adj_E[0..3]: per stage the adjoint time pass, then one slice pass that finishes the
// stage (cotangent of q, RK bookkeeping) and forms the next stage's cotangent of J.  dred_d is
// accumulated from zero.
static int reverse_sweep_fused(UppeHandle* h, const float2* lam_out, float2* lam_in, double z_phase, double dz,
                               double* dred_out) {
    CUDA_TRY(h, cudaMemsetAsync(h->dred_d, 0, sizeof(double), h->stream));
    CUDA_TRY(h, launch_adj_rk(h, 0, lam_out, nullptr, (float)(dz / 6), 0.f));
    const StepArgs z0 = split_z(h, z_phase), zh = split_z(h, z_phase + 0.5 * dz), ze = split_z(h, z_phase + dz);
    const float2* const Es[4] = {h->adj_E[3], h->adj_E[2], h->adj_E[1], h->adj_E[0]};
    const float af[3] = {(float)(dz / 3), (float)(dz / 3), (float)(dz / 6)};
    const float am[3] = {(float)dz, (float)(dz / 2), (float)(dz / 2)};
    const StepArgs ze_[4] = {ze, zh, zh, z0};
    h->E_valid = 0;
    PROF_TRY(h, UPPE_CLASS_OTHER, adj_pass(h, ADJ_S, h->adj_lk, h->J, ze));
    for (int s = 0; s < 4; ++s) {
        PROF_TRY(h, UPPE_CLASS_OTHER, launch_time_adjoint(h, Es[s], h->J, h->k1, h->dred_d));
        const int mode = (s < 3) ? 1 : 2;
        float2* const out = (s < 3) ? h->J : lam_in;
        const float a_f = (s < 3) ? af[s] : 0.f, a_mu = (s < 3) ? am[s] : 0.f;
        const StepArgs z_s = (s < 3) ? ze_[s + 1] : z0;
        if (h->slice_big) {
            PROF_TRY(h, UPPE_CLASS_OTHER, launch_adj_fused_big(h, mode, h->k1, out, a_f, a_mu, ze_[s], z_s));
        } else {
            PROF_TRY(h, UPPE_CLASS_OTHER, launch_adj_fused_reg(h, mode, h->k1, out, a_f, a_mu, ze_[s], z_s));
        }
    }
    if (dred_out) {
        double d = 0.0;
        CUDA_TRY(h, cudaMemcpyAsync(&d, h->dred_d, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        *dred_out += d;
    }
    return UPPE_OK;
}

// The reverse RK4 sweep with separate transverse passes (cylindrical grids and the generic Cartesian
// slices), from the stage estimates adj_q1..3 and the E of the stage states q0, q1', q2' in
// adj_E[0..2].  E of q3' is formed here unless q0 is NULL, in which case adj_E[3] holds it (a kept
// step).  dred_d is accumulated from zero.
static int reverse_sweep_generic(UppeHandle* h, const float2* lam_out, float2* lam_in, double z_phase, double dz,
                                 double* dred_out, const float2* q0) {
    int rc;
    CUDA_TRY(h, cudaMemsetAsync(h->dred_d, 0, sizeof(double), h->stream));
    CUDA_TRY(h, launch_adj_rk(h, 0, lam_out, nullptr, (float)(dz / 6), 0.f));
    if ((rc = vjp_rhs(h, h->adj_q3, z_phase + dz, h->adj_lk, h->adj_mu, q0 ? nullptr : h->adj_E[3]))) return rc;
    CUDA_TRY(h, launch_adj_rk(h, 1, nullptr, nullptr, (float)(dz / 3), (float)dz));
    if ((rc = vjp_rhs(h, h->adj_q2, z_phase + 0.5 * dz, h->adj_lk, h->adj_mu, h->adj_E[2]))) return rc;
    CUDA_TRY(h, launch_adj_rk(h, 1, nullptr, nullptr, (float)(dz / 3), (float)(dz / 2)));
    if ((rc = vjp_rhs(h, h->adj_q1, z_phase + 0.5 * dz, h->adj_lk, h->adj_mu, h->adj_E[1]))) return rc;
    CUDA_TRY(h, launch_adj_rk(h, 1, nullptr, nullptr, (float)(dz / 6), (float)(dz / 2)));
    if ((rc = vjp_rhs(h, q0, z_phase, h->adj_lk, h->adj_mu, h->adj_E[0]))) return rc;
    CUDA_TRY(h, launch_adj_rk(h, 2, nullptr, lam_in, 0.f, 0.f));
    if (dred_out) {
        double d = 0.0;
        CUDA_TRY(h, cudaMemcpyAsync(&d, h->dred_d, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        *dred_out += d;
    }
    return UPPE_OK;
}

extern "C" int uppe_adjoint_rk4_step(UppeHandle* h, const void* q0v, const void* lam_out, void* lam_in, double z_phase,
                                     double dz, double* dred_out) {
    if (!h || !q0v || !lam_out || !lam_in) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    int rc = check_ready(h, false);
    if (rc) return rc;
    rc = ensure_adjoint(h);
    if (rc) return rc;
    rc = check_range(h, z_phase + dz);
    if (rc) return rc;
    const float2* q0 = (const float2*)q0v;
    h->kept_valid = 0;  // the recompute below overwrites the kept stage fields
    CUDA_TRY(h, cudaMemsetAsync(h->dred_d, 0, sizeof(double), h->stream));
    // recompute the stage estimates q1', q2', q3' of the forward step (uppe_kernel.py:305-322)
    CUDA_TRY(h, cudaMemcpyAsync(h->qi, q0, h->P * sizeof(float2), cudaMemcpyDeviceToDevice, h->stream));
    h->E_valid = 0;
    // register-resident Cartesian slices: the forward step's own kernels, the time pass and the fused
    // slice pass per stage, with the fused pass also storing the stage estimate (stage_q) and its E
    // going to the buffer the reverse sweep reads, so that E of q3' at z + dz is kept as well
    const bool fused = !h->cfg.cylindrical && (h->slice_big || h->slice_reg);
    if (fused) {
        const StepArgs z0 = split_z(h, z_phase), zh = split_z(h, z_phase + 0.5 * dz), ze = split_z(h, z_phase + dz);
        float2* const E_main = h->E;
        float2* const qs[3] = {h->adj_q1, h->adj_q2, h->adj_q3};
        const int modes[3] = {SPEC_STAGE1, SPEC_STAGE23, SPEC_STAGE23};
        const float cs[3] = {(float)(dz / 6), (float)(dz / 3), (float)(dz / 3)};
        const float ce[3] = {(float)(dz / 2), (float)(dz / 2), (float)dz};
        const StepArgs zr[3] = {z0, zh, zh}, zn[3] = {zh, zh, ze};
        h->E = h->adj_E[0];
        cudaError_t e = eval_to_J(h, h->qi, z0);
        for (int s = 0; s < 3 && e == cudaSuccess; ++s) {
            h->E = h->adj_E[s + 1];
            h->stage_q = qs[s];
            {
                ProfScope ps(h, UPPE_CLASS_OTHER);
                e = launch_fused_cart(h, modes[s], cs[s], ce[s], zr[s], zn[s]);
            }
            h->stage_q = nullptr;
            if (e == cudaSuccess && s < 2) {
                ProfScope ps(h, UPPE_CLASS_TIME);
                e = launch_time_pass(h, TIME_J, h->E, h->J, nullptr);
            }
        }
        h->E = E_main;
        h->stage_q = nullptr;
        CUDA_TRY(h, e);
    } else {
        const StepArgs z0 = split_z(h, z_phase), zh = split_z(h, z_phase + 0.5 * dz);
        // each stage writes its estimate straight into the buffer the reverse sweep reads, and each
        // evaluation keeps its E (the inverse pass writes into h->E, pointed at adj_E[s] meanwhile)
        float2* const E_main = h->E;
        h->E = h->adj_E[0];
        cudaError_t e = eval_to_J(h, h->qi, z0);
        h->E = E_main;
        CUDA_TRY(h, e);
        PROF_TRY(h, UPPE_CLASS_OTHER, spec_pass(h, SPEC_STAGE1, h->J, h->adj_q1, h->qf, h->qi, (float)(dz / 6), (float)(dz / 2), z0));
        h->E = h->adj_E[1];
        e = eval_to_J(h, h->adj_q1, zh);
        h->E = E_main;
        CUDA_TRY(h, e);
        PROF_TRY(h, UPPE_CLASS_OTHER, spec_pass(h, SPEC_STAGE23, h->J, h->adj_q2, h->qf, h->qi, (float)(dz / 3), (float)(dz / 2), zh));
        h->E = h->adj_E[2];
        e = eval_to_J(h, h->adj_q2, zh);
        h->E = E_main;
        CUDA_TRY(h, e);
        PROF_TRY(h, UPPE_CLASS_OTHER, spec_pass(h, SPEC_STAGE23, h->J, h->adj_q3, h->qf, h->qi, (float)(dz / 3), (float)dz, zh));
    }
    // reverse sweep through the four stages
    if (fused) return reverse_sweep_fused(h, (const float2*)lam_out, (float2*)lam_in, z_phase, dz, dred_out);
    return reverse_sweep_generic(h, (const float2*)lam_out, (float2*)lam_in, z_phase, dz, dred_out, q0);
}

// One fixed RK4 step (as uppe_rk4_step with dzmin = L - z_sub) that keeps the E of its four stage
// states in adj_E[0..3] (and, with separate transverse passes, the stage estimates in adj_q1..3),
// for uppe_adjoint_rk4_step_kept.  On the register-resident and big-slice passes the slices without
// current are processed in every stage (their E is kept).
extern "C" int uppe_rk4_step_keep(UppeHandle* h, double z_phase, double dz) {
    if (!h) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    int rc = check_ready(h, true);
    if (rc) return rc;
    if (!(dz > 0.0)) {
        uppe_set_error(h, "step must be positive");
        return UPPE_E_ARG;
    }
    rc = ensure_adjoint(h);
    if (rc) return rc;
    rc = check_range(h, z_phase + dz);
    if (rc) return rc;
    h->kept_valid = 0;
    const StepArgs z0 = split_z(h, z_phase), zh = split_z(h, z_phase + 0.5 * dz), ze = split_z(h, z_phase + dz);
    float2* const E_main = h->E;
    if (h->cfg.cylindrical || !(h->slice_reg || h->slice_big)) {
        // separate passes per evaluation: each evaluation's E and each stage estimate kept
        float2* const qs[3] = {h->adj_q1, h->adj_q2, h->adj_q3};
        const float2* const qin[4] = {h->qi, h->adj_q1, h->adj_q2, h->adj_q3};
        const int modes[4] = {SPEC_STAGE1, SPEC_STAGE23, SPEC_STAGE23, SPEC_FINISH};
        const float cs[4] = {(float)(dz / 6), (float)(dz / 3), (float)(dz / 3), (float)(dz / 6)};
        const float ce[4] = {(float)(dz / 2), (float)(dz / 2), (float)dz, 0.f};
        const StepArgs zr[4] = {z0, zh, zh, ze};
        h->E_valid = 0;
        cudaError_t e = cudaSuccess;
        for (int s = 0; s < 4 && e == cudaSuccess; ++s) {
            h->E = h->adj_E[s];
            e = eval_to_J(h, qin[s], zr[s]);
            h->E = E_main;
            if (e != cudaSuccess) break;
            ProfScope ps(h, UPPE_CLASS_TRANSVERSE_FWD);
            e = (s < 3) ? spec_pass(h, modes[s], h->J, qs[s], h->qf, h->qi, cs[s], ce[s], zr[s])
                        : spec_pass(h, SPEC_FINISH, h->J, h->qi, h->qf, nullptr, cs[s], 0.f, zr[s]);
        }
        CUDA_TRY(h, e);
        h->kept_valid = 1;
        h->kept_z = z_phase;
        h->kept_dz = dz;
        h->kept_mat = h->mat_version;
        return UPPE_OK;
    }
    // E of q0 at z0 into adj_E[0]: the E left by the previous step's finish when it is current
    if (h->E_valid && h->E_mat == h->mat_version && same_z(h->E_z, z_phase)) {
        h->E = h->adj_E[0];
        h->adj_E[0] = E_main;
    } else {
        h->E = h->adj_E[0];
        cudaError_t e = launch_real_cart(h, REAL_E, h->qi, nullptr, z0);
        h->E = E_main;
        PROF_TRY(h, UPPE_CLASS_TRANSVERSE_INV, e);
    }
    float2* const E_next = h->E;  // the buffer that takes E of the step's result
    h->E_valid = 0;
    const int modes[4] = {SPEC_STAGE1, SPEC_STAGE23, SPEC_STAGE23, SPEC_FINISH};
    const float cs[4] = {(float)(dz / 6), (float)(dz / 3), (float)(dz / 3), (float)(dz / 6)};
    const float ce[4] = {(float)(dz / 2), (float)(dz / 2), (float)dz, 0.f};
    const StepArgs zr[4] = {z0, zh, zh, ze}, zn[4] = {zh, zh, ze, ze};
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < 4 && e == cudaSuccess; ++s) {
        {
            ProfScope ps(h, UPPE_CLASS_TIME);
            e = launch_time_pass(h, TIME_J, h->adj_E[s], h->J, nullptr);
        }
        if (e != cudaSuccess) break;
        h->E = (s < 3) ? h->adj_E[s + 1] : E_next;
        ProfScope ps(h, UPPE_CLASS_TRANSVERSE_FWD);
        e = launch_fused_cart(h, modes[s], cs[s], ce[s], zr[s], zn[s], /*zs_current=*/false);
    }
    h->E = E_next;
    CUDA_TRY(h, e);
    h->E_valid = 1;
    h->E_z = z_phase + dz;
    h->E_mat = h->mat_version;
    h->kept_valid = 1;
    h->kept_z = z_phase;
    h->kept_dz = dz;
    h->kept_mat = h->mat_version;
    return UPPE_OK;
}

// The vector-Jacobian product of the step last taken by uppe_rk4_step_keep (lam_in = (dq1/dq0)^H
// lam_out), from its kept stage fields: uppe_adjoint_rk4_step without the recompute.
extern "C" int uppe_adjoint_rk4_step_kept(UppeHandle* h, const void* lam_out, void* lam_in, double* dred_out) {
    if (!h || !lam_out || !lam_in) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (!h->kept_valid || h->kept_mat != h->mat_version) {
        uppe_set_error(h, "uppe_adjoint_rk4_step_kept: no step kept by uppe_rk4_step_keep for the current material");
        return UPPE_E_ARG;
    }
    if (h->cfg.cylindrical || !(h->slice_reg || h->slice_big))
        return reverse_sweep_generic(h, (const float2*)lam_out, (float2*)lam_in, h->kept_z, h->kept_dz, dred_out,
                                     nullptr);
    return reverse_sweep_fused(h, (const float2*)lam_out, (float2*)lam_in, h->kept_z, h->kept_dz, dred_out);
}

extern "C" int uppe_adjoint_load(UppeHandle* h, const void* lam_q, void* lam_a) {
    if (!h || !lam_q || !lam_a) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    if (!h->have_grid) {
        uppe_set_error(h, "uppe_adjoint_load before uppe_set_grid");
        return UPPE_E_ARG;
    }
    int rc = ensure_adjoint(h);
    if (rc) return rc;
    CUDA_TRY(h, adj_pass(h, ADJ_LOAD, (const float2*)lam_q, (float2*)lam_a, split_z(h, 0.0)));
    return UPPE_OK;
}

extern "C" int uppe_adjoint_finish(UppeHandle* h, double z_phase, const void* lam_A, void* lam_q) {
    if (!h || !lam_A || !lam_q) return UPPE_E_ARG;
    h->atc_next = 0;  // Atc tiles carried between rk4 steps are void after any other call
    int rc = check_ready(h, false);
    if (rc) return rc;
    rc = ensure_adjoint(h);
    if (rc) return rc;
    CUDA_TRY(h, adj_pass(h, ADJ_FIN, (const float2*)lam_A, (float2*)lam_q, split_z(h, z_phase)));
    return UPPE_OK;
}

extern "C" int uppe_profile_enable(UppeHandle* h, int enable) {
    if (!h) return UPPE_E_ARG;
    if (enable) {
        if (!h->prof) h->prof = new (std::nothrow) ProfState();
        if (!h->prof) return UPPE_E_NOMEM;
        ProfState* ps = (ProfState*)h->prof;
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        ps->pending.clear();
        ps->next = 0;
        for (int i = 0; i < UPPE_NCLASS; ++i) {
            ps->ms[i] = 0.0;
            ps->count[i] = 0;
        }
    } else if (h->prof) {
        CUDA_TRY(h, prof_resolve(h));
        ProfState* ps = (ProfState*)h->prof;
        for (cudaEvent_t e : ps->pool) cudaEventDestroy(e);
        delete ps;
        h->prof = nullptr;
    }
    return UPPE_OK;
}

extern "C" int uppe_profile_read(UppeHandle* h, double* ms, long long* count) {
    if (!h || !ms || !count) return UPPE_E_ARG;
    ProfState* ps = (ProfState*)h->prof;
    if (!ps) {
        uppe_set_error(h, "profiling is not enabled");
        return UPPE_E_ARG;
    }
    CUDA_TRY(h, prof_resolve(h));
    for (int i = 0; i < UPPE_NCLASS; ++i) {
        ms[i] = ps->ms[i];
        count[i] = ps->count[i];
    }
    return UPPE_OK;
}

extern "C" int uppe_launch_count(UppeHandle* h, long long* n) {
    if (!h || !n) return UPPE_E_ARG;
    *n = h->launches;
    return UPPE_OK;
}

extern "C" const char* uppe_class_name(int cls) {
    static const char* names[UPPE_NCLASS] = {"operator", "transverse_inverse", "time_pass", "transverse_forward_rk",
                                             "step_size", "finish"};
    return (cls >= 0 && cls < UPPE_NCLASS) ? names[cls] : "unknown";
}

extern "C" const char* uppe_last_error(const UppeHandle* h) { return h ? h->err : g_create_error; }
