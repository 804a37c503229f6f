// Adaptive step-size estimate that performs no device allocation.
//
// Who needs it: a caller whose own host program may not allocate device memory once it is
// running.  Examples are a driver that reserves all device memory up front and forbids later
// cudaMalloc calls, or a code path whose allocator would synchronise the device mid-stream.  Such a
// caller cannot create a handle (uppe_create allocates the work buffers).  It can still ask for the
// next RK4 step size from q and S = dq/dz, which it keeps in its own device memory.
//
// The reduction scratch is a file-scope __device__ array of fixed size.  It lives in this file's
// own CUDA module, which the runtime loads onto a device on first use (lazy module loading, the
// default in current CUDA): the first call on each device therefore loads the module, resolves the
// array's address and loads the four kernels, and only that first call may allocate device memory
// (for the array and the kernels' code).  From then on the array stays on that device until the
// process exits.  The caller passes only inputs (q, S) and the output (dz, one float in device
// memory).
#include <math.h>
#include <mutex>

#include "common.cuh"
#include "uppe_internal.h"

#define NOALLOC_CHUNK 8192                                           // points per block
#define NOALLOC_MAX_BLOCKS (UPPE_NOALLOC_MAX_POINTS / NOALLOC_CHUNK)  // 16384
// layout: [0, MAXB) partial max|q|; [MAXB, 2 MAXB) partial min dz; [2 MAXB] max|q|
#define NOALLOC_SCRATCH_FLOATS (2 * NOALLOC_MAX_BLOCKS + 4)

static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCRATCH_FLOATS];

__device__ __forceinline__ float na_warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float na_warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reduction of one float; identity `id`, op max (is_max) or min.
__device__ __forceinline__ float na_block_reduce(float v, bool is_max, float id) {
    __shared__ float sred[32];
    v = is_max ? na_warp_max(v) : na_warp_min(v);
    if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = id;
    if (threadIdx.x < 32) {
        r = (threadIdx.x < (blockDim.x >> 5)) ? sred[threadIdx.x] : id;
        r = is_max ? na_warp_max(r) : na_warp_min(r);
    }
    return r;  // valid in thread 0
}

// fmaxf and fminf drop NaN operands, so a non-finite value is tracked separately: a block's
// partial result becomes NaN when its chunk holds one, and the final reductions pass NaN on.

// Pass 1: each block writes max|q| over its chunk (NaN if the chunk holds a non-finite q).
__global__ void k_na_absmax_partial(const float2* __restrict__ q, long long n, float* scratch) {
    const long long b0 = (long long)blockIdx.x * NOALLOC_CHUNK;
    long long b1 = b0 + NOALLOC_CHUNK;
    if (b1 > n) b1 = n;
    float m = 0.f;
    bool bad = false;
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        float2 v = q[i];
        const float a = sqrtf(v.x * v.x + v.y * v.y);
        bad = bad || !isfinite(a);
        m = fmaxf(m, a);
    }
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    m = na_block_reduce(m, true, 0.f);
    if (threadIdx.x == 0) scratch[blockIdx.x] = bad ? NAN : m;
}

// Pass 2: one block reduces the partial maxima into scratch[2 MAXB] (NaN if any partial is NaN).
__global__ void k_na_absmax_final(int nblocks, float* scratch) {
    float m = 0.f;
    bool bad = false;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        const float v = scratch[i];
        bad = bad || isnan(v);
        m = fmaxf(m, v);
    }
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    m = na_block_reduce(m, true, 0.f);
    if (threadIdx.x == 0) scratch[2 * NOALLOC_MAX_BLOCKS] = bad ? NAN : m;
}

// Pass 3: per-block min of dphi / K (paraxial.cl:40-58) with amin = rel_amin * max|q|.
__global__ void k_na_dz_partial(const float2* __restrict__ q, const float2* __restrict__ k, long long n,
                                float* scratch, float minRate, float dphi, float rel_amin) {
    const float amin = rel_amin * scratch[2 * NOALLOC_MAX_BLOCKS];
    const float amin2 = amin * amin;
    const long long b0 = (long long)blockIdx.x * NOALLOC_CHUNK;
    long long b1 = b0 + NOALLOC_CHUNK;
    if (b1 > n) b1 = n;
    float m = INFINITY;
    bool bad = isnan(amin);
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        float2 Q = q[i], S = k[i];
        bad = bad || !isfinite(S.x) || !isfinite(S.y);
        float den = Q.x * Q.x + Q.y * Q.y + amin2;
        float alpha = (Q.x * S.x + Q.y * S.y) / den;
        float keff = (Q.x * S.y - Q.y * S.x) / den;
        float K = minRate + fabsf(keff) - (alpha < 0.f ? alpha : 0.f);
        m = fminf(m, dphi / K);
    }
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    m = na_block_reduce(m, false, INFINITY);
    if (threadIdx.x == 0) scratch[NOALLOC_MAX_BLOCKS + blockIdx.x] = bad ? NAN : m;
}

// Pass 4: one block reduces the partial minima into the caller's output (NaN if any is NaN).
__global__ void k_na_dz_final(int nblocks, const float* scratch, float* dz_out) {
    float m = INFINITY;
    bool bad = false;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        const float v = scratch[NOALLOC_MAX_BLOCKS + i];
        bad = bad || isnan(v);
        m = fminf(m, v);
    }
    bad = __syncthreads_or(bad ? 1 : 0) != 0;
    m = na_block_reduce(m, false, INFINITY);
    if (threadIdx.x == 0) *dz_out = bad ? NAN : m;
}

// Device address of the scratch array, looked up once per device with that device current.  The
// same set-up loads the four kernels (cudaFuncGetAttributes), so that under lazy module loading
// no later call loads anything.  The address is that of the device's primary context (the one the
// runtime API uses); it is not refreshed after cudaDeviceReset.
#define NOALLOC_MAX_DEVICES 64
static float* g_scratch_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mutex;

static int scratch_for_current_device(float** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        uppe_set_error(nullptr, "uppe_step_size_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return UPPE_E_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            uppe_set_error(nullptr, "uppe_step_size_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return UPPE_E_CUDA;
        }
        const void* kernels[] = {(const void*)k_na_absmax_partial, (const void*)k_na_absmax_final,
                                 (const void*)k_na_dz_partial, (const void*)k_na_dz_final};
        for (const void* f : kernels) {
            cudaFuncAttributes attr;
            e = cudaFuncGetAttributes(&attr, f);
            if (e != cudaSuccess) {
                uppe_set_error(nullptr, "uppe_step_size_noalloc: loading its kernels failed: %s", cudaGetErrorString(e));
                return UPPE_E_CUDA;
            }
        }
        g_scratch_ptr[dev] = (float*)ptr;
    }
    *out = g_scratch_ptr[dev];
    return UPPE_OK;
}

extern "C" int uppe_step_size_noalloc(const void* q, const void* S, long long n, double L, double dphi,
                                      double rel_amin, void* dz_out, void* stream) {
    if (!q || !S || !dz_out) {
        uppe_set_error(nullptr, "uppe_step_size_noalloc: null pointer argument");
        return UPPE_E_ARG;
    }
    if (n <= 0) {
        uppe_set_error(nullptr, "uppe_step_size_noalloc: n must be positive (got %lld)", n);
        return UPPE_E_ARG;
    }
    if (n > (long long)UPPE_NOALLOC_MAX_POINTS) {
        uppe_set_error(nullptr,
                       "uppe_step_size_noalloc: %lld points exceed the fixed scratch limit of %lld points; "
                       "use a handle (uppe_rk4_step) for larger grids",
                       n, (long long)UPPE_NOALLOC_MAX_POINTS);
        return UPPE_E_RANGE;
    }
    if (!(L > 0.0) || !(dphi > 0.0)) {
        uppe_set_error(nullptr, "uppe_step_size_noalloc: L and dphi must be positive");
        return UPPE_E_ARG;
    }
    float* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int nblocks = (int)((n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK);
    // every cell read below is written earlier in the same call, so no clearing is needed
    k_na_absmax_partial<<<nblocks, 256, 0, st>>>((const float2*)q, n, scratch);
    k_na_absmax_final<<<1, 1024, 0, st>>>(nblocks, scratch);
    k_na_dz_partial<<<nblocks, 256, 0, st>>>((const float2*)q, (const float2*)S, n, scratch,
                                             (float)(0.5 * dphi / L), (float)dphi, (float)rel_amin);
    k_na_dz_final<<<1, 1024, 0, st>>>(nblocks, scratch, (float*)dz_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        uppe_set_error(nullptr, "uppe_step_size_noalloc: launch failed: %s", cudaGetErrorString(e));
        return UPPE_E_CUDA;
    }
    return UPPE_OK;
}
