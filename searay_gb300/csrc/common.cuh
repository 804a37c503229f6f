// Shared device helpers for the GB300 UPPE propagator: complex arithmetic on float2, float-float
// ("double-single") arithmetic for the FP64-grade islands, and the propagator phase.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define UPPE_DEV __device__ __forceinline__

// Programmatic dependent launch.  A kernel launched with launch_pdl may start (its blocks resident,
// their set-up done) while the kernel before it in the stream is still draining; it calls
// pdl_begin() before its first global-memory access.  pdl_begin lets the next kernel of the stream
// launch once every block of this one has begun (griddepcontrol.launch_dependents: all of this
// grid's blocks are then resident, so the next grid's waiting blocks can never keep one of them
// out), then waits for the previous kernel to complete with its memory visible
// (griddepcontrol.wait; it returns at once when there is none, or the kernel was launched plainly).
UPPE_DEV void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

#ifdef __CUDACC__
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args... args) {
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

UPPE_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
UPPE_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
UPPE_DEV float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
UPPE_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
UPPE_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by +i / -i
UPPE_DEV float2 cmul_i(float2 a) { return make_float2(-a.y, a.x); }
UPPE_DEV float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }
// a / b for complex b
UPPE_DEV float2 cdiv(float2 a, float2 b) {
    float d = b.x * b.x + b.y * b.y;
    return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// ---------------------------------------------------------------------------------------------
// float-float arithmetic.  GB300 runs FP64 at a small fraction of its FP32 rate, so the two places
// that need more than FP32 (the (kz+kg)z phase over long z and the time-integrated ionization
// density) carry a value as an unevaluated sum hi + lo of two floats, about 48 significant bits.
// Error-free transformations: Knuth's two-sum and the FMA-based two-product.
// ---------------------------------------------------------------------------------------------
struct ffloat {
    float hi, lo;
};

UPPE_DEV ffloat ff_two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

UPPE_DEV ffloat ff_quick(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}

UPPE_DEV ffloat ff_add(ffloat a, ffloat b) {
    ffloat s = ff_two_sum(a.hi, b.hi);
    float e = s.lo + (a.lo + b.lo);
    return ff_quick(s.hi, e);
}

UPPE_DEV ffloat ff_add_f(ffloat a, float b) {
    ffloat s = ff_two_sum(a.hi, b);
    float e = s.lo + a.lo;
    return ff_quick(s.hi, e);
}

UPPE_DEV float ff_value(ffloat a) { return a.hi + a.lo; }

// 2*pi split in three floats (Cody-Waite): TWO_PI_A has its low bits clear enough that n*TWO_PI_A
// subtracted from a float phase with an FMA is exact for |phase| < 2^24.
#define UPPE_TWO_PI_A 6.28318548202514648437e+00f
#define UPPE_TWO_PI_B -1.74845553146951715461e-07f
#define UPPE_INV_TWO_PI 1.59154943091895335769e-01f

// Phase (K z) mod 2*pi from K = Khi + Klo and z = zhi + zlo, each a float-float value.
// The product is formed with an exact two-product of the high parts; the result is accurate to
// about 3e-7 rad for |K z| up to ~1e8 rad.
UPPE_DEV float ff_phase(float Khi, float Klo, float zhi, float zlo) {
    float p = Khi * zhi;
    float e = fmaf(Khi, zhi, -p);
    e = fmaf(Khi, zlo, e);
    e = fmaf(Klo, zhi, e);
    float n = rintf(p * UPPE_INV_TWO_PI);
    float r = fmaf(-n, UPPE_TWO_PI_A, p);
    r = fmaf(-n, UPPE_TWO_PI_B, r);
    return r + e;
}

// Per-point linear operator, built once per material update.  The propagator factor is
//   exp(i (kz + kg) z) = exp(-Im(kz) z) * exp(i K z),   K = Re(kz) + kg(w),
// so every point stores K as a float-float pair (8 bytes).  Re(kz) is recovered as K - kg(w) with
// kg(w) = -w/v_window held per frequency (also float-float); Im(kz) is stored per point only for
// absorbing media (complex chi), otherwise it is zero.
struct OpView {
    const float2* __restrict__ K;    // [P] {hi, lo}
    const float* __restrict__ ki;    // [P] Im kz, or nullptr when the medium is real
    const float2* __restrict__ kg;   // [N0] {hi, lo}; envelope solver: {k0(w), 0}
    int envelope;                    // paraxial envelope solver: E = A, RHS divisor k0(w)
    int ncond;                       // w-bins zeroed by the DC conditioner (4, or 0 for the envelope)
};

struct OpPoint {
    float Khi, Klo, kzr, kzi;
};

UPPE_DEV OpPoint op_at(const OpView& v, size_t idx, float2 kgw) {
    const float2 k = v.K[idx];
    OpPoint o;
    o.Khi = k.x;
    o.Klo = k.y;
    // kzr: Re kz (the RHS divisor and the i kz factor of E); the envelope solver divides by k0(w)
    o.kzr = v.envelope ? kgw.x : (k.x - kgw.x) + (k.y - kgw.y);
    o.kzi = v.ki ? v.ki[idx] : 0.f;
    return o;
}

// i kz
UPPE_DEV float2 op_ikz(const OpPoint& o) { return make_float2(-o.kzi, o.kzr); }

// The field that the time pass reads, from the real-space spectral amplitude a: E = i kz a for UPPE
// (uppe_kernel.py:212), a itself for the envelope solver (paraxial_kernel.py:196).
UPPE_DEV float2 op_field(const OpView& v, const OpPoint& o, float2 a) { return v.envelope ? a : cmul(op_ikz(o), a); }

struct PhaseArgs {
    float zhi, zlo;  // z as float-float
    int plain;       // 1: plain FP32 phase K*z (no float-float), for the plain-FP32 form
};

UPPE_DEV float2 propagator_factor(const OpPoint& o, PhaseArgs pa, float sign) {
    float s, c;
    if (pa.plain) {
        // plain FP32 form: the phase K z in FP32, full-range sincos
        sincosf(o.Khi * (pa.zhi + pa.zlo), &s, &c);
    } else {
        // float-float phase already reduced to about [-pi, pi]: the hardware sin/cos is accurate to
        // a few 1e-7 absolute on that range
        __sincosf(ff_phase(o.Khi, o.Klo, pa.zhi, pa.zlo), &s, &c);
    }
    // sign=+1: exp(i K z) exp(-Ki z);  sign=-1: exp(-i K z) exp(+Ki z)
    if (o.kzi == 0.f) return make_float2(c, sign * s);
    const float amp = expf(-sign * o.kzi * (pa.zhi + pa.zlo));
    return make_float2(amp * c, sign * amp * s);
}

// Ask the memory system to bring `bytes` (a multiple of 16, 16-byte aligned) into L2 ahead of use.
UPPE_DEV void prefetch_l2(const void* p, size_t bytes) {
    const char* c = (const char*)p;
    for (size_t off = 0; off < bytes; off += 32768) {
        const unsigned n = (unsigned)((bytes - off) < 32768 ? (bytes - off) : 32768);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(c + off), "r"(n) : "memory");
    }
}

__host__ __device__ inline int ilog2_exact(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}
