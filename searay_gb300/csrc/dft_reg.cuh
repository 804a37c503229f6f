// In-register DFTs of 16 and 32 points (natural order in and out) with compile-time twiddles,
// shared by the register-resident slice transforms (slice_reg.cuh) and the register-resident time
// pass (timepass_reg.cu).  Forward: X[k] = sum_n x[n] exp(-2 pi i n k / N); INV: the conjugate
// twiddles, unnormalised.
#pragma once
#include "common.cuh"
#include "fft_smem.cuh"

#define UPPE_COS_PI8 0.92387953251128675613f
#define UPPE_SIN_PI8 0.38268343236508977173f
#define UPPE_COS_PI16 0.98078528040323044913f
#define UPPE_SIN_PI16 0.19509032201612826785f
#define UPPE_COS_3PI16 0.83146961230254523708f
#define UPPE_SIN_3PI16 0.55557023301960222474f

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

// v * W32^K, W32 = exp(-2 pi i / 32) (K in [0, 16)); conjugated for the inverse transform.
// W32^K = cos(pi K / 16) - i sin(pi K / 16).
template <int K, bool INV>
UPPE_DEV float2 mul_w32(float2 v) {
    if constexpr (K == 0) {
        return v;
    } else if constexpr (K == 8) {
        return INV ? cmul_i(v) : cmul_mi(v);
    } else {
        constexpr float C[16] = {1.f,           UPPE_COS_PI16,  UPPE_COS_PI8,    UPPE_COS_3PI16,
                                 UPPE_SQRT1_2,  UPPE_SIN_3PI16, UPPE_SIN_PI8,    UPPE_SIN_PI16,
                                 0.f,           -UPPE_SIN_PI16, -UPPE_SIN_PI8,   -UPPE_SIN_3PI16,
                                 -UPPE_SQRT1_2, -UPPE_COS_3PI16, -UPPE_COS_PI8,  -UPPE_COS_PI16};
        constexpr float S[16] = {0.f,          UPPE_SIN_PI16, UPPE_SIN_PI8,   UPPE_SIN_3PI16,
                                 UPPE_SQRT1_2, UPPE_COS_3PI16, UPPE_COS_PI8,  UPPE_COS_PI16,
                                 1.f,          UPPE_COS_PI16, UPPE_COS_PI8,   UPPE_COS_3PI16,
                                 UPPE_SQRT1_2, UPPE_SIN_3PI16, UPPE_SIN_PI8,  UPPE_SIN_PI16};
        return cmul(v, make_float2(C[K], INV ? S[K] : -S[K]));
    }
}

// In-register 32-point DFT, natural order in and out: the 16-point DFTs of the even and odd
// samples, combined with the W32 twiddles.
template <int K, bool INV>
UPPE_DEV void dft32_combine(float2 (&v)[32], const float2 (&e)[16], const float2 (&o)[16]) {
    if constexpr (K < 16) {
        const float2 t = mul_w32<K, INV>(o[K]);
        v[K] = cadd(e[K], t);
        v[K + 16] = csub(e[K], t);
        dft32_combine<K + 1, INV>(v, e, o);
    }
}

template <bool INV>
UPPE_DEV void dft32(float2 (&v)[32]) {
    float2 e[16], o[16];
#pragma unroll
    for (int n = 0; n < 16; ++n) {
        e[n] = v[2 * n];
        o[n] = v[2 * n + 1];
    }
    dft16<INV>(e);
    dft16<INV>(o);
    dft32_combine<0, INV>(v, e, o);
}

// DFT of N = 16 or 32 points on N consecutive entries of a register array, starting at OFF.
template <int N, int OFF, bool INV, int L>
UPPE_DEV void dft_at(float2 (&v)[L]) {
    static_assert(N == 16 || N == 32, "register DFT of 16 or 32 points");
    float2 u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) u[i] = v[OFF + i];
    if constexpr (N == 16)
        dft16<INV>(u);
    else
        dft32<INV>(u);
#pragma unroll
    for (int i = 0; i < N; ++i) v[OFF + i] = u[i];
}
