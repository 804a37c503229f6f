// RK4 stage update of the spectral amplitude, shared by the Cartesian slice kernels.
#pragma once
#include "common.cuh"
#include "uppe_internal.h"

// ODE right-hand side S = (i/2) exp(-i(kz+kg)z) J / Re kz (uppe.cl:73-91) and the RK4 bookkeeping of
// RKStage/RKFinish (uppe.cl:22-52) with the DC conditioner (uppe_kernel.py:127-137) on the stage
// estimate.  Returns the new stage estimate (qw), or S itself for SPEC_STORE_K.
UPPE_DEV float2 spec_update(int mode, size_t idx, float2 v, const OpPoint& o, float cond,
                                              float2* __restrict__ q_out, float2* __restrict__ qf,
                                              const float2* __restrict__ qi, float Cs, float Ce, const PhaseArgs& pa,
                                              bool store_q) {
    if (mode == SPEC_LOAD) {
        q_out[idx] = v;
        return v;
    }
    const float2 f = propagator_factor(o, pa, -1.f);
    const float2 s = cscale(cmul_i(cmul(f, v)), 0.5f / o.kzr);
    float2 qw;
    switch (mode) {
        case SPEC_STORE_K:
            q_out[idx] = s;
            return s;
        case SPEC_STAGE1: {
            const float2 a = qi[idx];
            qf[idx] = cadd(a, cscale(s, Cs));
            qw = cscale(cadd(a, cscale(s, Ce)), cond);
        } break;
        case SPEC_STAGE23: {
            const float2 a = qi[idx];
            const float2 b = qf[idx];
            qf[idx] = cadd(b, cscale(s, Cs));
            qw = cscale(cadd(a, cscale(s, Ce)), cond);
        } break;
        default: {  // SPEC_FINISH
            const float2 b = qf[idx];
            qw = cscale(cadd(b, cscale(s, Cs)), cond);
        } break;
    }
    if (store_q) q_out[idx] = qw;
    return qw;
}

