// Launch of the register-resident Cartesian slice vector-Jacobian products (slice_reg.cuh).
#include "slice_reg.cuh"

template <int LN1, int LN2>
struct AdjReg {
    static cudaError_t configure() {
        return cudaFuncSetAttribute(k_adj_reg<LN1, LN2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    RegSlice<LN1, LN2>::SMEM);
    }
    static cudaError_t run(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
        using RS = RegSlice<LN1, LN2>;
        k_adj_reg<LN1, LN2><<<h->N0, RS::T, RS::SMEM, h->stream>>>(mode, in, uppe_op_view(h), out, h->tw, h->twLog,
                                                                   z);
        return cudaGetLastError();
    }
};

template <int LN1, int LN2>
struct AdjFusedReg {
    static cudaError_t configure() {
        return cudaFuncSetAttribute(k_adj_fused_reg<LN1, LN2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    RegSlice<LN1, LN2>::SMEM);
    }
    static cudaError_t run(UppeHandle* h, int mode, const float2* g, float2* out, float a_f, float a_mu, StepArgs z_e,
                           StepArgs z_s) {
        using RS = RegSlice<LN1, LN2>;
        k_adj_fused_reg<LN1, LN2><<<h->N0, RS::T, RS::SMEM, h->stream>>>(mode, g, uppe_op_view(h), h->adj_lf,
                                                                         h->adj_acc, out, a_f, a_mu, h->tw, h->twLog,
                                                                         z_e, z_s);
        return cudaGetLastError();
    }
};

cudaError_t configure_adj_reg() {
    cudaError_t e = cudaSuccess;
#define UPPE_CONF(A_, B_) \
    if (e == cudaSuccess) e = AdjReg<A_, B_>::configure(); \
    if (e == cudaSuccess) e = AdjFusedReg<A_, B_>::configure();
    UPPE_REG_SHAPES(UPPE_CONF)
#undef UPPE_CONF
    return e;
}

cudaError_t launch_adj_reg(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z) {
    return reg_dispatch<AdjReg>(h, mode, in, out, z);
}

cudaError_t launch_adj_fused_reg(UppeHandle* h, int mode, const float2* g, float2* out, float a_f, float a_mu,
                                 StepArgs z_e, StepArgs z_s) {
    return reg_dispatch<AdjFusedReg>(h, mode, g, out, a_f, a_mu, z_e, z_s);
}

bool reg_slice_supported(int N1, int N2) {
    auto ok = [](int n) { return n == 16 || n == 32 || n == 64 || n == 128; };
    return ok(N1) && ok(N2);
}
