// Launch of the register-resident forward Cartesian slice transform and spectral update (slice_reg.cuh).
#include "slice_reg.cuh"

template <int LN1, int LN2>
struct SpecReg {
    static cudaError_t configure() {
        return cudaFuncSetAttribute(k_spec_reg<LN1, LN2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    RegSlice<LN1, LN2>::SMEM);
    }
    static cudaError_t run(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                           float Cs, float Ce, StepArgs z) {
        using RS = RegSlice<LN1, LN2>;
        k_spec_reg<LN1, LN2><<<h->N0, RS::T, RS::SMEM, h->stream>>>(mode, src, uppe_op_view(h), q_out, qf, qi, Cs, Ce,
                                                                    h->tw, h->twLog, z);
        return cudaGetLastError();
    }
};

cudaError_t configure_spec_reg() {
    cudaError_t e = cudaSuccess;
#define UPPE_CONF(A_, B_) \
    if (e == cudaSuccess) e = SpecReg<A_, B_>::configure();
    UPPE_REG_SHAPES(UPPE_CONF)
#undef UPPE_CONF
    return e;
}

cudaError_t launch_spec_reg(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                            float Cs, float Ce, StepArgs z) {
    return reg_dispatch<SpecReg>(h, mode, src, q_out, qf, qi, Cs, Ce, z);
}
