// Launch of the register-resident inverse Cartesian slice transform (slice_reg.cuh).
#include "slice_reg.cuh"

template <int LN1, int LN2>
struct RealReg {
    static cudaError_t configure() {
        return cudaFuncSetAttribute(k_real_reg<LN1, LN2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    RegSlice<LN1, LN2>::SMEM);
    }
    static cudaError_t run(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1, float2* qf,
                           float Cs, float Ce, StepArgs z, int iw0, int count) {
        using RS = RegSlice<LN1, LN2>;
        k_real_reg<LN1, LN2><<<count, RS::T, RS::SMEM, h->stream>>>(mode, src, uppe_op_view(h), h->E, A_out, k1, qf,
                                                                    Cs, Ce, h->tw, h->twLog, z, iw0,
                                                                    mode >= REAL_ZS1 ? h->stage_q : nullptr);
        return cudaGetLastError();
    }
};

cudaError_t configure_real_reg() {
    cudaError_t e = cudaSuccess;
#define UPPE_CONF(A_, B_) \
    if (e == cudaSuccess) e = RealReg<A_, B_>::configure();
    UPPE_REG_SHAPES(UPPE_CONF)
#undef UPPE_CONF
    return e;
}

cudaError_t launch_real_reg(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1, float2* qf,
                            float Cs, float Ce, StepArgs z) {
    return reg_dispatch<RealReg>(h, mode, src, A_out, k1, qf, Cs, Ce, z, 0, h->N0);
}

cudaError_t launch_real_reg_range(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1,
                                  float2* qf, float Cs, float Ce, StepArgs z, int iw0, int count) {
    return reg_dispatch<RealReg>(h, mode, src, A_out, k1, qf, Cs, Ce, z, iw0, count);
}
