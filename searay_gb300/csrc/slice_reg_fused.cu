// Launch of the register-resident fused Cartesian evaluation tail (slice_reg.cuh).
#include "slice_reg.cuh"

template <int LN1, int LN2>
struct FusedReg {
    static cudaError_t configure() {
        return cudaFuncSetAttribute(k_fused_reg<LN1, LN2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    FusedPlan<LN1, LN2>::SMEM);
    }
    static cudaError_t run(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next, int n) {
        using RS = RegSlice<LN1, LN2>;
        const int grid = n < h->num_sms ? n : h->num_sms;  // persistent: one CTA per multiprocessor
        k_fused_reg<LN1, LN2><<<grid, RS::T, FusedPlan<LN1, LN2>::SMEM, h->stream>>>(
            mode, h->J, uppe_op_view(h), h->qi, h->qf, h->qi, h->E, Cs, Ce, h->tw, h->twLog, z_rhs, z_next, n,
            h->stage_q);
        return cudaGetLastError();
    }
};

cudaError_t configure_fused_reg() {
    cudaError_t e = cudaSuccess;
#define UPPE_CONF(A_, B_) \
    if (e == cudaSuccess) e = FusedReg<A_, B_>::configure();
    UPPE_REG_SHAPES(UPPE_CONF)
#undef UPPE_CONF
    return e;
}

// The fused pass over the slices [0, nslices).
cudaError_t launch_fused_reg(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                             int nslices) {
    return reg_dispatch<FusedReg>(h, mode, Cs, Ce, z_rhs, z_next, nslices);
}
