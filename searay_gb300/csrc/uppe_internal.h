// Internal interfaces between the translation units of libsearay_uppe: the handle and the launch
// wrappers of each kernel family.  Not part of the C ABI (see include/searay_uppe.h).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/searay_uppe.h"

// Modes of the spectral-side kernels.
enum UppeSpecMode {
    SPEC_LOAD = 0,      // initial kspacex of the incoming field: q <- T(a)
    SPEC_STORE_K = 1,   // k1 <- S(J)                               (adaptive first stage)
    SPEC_STAGE1 = 2,    // q <- qi + Ce S ; qf <- qi + Cs S
    SPEC_STAGE23 = 3,   // q <- qi + Ce S ; qf <- qf + Cs S
    SPEC_FINISH = 4,    // qi <- qf + Cs S
};

// Modes of the real-side kernels (inverse transverse transform).
enum UppeRealMode {
    REAL_E = 0,       // E <- T^-1( i kz exp(i(kz+kg)z) q )
    REAL_FINISH = 1,  // A <- T^-1( exp(i(kz+kg)z) q ) and E <- i kz A   (uppe_kernel.py:250-253)
    REAL_APPLY1 = 2,  // first RK stage from k1 (q <- qi + Ce k1, qf <- qi + Cs k1), then E from q
    // an RK stage on a slice without current (S = 0, the NL filter), then E at the next z from the
    // stage estimate: the fused pass's arithmetic there (rk_stage.cuh spec_update with S = 0)
    REAL_ZS1 = 3,     // q <- cond qi, qf <- qi
    REAL_ZS23 = 4,    // q <- cond qi (qf unchanged)
    REAL_ZSF = 5,     // q <- cond qf, written as the step's result
};

// Modes of the time-axis pass.
enum UppeAdjMode {
    ADJ_S = 0,     // cotangent of S -> cotangent of J (before the forward transverse transform)
    ADJ_LOAD = 1,  // transpose of the load transform
    ADJ_E = 2,     // cotangent of E -> cotangent of q
    ADJ_FIN = 3,   // cotangent of the finish A -> cotangent of q
};

enum UppeTimeMode {
    TIME_J = 0,       // J(w) from E(w): Kerr + plasma current, NL filter
    TIME_CHI_NE = 1,  // rfft of chi(t) and ne(t) (diagnostic outputs of finish)
};

struct StepArgs {
    float zhi, zlo;
    int plain;
};

struct UppeHandle {
    UppeConfig cfg;
    int N0, N1, N2, Nk, Nt, M, S;  // S = N1*N2 transverse points
    size_t P;                      // N0*N1*N2
    int twLog;                     // twiddle table size 2^twLog
    int time_cols;                 // transverse points per CTA in the time pass
    int time_spt;                  // time samples per thread in the time pass (16 or 32)
    int num_sms;                   // multiprocessors of the device
    int smem_per_sm;               // shared memory per multiprocessor (bytes)
    int slice_reg;                 // Cartesian slices use the register-resident transforms (slice_reg.cuh)
    int slice_big;                 // Cartesian slices above 128 x 128: row and column passes (slice_big.cu)
    int time_reg;                  // TIME_J through the register-resident time pass where it applies (timepass_reg.cu)
    int slice_cluster;             // 256 x 256 slices: the fused tail in one cluster launch (slice_cluster.cu)
    int tc_next;                   // tensor-core Hankel: stage updates write the next inverse transform's operand
    cudaStream_t stream;
    // library-owned device buffers
    float2 *q, *qi, *qf, *k1, *E, *J, *scratch;
    float2* opK;     // [P] K = Re kz + kg as float-float
    float* opKi;     // [P] Im kz (read only when complex_medium)
    float2* kg2;     // [N0] kg as float-float
    int complex_medium;
    float* ng;
    float2* tw;
    float2* tw_reg;  // twiddle tables of the register-resident time pass (timepass_reg.cu), or NULL
    float2* tscr;    // its parking scratch for ionizing columns ([S][2 (M + 1)]), or NULL
    int* adj_live;   // register-resident adjoint time pass: count + column groups left to k_time_adj, or NULL
    float2* adj_park; // its parking scratch for e(t) ([S][M]) when tscr is NULL, or NULL
    float* w;        // omega per bin (FP32)
    float* nlfilt;   // NL filter per bin
    float* Minv;     // cylindrical: [N2][Nr][Nk]
    float* Mfwd;     // cylindrical: [N2][Nr][Nr] (rows >= Nk zero)
    uint8_t* Minv_tc; // the same, split into bf16 hi/lo tensor-core tiles (mixed form)
    uint8_t* Mfwd_tc;
    uint8_t* MfwdT_tc; // the transposed matrices of the adjoint transforms, split the same way
    uint8_t* MinvT_tc;
    uint8_t* Atc;     // pre-split A operand tiles of the tensor-core Hankel transform (mixed form)
    size_t Atc_bytes;
    int time_atc;                // the next TIME_J pass writes J into Atc (the forward transform's operand)
    int atc_fwd;                 // Atc holds the operand of the transform `atc_fwd_which` (0: forward of J,
    int atc_fwd_which;           // 3: the adjoint's Minv^T of gE) of atc_fwd_src, written by a time pass
    const void* atc_fwd_src;
    int atc_next;                // Atc holds the operand of the inverse transform of atc_next_src at atc_next_z
    const void* atc_next_src;
    StepArgs atc_next_z;
    long long atc_next_mat;      // the material version the tiles were formed with
    double* kr2_d;   // [S] transverse eigenvalues (FP64)
    double* w2n2_d;  // [N0] complex w^2 (1 + chi0) interleaved
    double* kg_d;    // [N0]
    float* red;      // reduction scalars: [0] max|q|, [1] min dz, [2] nonfinite flag
    int* dev_err;    // set by a kernel whose bounded wait expired
    int have_grid, have_material, have_field;
    double max_abs_K;   // max |Re kz + kg| of the current operator
    double max_Ki;      // max Im kz of the current operator
    double redchi3;        // chi3 / density reference in use (uppe_set_chi3)
    int rot_pairs;         // rotational Raman transitions in use (uppe_set_rotator), in pairs; 0 = none
    float* rot;            // their tables: [rot_pairs][80] then the phasors [rot_pairs][Nt/16] (float4)
    // adjoint work buffers (allocated by the first adjoint call)
    float2 *adj_q1, *adj_q2, *adj_q3, *adj_lf, *adj_acc, *adj_lk, *adj_mu;
    float2* adj_E[4];      // E of the recomputed stage states q0, q1', q2', q3' (reused by the reverse sweep)
    float2* stage_q;       // when set, the Cartesian fused pass also stores each stage estimate here
    int kept_valid;        // adj_E[0..3] hold the stage fields of the step taken by uppe_rk4_step_keep
    double kept_z, kept_dz;
    long long kept_mat;
    float* MfwdT;          // cylindrical adjoint: [Nr][Nr], MfwdT[r][k] = Mfwd[k][r]
    float* MinvT;          // [Nr][Nr], MinvT[k][r] = Minv[r][k] for k < Nk, 0 beyond
    double* dred_d;        // device accumulator of d(loss)/d(chi3/nref)
    long long mat_version; // incremented by every uppe_set_material
    int E_valid;           // E holds T^-1(i kz e^{..} qi) for (E_z, E_mat): reusable by the next step
    double E_z;
    long long E_mat;
    long long launches; // kernels launched by this handle
    void* prof;         // profiling state (capi.cu), NULL when off
    char err[512];
};

int uppe_set_error(UppeHandle* h, const char* fmt, ...);

struct OpView;
OpView uppe_op_view(const UppeHandle* h);

// ---- kernel launch wrappers (uppe_kernels.cu) ----
cudaError_t launch_build_operator(UppeHandle* h);
cudaError_t launch_operator_bounds(UppeHandle* h);  // red[0] = max |K|, red[1] = max Im kz
cudaError_t uppe_configure_slice_kernels(size_t smem_bytes);
cudaError_t uppe_configure_time_kernel(size_t smem_bytes);
cudaError_t launch_real_cart(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z);
cudaError_t launch_spec_cart(UppeHandle* h, int mode, const float2* src_real, float2* q_out, float2* qf_io,
                             const float2* qi, float Cs, float Ce, StepArgs z);
// Cartesian fused pass: forward FFT of J, RHS, RK stage (SPEC_STAGE1/STAGE23/FINISH), then E at
// z_next from the new stage estimate; writes qf / qi as the stage requires and E.
// zs_current: the slices without current (w >= nl_cut_off) already hold this stage's q and E (stage 2,
// whose E is at the same z as stage 1's, and the finish, whose E is at the same z as stage 3's)
cudaError_t launch_fused_cart(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                              bool zs_current = false);
// Cartesian first stage from k1 (adaptive step) fused with the inverse transform to E.
cudaError_t launch_apply1_cart(UppeHandle* h, float Cs, float Ce, StepArgs z);
cudaError_t launch_time_pass(UppeHandle* h, int mode, const float2* E, float2* out0, float2* out1);
// register-resident time pass (timepass_reg.cu): TIME_J for M = 256, 512, 1024 without a rotator
bool time_reg_supported(const UppeHandle* h);
size_t time_reg_table_len(int M);
int time_reg_tables(int M, float2* host);
size_t time_reg_scratch_len(const UppeHandle* h);
cudaError_t uppe_configure_time_reg();
cudaError_t launch_time_reg(UppeHandle* h, const float2* E, float2* J);
// register-resident adjoint time pass (timepass_adj_reg.cu): the columns without ionization
int time_adj_reg_group(int M);
size_t time_adj_reg_list_len(const UppeHandle* h);
bool time_adj_reg_ready(const UppeHandle* h);
cudaError_t uppe_configure_time_adj_reg();
cudaError_t launch_time_adj_reg(UppeHandle* h, const float2* E, const float2* G, float2* gE, double* dred);
// paraxial envelope time pass (envelope.cu)
cudaError_t launch_time_env(UppeHandle* h, int mode, const float2* A, float2* out0, float2* out1);
cudaError_t uppe_configure_env_kernel(size_t smem_bytes);
size_t uppe_env_smem_bytes(const UppeHandle* h);
cudaError_t launch_absmax(UppeHandle* h, const float2* q);
cudaError_t launch_step_size(UppeHandle* h, const float2* q, const float2* k, double L, double dphi, double rel_amin);
cudaError_t launch_apply_stage1(UppeHandle* h, float Cs, float Ce);
cudaError_t launch_ikz(UppeHandle* h, const float2* A, float2* E);

cudaError_t launch_adj_cart(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z);

// ---- register-resident Cartesian slice kernels (slice_reg_*.cu), N1, N2 in {16, 32, 64, 128} ----
bool reg_slice_supported(int N1, int N2);
cudaError_t configure_fused_reg();
cudaError_t configure_real_reg();
cudaError_t configure_spec_reg();
cudaError_t configure_adj_reg();
cudaError_t launch_fused_reg(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                             int nslices);
// k_real_reg over the slices [iw0, iw0 + count)
cudaError_t launch_real_reg_range(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1,
                                  float2* qf, float Cs, float Ce, StepArgs z, int iw0, int count);
cudaError_t launch_real_reg(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1, float2* qf,
                            float Cs, float Ce, StepArgs z);
cudaError_t launch_spec_reg(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                            float Cs, float Ce, StepArgs z);
cudaError_t launch_adj_reg(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z);
cudaError_t launch_adj_fused_reg(UppeHandle* h, int mode, const float2* g, float2* out, float a_f, float a_mu,
                                 StepArgs z_e, StepArgs z_s);
cudaError_t launch_spec_point(UppeHandle* h, int mode, const float2* C, float2* q_out, float2* qf, const float2* qi,
                              float Cs, float Ce, StepArgs z, const StepArgs* z_next);
struct TcNext;
TcNext hankel_tc_next(const UppeHandle* h, StepArgs z_next);
cudaError_t launch_adj_fused_big(UppeHandle* h, int mode, const float2* g, float2* out, float a_f, float a_mu,
                                 StepArgs z_e, StepArgs z_s);

// ---- Cartesian slices of 128 x 256, 256 x 128, 256 x 256 (slice_big.cu): row + column passes ----
bool big_slice_supported(int N1, int N2);
struct BigColArgs;
// the fused tail of 256 x 256 slices in one launch (a cluster of 8 CTAs per slice); returns
// cudaErrorNotSupported where the cluster form cannot run
bool cluster_slice_supported(int N1, int N2);
cudaError_t launch_fused_cluster(UppeHandle* h, const BigColArgs& a, int nfwd, int nall);
cudaError_t launch_fused_big(UppeHandle* h, int mode, float Cs, float Ce, StepArgs z_rhs, StepArgs z_next,
                             bool zs_current = false);
cudaError_t launch_real_big(UppeHandle* h, int mode, const float2* src, float2* A_out, const float2* k1, float2* qf,
                            float Cs, float Ce, StepArgs z);
cudaError_t launch_spec_big(UppeHandle* h, int mode, const float2* src, float2* q_out, float2* qf, const float2* qi,
                            float Cs, float Ce, StepArgs z);
cudaError_t launch_adj_big(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z);
cudaError_t launch_adj_rk(UppeHandle* h, int mode, const float2* lam_out, float2* lam_in, float a_f, float a_mu);
cudaError_t launch_time_adjoint(UppeHandle* h, const float2* E, const float2* G, float2* gE, double* dred);
cudaError_t uppe_configure_time_adj_kernel(size_t smem_bytes);
cudaError_t launch_adj_cyl(UppeHandle* h, int mode, const float2* in, float2* out, StepArgs z);

// ---- cylindrical transverse transform (hankel.cu) ----
cudaError_t launch_real_cyl(UppeHandle* h, int mode, const float2* src, float2* A_out, StepArgs z);
cudaError_t launch_spec_cyl(UppeHandle* h, int mode, const float2* src_real, float2* q_out, float2* qf_io,
                            const float2* qi, float Cs, float Ce, StepArgs z, const StepArgs* z_next = nullptr);
