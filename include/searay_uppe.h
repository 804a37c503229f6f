/*
 * searay_uppe.h - C ABI of the GB300 (sm_103a) UPPE z-step library, libsearay_uppe.so.
 *
 * The library is a drop-in for the device side of SeaRay's unidirectional pulse propagation
 * (UPPE) path: modules/uppe_kernel.py (Material, Source, load_source, update_current, propagator,
 * finish) together with the OpenCL kernels it enqueues (kernels/uppe.cl, kernels/fft.cl,
 * kernels/ionization.cl, kernels/paraxial.cl:27-58).  The host side that parses the volume input
 * dictionary (uppe_kernel.track) stays in Python (searay_gb300/uppe.py) and calls these entry
 * points with plain pointers and sizes.
 *
 * Conventions
 *   - Every call returns an int status: 0 on success, a negative UPPE_E* code on error.  Nothing
 *     traps; uppe_last_error() gives the message of the last failure on a handle.
 *   - Field arrays are complex64 (interleaved float pairs) in the reference layout [w][x|r][y|phi],
 *     C order, N0 x N1 x N2 elements, and live in device memory owned by the caller.  Host-side
 *     tables (frequencies, eigenvalues, Hankel basis, material) are FP64 host arrays, copied in.
 *   - Work buffers are owned by the handle.  All work of a handle is issued on its stream, in
 *     order.  A handle is not thread-safe; distinct handles are independent.
 */
#ifndef SEARAY_UPPE_H
#define SEARAY_UPPE_H

#ifdef __cplusplus
extern "C" {
#endif

#define UPPE_OK 0
#define UPPE_E_ARG (-1)      /* invalid argument, shape or state */
#define UPPE_E_CUDA (-2)     /* a CUDA runtime call failed */
#define UPPE_E_NOMEM (-3)    /* device allocation failed */
#define UPPE_E_RANGE (-4)    /* a value lies outside what the mixed-precision path represents */
#define UPPE_E_NONFINITE (-5) /* the field holds NaN or Inf */

/* Precision forms. */
#define UPPE_PREC_MIXED 0 /* FP32 transforms/sources; float-float phase and density scan */
#define UPPE_PREC_FP32 1  /* everything in FP32, including phase and density scan */

/* Ionization rate forms (kernels/ionization.cl). */
#define UPPE_RATE_NONE 0
#define UPPE_RATE_EXPLICIT 1 /* ExplicitRate, ionization.cl:22-44 */
#define UPPE_RATE_SERIES 2   /* ExplicitRateSeries, ionization.cl:71-97 */

typedef struct UppeConfig {
    int n0;            /* frequency nodes, 2^n + 1 (uppe_kernel.py:354-356) */
    int n1;            /* x nodes (Cartesian) or radial nodes (cylindrical), 2^n */
    int n2;            /* y nodes (Cartesian) or azimuthal nodes (cylindrical), 2^n */
    int radial_modes;  /* Nk <= n1 for cylindrical (grid_tools.py:254-258); ignored for Cartesian */
    int cylindrical;   /* 0: FourierTransformTool, 1: HankelTransformTool */
    int precision;     /* UPPE_PREC_* */
    double dt;         /* pi / max(w)  (uppe_kernel.py:96) */
    double chi3_over_nref; /* chi3 / density reference (uppe_kernel.py:52) */
    int nl_cut_on;     /* int(NL_band[0]/dw) (uppe_kernel.py:122) */
    int nl_cut_off;    /* int(NL_band[1]/dw) (uppe_kernel.py:123) */
    int rate_form;     /* UPPE_RATE_* */
    double field_conv; /* field_sim_to_au(1) (ionization.py:132) */
    double rate_conv;  /* rate_au_to_sim(1) (ionization.py:133) */
    double field_cutoff; /* 1e-3 a.u. (ionization.py:102) */
    double c_pre, c_pow, c_exp; /* explicit form coefficients */
    double clog[6];    /* series form coefficients */
    double damping;    /* iDtSpectral damping, 0.1 (uppe_kernel.py:171) */
    int window_cutoff; /* SoftTimeWindow cutoff, 4 (uppe_kernel.py:168) */
    int window_width;  /* SoftTimeWindow width, 64 */
    int envelope;      /* 0: UPPE (uppe_kernel.py); 1: paraxial envelope solver (paraxial_kernel.py):
                        * n0 = 2^n absolute frequencies in FFT order (np.fft.ifftshift of the band),
                        * dt = 2 pi / bandwidth (paraxial_kernel.py:98-103), uppe_set_material takes the
                        * envelope tables, no DC conditioner, NL filter or soft time window; Cartesian
                        * slices up to 128 x 128; no adjoint */
} UppeConfig;

typedef struct UppeHandle UppeHandle;

/* Allocate a propagator for one grid.  Replaces the buffer set-up of Source.__init__
 * (uppe_kernel.py:95-129), Material.__init__ (:35-66) and TransverseModeTool.AllocateDeviceMemory
 * (grid_tools.py:299-303).  The whole configuration is checked on the host before any CUDA call
 * (UPPE_E_ARG, with the reference's ValueError wording for grids, uppe_kernel.py:354-360); then
 * UPPE_E_NOMEM when device memory runs out, UPPE_E_CUDA for any other CUDA failure (no device, no
 * driver).  *out is NULL on every error; uppe_last_error(NULL) holds the message. */
int uppe_create(const UppeConfig* cfg, UppeHandle** out);

/* Release a handle and its device buffers (grid_tools.py:304-307). */
int uppe_destroy(UppeHandle* h);

/* Issue the handle's work on this CUDA stream (cudaStream_t; NULL = legacy default stream). */
int uppe_set_stream(UppeHandle* h, void* stream);

/* Grid tables, once per handle.  w: N0 frequencies (caustic_tools.py:88-96); kr2: the transverse
 * eigenvalues, N1*N2 values (Cartesian FD k^2, grid_tools.py:245-250, or -vals of the Hankel
 * basis, grid_tools.py:357-358); H: Hankel basis (Nk, Nr, N2) and Lambda (Nr) for cylindrical
 * grids (grid_tools.py:252-294), NULL for Cartesian.  Replaces the H/L uploads of
 * HankelTransformTool.AllocateDeviceMemory (grid_tools.py:299-303). */
int uppe_set_grid(UppeHandle* h, const double* w, const double* kr2, const double* H, const double* Lambda);

/* Material at the current subcycle.  w2n2: N0 complex values w^2 (1 + chi0(w)) as interleaved
 * doubles; kg: N0 values -w/v_window; ng: N1*N2 gas densities n_ref*dens.  Builds kz on the device
 * with the reference's guards (Im kz >= 0; Re kz == 0 -> 1).  Replaces Material.UpdateMaterial's
 * kz/kg/ng uploads (uppe_kernel.py:67-90). */
int uppe_set_material(UppeHandle* h, const double* w2n2, const double* kg, const double* ng);
/* With cfg.envelope = 1 the same call takes the paraxial Material.UpdateMaterial tables
 * (paraxial_kernel.py:67-91), in FFT order: w2n2 = f(w) = w^2 (1 + chi0 - ng^2) - w0^2 dn^2 - 2 w w0 ng dn
 * (complex, interleaved), kg = k0(w) = w0 dn + w ng, ng = the gas density plane; the operator is
 * kz = (f(w) - kperp^2) / (2 k0(w)) and the right-hand side divides by k0(w). */

/* Load the incoming field a (device, real space, complex64) and transform it to the transverse
 * spectral representation q.  Replaces Source(...) + T.kspacex(qw) (uppe_kernel.py:290-291). */
int uppe_load_field(UppeHandle* h, const void* a);

/* One classic RK4 step of the interaction-picture amplitude (uppe_kernel.py:304-325 body).
 * z_phase: local coordinate of the step start used in the propagator phase (z0 - zi + z);
 * L: subcycle length; z_sub: position of the step inside the subcycle; dzmin: minimum step.
 * The adaptive estimate (paraxial.cl:27-58, uppe_kernel.py:217-232) runs only when dzmin < L - z_sub;
 * otherwise dz = L - z_sub.  *dz_out receives the step taken. */
int uppe_rk4_step(UppeHandle* h, double z_phase, double L, double z_sub, double dzmin, double* dz_out);

/* Final phase to z_phase, inverse transverse transform and source diagnostics (uppe_kernel.py:234-258).
 * Device outputs, complex64 [N0][N1][N2]: A (real-space vector potential), J (real-space current),
 * chi_w = rfft_t(chi), ne_w = rfft_t(ne).  Any output may be NULL. */
int uppe_finish(UppeHandle* h, double z_phase, void* A, void* J, void* chi_w, void* ne_w);

/* One right-hand-side evaluation S(q, z) = load_source (uppe_kernel.py:188-216), for tests:
 * q_in and S_out are device complex64 [N0][N1][N2] in the transverse spectral representation. */
int uppe_eval_rhs(UppeHandle* h, const void* q_in, double z_phase, void* S_out);

/* Copy the current spectral amplitude q to a device buffer (complex64 [N0][N1][N2]). */
int uppe_get_field(UppeHandle* h, void* q_out);

/* Set *nonfinite to 1 if the current q holds NaN or Inf (the '!' check of uppe_kernel.py:219-220). */
int uppe_check_finite(UppeHandle* h, int* nonfinite);

/* ---- adjoint (vector-Jacobian products), for gradients through torch.autograd ----
 * The reference has no adjoint; these entry points give the transposed linearisation of the maps
 * above so that gradients of a loss on the outputs reach the incoming field and chi3 (n2).
 * Cotangents are complex64 device arrays [N0][N1][N2] in the real-pair convention
 * g = dL/dRe + i dL/dIm.  Cylindrical grids need one azimuthal node. */

/* Replace chi3 / density reference (the Kerr coefficient, uppe_kernel.py:52) used from now on. */
int uppe_set_chi3(UppeHandle* h, double chi3_over_nref);

/* Rotational Raman response (SeaRay's 'rotator', rotations.py:13-73, added to chi before the Kerr
 * term as uppe_kernel.py:173-179 does, by AddChiUPPE, rotations.cl:85-129).  Host arrays of a
 * Rotator's tables, nstates entries: Tj (population differences T_j) and Wj (complex transition
 * frequencies W_j interleaved as re, im), with its dalpha and hbar; transitions j -> j-2 for
 * j >= 2.  nstates = 0 removes the response.  The adjoint entry points include it (the transpose
 * of the Raman map in the adjoint time pass). */
int uppe_set_rotator(UppeHandle* h, int nstates, const double* Tj, const double* Wj, double dalpha, double hbar);

/* Set the spectral amplitude q directly (a checkpoint restart), device complex64 [N0][N1][N2]. */
int uppe_set_field(UppeHandle* h, const void* q);

/* VJP of one fixed RK4 step q0 -> q1 at z_phase with step dz (the body of uppe_kernel.py:305-325
 * with dz fixed): lam_in = (dq1/dq0)^H lam_out.  Recomputes the stage estimates from q0.  Adds
 * d(loss)/d(chi3/nref) of this step to *dred (may be NULL).  Overwrites the handle's q. */
int uppe_adjoint_rk4_step(UppeHandle* h, const void* q0, const void* lam_out, void* lam_in, double z_phase,
                          double dz, double* dred);

/* One fixed RK4 step of the held field (the step of uppe_rk4_step with dzmin = L - z_sub = dz) that
 * keeps what the reverse sweep reads (the E of its four stage states, and with separate transverse
 * passes the stage estimates) for uppe_adjoint_rk4_step_kept.  The grids the adjoint supports;
 * UPPE_E_ARG otherwise.  Allocates the adjoint buffers on first use. */
int uppe_rk4_step_keep(UppeHandle* h, double z_phase, double dz);

/* VJP of the step last taken by uppe_rk4_step_keep: lam_in = (dq1/dq0)^H lam_out, without the
 * recompute of uppe_adjoint_rk4_step.  UPPE_E_ARG when no such step is kept for the current
 * material (uppe_rk4_step, uppe_adjoint_rk4_step and uppe_set_material end it).  Adds
 * d(loss)/d(chi3/nref) to *dred (may be NULL). */
int uppe_adjoint_rk4_step_kept(UppeHandle* h, const void* lam_out, void* lam_in, double* dred);

/* VJP of uppe_load_field (q = T a): lam_a = T^H lam_q. */
int uppe_adjoint_load(UppeHandle* h, const void* lam_q, void* lam_a);

/* VJP of the field output of uppe_finish (A = T^-1 exp(i(kz+kg)z) q): lam_q from lam_A. */
int uppe_adjoint_finish(UppeHandle* h, double z_phase, const void* lam_A, void* lam_q);

/* Timing classes of the kernels, for uppe_profile_read. */
#define UPPE_NCLASS 6
#define UPPE_CLASS_OPERATOR 0   /* kz build (UpdateMaterial) */
#define UPPE_CLASS_TRANSVERSE_INV 1 /* propagator phase + i kz + inverse transverse transform */
#define UPPE_CLASS_TIME 2       /* time-axis pass: irfft, sources, density scan, rfft */
#define UPPE_CLASS_TRANSVERSE_FWD 3 /* forward transverse transform + ODE RHS + RK4 stage */
#define UPPE_CLASS_STEP_SIZE 4  /* adaptive step estimate */
#define UPPE_CLASS_OTHER 5

/* Record CUDA events on the handle's stream around every kernel class (enable=1), or stop
 * (enable=0).  Enabling clears the accumulated times.  Adds event records between launches, so
 * time headline numbers with profiling off.  (SeaRay has only a wall-clock print, rays.py:85,136.) */
int uppe_profile_enable(UppeHandle* h, int enable);

/* Synchronise the stream and return, per class, the summed milliseconds and the number of timed
 * regions since profiling was enabled (arrays of UPPE_NCLASS entries). */
int uppe_profile_read(UppeHandle* h, double* ms, long long* count);

/* Number of kernels this handle has launched since it was created. */
int uppe_launch_count(UppeHandle* h, long long* n);

/* Name of a timing class. */
const char* uppe_class_name(int cls);

/* Adaptive step-size estimate without any device allocation.  This entry point has no
 * counterpart in the reference; it exists for callers that may not allocate device memory once
 * they run.  Examples: a host program that reserves all GPU memory at start-up and forbids later
 * cudaMalloc, or a loop in which an allocation would synchronise the device.  Such a caller cannot
 * create a handle, which allocates its work buffers.
 *
 * From q and S = dq/dz (device complex64 arrays of n points, caller-owned) it writes to *dz_out
 * (one float in device memory) the unclamped estimate min over the grid of dphi / K, computed as in
 * uppe_rk4_step's adaptive step: amin = rel_amin * max|q|, K = 0.5 dphi/L + |Im(S q*)|/(|q|^2 +
 * amin^2) - min(Re(S q*)/(|q|^2 + amin^2), 0)  (paraxial.cl:40-58, uppe_kernel.py:217-223).  The
 * caller applies the dzmin and end-of-subcycle clamps.
 *
 * If q or S holds a non-finite value, *dz_out is NaN.
 *
 * Its reduction scratch is one fixed array in device memory, about 128 KB.  Limits and rules:
 *   - n may not exceed UPPE_NOALLOC_MAX_POINTS; larger grids get UPPE_E_RANGE and a message.
 *   - The first call on each device, made with that device current, loads this entry point's
 *     CUDA module onto the device (the runtime loads modules lazily by default), looks up the
 *     array's device address and loads its kernels.  That first call is the only one that may
 *     allocate device memory (the array and the kernels' code).  Make it before the caller's
 *     no-allocation phase begins (for example before reserving all remaining device memory) and
 *     before any CUDA stream capture.  From then on the array stays on that device until the
 *     process exits.
 *   - Only the device's primary context (the one the CUDA runtime API uses) is supported, and the
 *     entry point must not be used across a cudaDeviceReset: the address looked up in the first
 *     call is kept for the life of the process.
 *   - All calls share the one array, which keeps the contents of the last call.  Calls whose work
 *     overlaps on the GPU (for example on two streams at once) race; serialise them.
 * Work is issued on `stream` (cudaStream_t, NULL = legacy default stream).  Errors are reported by
 * uppe_last_error(NULL). */
#define UPPE_NOALLOC_MAX_POINTS (1LL << 27)
int uppe_step_size_noalloc(const void* q, const void* S, long long n, double L, double dphi, double rel_amin,
                           void* dz_out, void* stream);

/* Message of the last error on h (or of the last failed uppe_create when h is NULL). */
const char* uppe_last_error(const UppeHandle* h);

#ifdef __cplusplus
}
#endif

#endif /* SEARAY_UPPE_H */
