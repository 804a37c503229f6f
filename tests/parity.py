"""Error metrics and tolerances shared by the GPU parity tests.

Every comparison is against an FP64 target on the same inputs: the golden fixtures made by running
SeaRay's own UPPE path (tests/golden/make_golden.py), or the FP64 oracle.

Metrics (each relative to the target's maximum, so that tiny values far from the pulse do not
dominate):
  * rel_err: max |x - x_ref| / max |x_ref| over an array;
  * fluence: F(x, y) = sum over w of |A|^2, one value per transverse point (and diagnostic plane);
    the error is max |F - F_ref| / max F_ref;
  * spectrum: P(w) = sum over the transverse points of |A|^2 (per diagnostic plane); the error is
    max |P - P_ref| / max P_ref.

Field tolerances (the bounds stated for the two precision forms):
  * 1e-5 wherever the transverse transforms run in FP32: every Cartesian grid (both forms: the
    mixed form differs only in its float-float phase and density sum) and cylindrical grids in the
    plain FP32 form;
  * 1e-4 for the mixed form's split-BF16x3 tensor-core Hankel transforms (about 1e-5 relative per
    transform).
Fluence and spectrum are held to the same bounds as the field.  Diagnostics that pass through the
exponentially stiff ionization rate (J, chi, n_e) are held to 1e-4."""
import numpy as np

FIELD_TOL = {"fp32": 1e-5, "tensor": 1e-4}
DIAG_TOL = 1e-4


def rel_err(x, ref):
    x = np.asarray(x)
    ref = np.asarray(ref)
    s = np.max(np.abs(ref))
    return float(np.max(np.abs(x - ref)) / s) if s > 0 else float(np.max(np.abs(x)))


def fluence(A):
    """Sum over w (axis 0) of |A|^2: one value per transverse point (and plane, if any)."""
    A = np.asarray(A)
    return np.sum(A.real.astype(np.float64) ** 2 + A.imag.astype(np.float64) ** 2, axis=0)


def spectrum(A):
    """Sum over the transverse axes (1, 2) of |A|^2: one value per w (and plane, if any)."""
    A = np.asarray(A)
    return np.sum(A.real.astype(np.float64) ** 2 + A.imag.astype(np.float64) ** 2, axis=(1, 2))


def field_errors(A, A_ref):
    """{"A": field error, "fluence": ..., "spectrum": ...} of A against A_ref."""
    return {"A": rel_err(A, A_ref), "fluence": rel_err(fluence(A), fluence(A_ref)),
            "spectrum": rel_err(spectrum(A), spectrum(A_ref))}


def field_tol(tensor_core):
    return FIELD_TOL["tensor" if tensor_core else "fp32"]


def check_field(errs, tensor_core):
    """Assert the field, fluence and spectrum errors in ``errs`` against the form's bound."""
    tol = field_tol(tensor_core)
    for key in ("A", "fluence", "spectrum"):
        if key in errs:
            assert errs[key] < tol, (key, errs[key], tol)


def fmt(errs):
    return {k: f"{v:.2e}" for k, v in errs.items()}
