"""Parity at the full sizes of the benchmark workloads, on the device against the FP64 oracle on the
same grid, in both precision forms:

* one fixed RK4 step from the incoming plane, with the finish (A, J, chi, n_e):
  - cart_filament_128: 513 x 128 x 128 Cartesian, Kerr + O2 tunneling + plasma current
    (register-resident slices, the zero-current slices split off);
  - cart_filament_256: 1025 x 256 x 256 Cartesian, the large filament (row and column passes of
    the big-slice kernels); the oracle step takes most of a minute on the host cores;
  - cyl_silica_512: 2049 x 512 cylindrical, fused silica with ionization (the tensor-core Hankel
    transforms in the mixed form, the SIMT ones in the plain FP32 form);
* twenty consecutive fixed RK4 steps of cart_filament_128 with the electron density non-zero
  throughout: the float-float (mixed) or FP32 (plain) phase and density sums carried through the
  stiff rate over 80 right-hand-side evaluations.

Metrics and bounds of tests/parity.py: field, fluence and spectrum within 1e-5 with FP32
transverse transforms and 1e-4 with the tensor-core transforms; J, chi, n_e within 1e-4.  Each
test prints its measured errors."""
import numpy as np
import pytest

from parity import DIAG_TOL, check_field, field_errors, fmt, rel_err

pytestmark = pytest.mark.gpu

_ORACLE = {}


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()


def _oracle(workload, steps):
    """(vd, a, dz, oracle outputs after ``steps`` fixed steps), cached for both precision forms."""
    key = (workload, steps)
    if key not in _ORACLE:
        _ORACLE.clear()  # one full-size result held at a time
        from oracle import uppe_oracle as O
        from searay_gb300 import grid, workloads
        vd = workloads.WORKLOADS[workload]()
        g = grid.VolumeGrid(vd)
        dz = vd["size"][2] / vd["subcycles"]
        a = vd["incoming wave"](g.w, g.x1, g.x2)
        A, J, chi, ne, n = O.Oracle(vd).propagator(a, 0.0, steps * dz, steps, dz)
        assert n == steps
        _ORACLE[key] = (vd, a, dz, (A, J, chi, ne))
    return _ORACLE[key]


def _device_run(workload, steps, precision):
    import torch
    from searay_gb300 import grid, ionization, uppe
    vd, a, dz, ref = _oracle(workload, steps)
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") is not None else None
    dev = uppe.DeviceGrid(g, vd, rates, precision)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd["chi3"], vd["density reference"],
                        vd["window speed"], vd["density lambda"])
    A, J, chi_w, ne, evals = uppe.propagator(dev, mat, torch.from_numpy(a.astype(np.complex64)).cuda(), steps, 0.0,
                                             steps * dz, dz)
    assert evals == 4 * steps
    assert not dev.nonfinite()
    out = tuple(t.cpu().numpy() for t in (A, J, chi_w, ne))
    dev.close()
    A_ref, J_ref, chi_ref, ne_ref = ref
    errs = field_errors(out[0], A_ref)
    errs.update({"J": rel_err(out[1], J_ref), "chi": rel_err(out[2], chi_ref), "ne": rel_err(out[3], ne_ref)})
    assert np.max(np.abs(ne_ref)) > 0
    return vd, errs


def _check(vd, errs, precision):
    tensor = vd["wave coordinates"] != "cartesian" and precision == "mixed"
    check_field(errs, tensor)
    for key in ("J", "chi", "ne"):
        assert errs[key] < DIAG_TOL, (key, errs[key])


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("workload", ["cart_filament_128", "cart_filament_256", "cyl_silica_512"])
def test_benchmark_workload_step_vs_oracle(workload, precision):
    vd, errs = _device_run(workload, 1, precision)
    print(workload, precision, "one step", fmt(errs))
    _check(vd, errs, precision)


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_filament_twenty_ionizing_steps_vs_oracle(precision):
    vd, errs = _device_run("cart_filament_128", 20, precision)
    print("cart_filament_128", precision, "20 steps", fmt(errs))
    _check(vd, errs, precision)
