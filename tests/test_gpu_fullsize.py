"""Parity at the full sizes of the benchmark workloads: one fixed RK4 step from the incoming plane
on the device (mixed precision) against the FP64 oracle on the same grid.

* cart_filament_128: 513 x 128 x 128 Cartesian, Kerr + O2 tunneling + plasma current (the
  default bench workload: register-resident slices, the zero-current slices split off);
* cyl_silica_512: 2049 x 512 cylindrical, fused silica with ionization (the tensor-core Hankel
  transforms).

The oracle step takes a few seconds on the host cores.  Bounds: the golden parity tolerances, field
2e-5 for the FP32 transverse transforms and 1e-4 for the split-BF16 tensor-core transforms; J, chi,
ne 1e-4.  Error metric max |x - x_ref| / max |x_ref|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()


def rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("workload,tol_field", [("cart_filament_128", 2e-5), ("cyl_silica_512", 1e-4)])
def test_benchmark_workload_step_vs_oracle(workload, tol_field):
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.WORKLOADS[workload]()
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") is not None else None
    dev = uppe.DeviceGrid(g, vd, rates, "mixed")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd["chi3"], vd["density reference"],
                        vd["window speed"], vd["density lambda"])
    dz = vd["size"][2] / vd["subcycles"]
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    A_ref, J_ref, chi_ref, ne_ref, n = O.Oracle(vd).propagator(a, 0.0, dz, 1, dz)
    assert n == 1
    A, J, chi_w, ne, evals = uppe.propagator(dev, mat, torch.from_numpy(a.astype(np.complex64)).cuda(), 1, 0.0, dz,
                                             dz)
    assert evals == 4
    errs = {"A": rel_err(A.cpu().numpy(), A_ref), "J": rel_err(J.cpu().numpy(), J_ref),
            "chi": rel_err(chi_w.cpu().numpy(), chi_ref), "ne": rel_err(ne.cpu().numpy(), ne_ref)}
    print(workload, {k: f"{v:.2e}" for k, v in errs.items()})
    assert np.max(np.abs(ne_ref)) > 0
    assert errs["A"] < tol_field and errs["J"] < 1e-4 and errs["chi"] < 1e-4 and errs["ne"] < 1e-4
    dev.close()
