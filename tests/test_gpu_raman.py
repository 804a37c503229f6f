"""Rotational Raman response on the GPU (the 'rotator' key: rotations.py Rotator, AddChiUPPE of
rotations.cl:85-129, added to chi before the Kerr term as uppe_kernel.py:173-179 does) against the
FP64 oracle, at shapes the golden case (tests/golden cyl_raman, checked in test_gpu_parity.py) does
not reach: Cartesian slices, Raman together with ionization, longer time axes (fewer transverse
points per block of the time pass) and a block of fewer than 32 threads.

Metrics and bounds of tests/parity.py: field, fluence and spectrum within 1e-5 with FP32
transverse transforms (1e-4 with the tensor-core Hankel transform), current and chi within 1e-4.

Inputs: the 800 nm filamentation medium of the bench workload (air, Kerr, O2 tunnelling, plasma
current, seeded transverse phase screen) with the N2 rotator of the golden case (32 states, 100 ps
dephasing), on smaller grids."""
import numpy as np
import pytest

import cases
from parity import DIAG_TOL, check_field, field_errors, fmt

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()
    return True


def rel_err(x, ref):
    s = np.max(np.abs(ref))
    return np.max(np.abs(x - ref)) / s if s > 0 else np.max(np.abs(x))


def n2_rotator():
    from searay_gb300 import rotations
    return rotations.Rotator(*cases.rotator_args(cases.CASES["cyl_raman"]["rotator"]))


def _setup(shape, rotator, ionize=True, precision="mixed"):
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=shape[1])
    vd["wave grid"] = (shape[0], shape[1], shape[2], 2)
    vd["rotator"] = rotator
    if not ionize:
        vd["ionizer"] = None
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd["ionizer"] is not None else None
    dev = uppe.DeviceGrid(g, vd, rates, precision)
    dev.set_rotator(rotator)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    return vd, g, dev, mat


# (N0, N1, N2): 16 points per block at Nt = 256; 4 at Nt = 2048; 1 at Nt = 8192
SHAPES = [(129, 16, 16), (1025, 16, 8), (4097, 4, 4)]


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_raman_rk4_step_vs_oracle(shape, precision):
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import uppe
    rot = n2_rotator()
    vd, g, dev, mat = _setup(shape, rot, precision=precision)
    L = vd["size"][2] / 400
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    orc = O.Oracle(vd)
    assert orc.rotator is rot
    A_ref, J_ref, chi_ref, ne_ref, nsteps = orc.propagator(a, 0.0, L, 1, L)
    assert nsteps == 1
    a_dev = torch.from_numpy(a.astype(np.complex64)).cuda()
    A, J, chi, ne, evals = uppe.propagator(dev, mat, a_dev, 1, 0.0, L, L)
    assert evals == 4
    errs = field_errors(A.cpu().numpy(), A_ref)
    errs.update({"J": rel_err(J.cpu().numpy(), J_ref), "chi": rel_err(chi.cpu().numpy(), chi_ref)})
    print(shape, precision, fmt(errs))
    check_field(errs, False)
    assert errs["J"] < DIAG_TOL and errs["chi"] < DIAG_TOL
    dev.close()


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_raman_small_cylindrical_block(precision):
    """17 frequencies on 4 radial nodes: 8 threads per block of the time pass (the scan without a
    full warp)."""
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import dispersion, grid, uppe
    c = cases.CASES["cyl_raman"]
    vd = dict(c["keys"])
    vd.update({"wave grid": (17, 4, 1, 2), "radial modes": 4, "precision": precision, "ionizer": None,
               "dispersion inside": dispersion.SimpleAir(cases.MKS_LENGTH), "rotator": n2_rotator(),
               "density lambda": cases.density_lambda(c["density"])})
    wave = dict(c["wave"], dw=0.4, E0=0.008)
    vd["incoming wave"] = cases.make_wave(wave, vd["size"][0])
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, None, precision)
    dev.set_rotator(vd["rotator"])
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd["chi3"], vd["density reference"],
                        vd["window speed"], vd["density lambda"])
    L = 2000.0
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    A_ref, J_ref, chi_ref, _, _ = O.Oracle(vd).propagator(a, 0.0, L, 1, L)
    a_dev = torch.from_numpy(a.astype(np.complex64)).cuda()
    A, J, chi_d, _, _ = uppe.propagator(dev, mat, a_dev, 1, 0.0, L, L)
    errs = field_errors(A.cpu().numpy(), A_ref)
    errs.update({"J": rel_err(J.cpu().numpy(), J_ref), "chi": rel_err(chi_d.cpu().numpy(), chi_ref)})
    print("17x4x1", precision, fmt(errs))
    # the 4-mode Hankel transform of the mixed form runs on the tensor cores (1e-4 bound)
    check_field(errs, precision == "mixed")
    assert errs["J"] < DIAG_TOL and errs["chi"] < DIAG_TOL
    dev.close()


def test_raman_changes_chi_and_can_be_removed():
    """The Raman part is a large share of chi here; removing the rotator gives the Kerr-only result."""
    import torch
    from searay_gb300 import uppe
    shape = (129, 16, 16)
    out = {}
    for key, rot in (("raman", n2_rotator()), ("kerr", None), ("removed", n2_rotator())):
        vd, g, dev, mat = _setup(shape, rot, ionize=False)
        if key == "removed":
            dev.set_rotator(None)
        L = vd["size"][2] / 400
        a_dev = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        A, J, chi, ne, _ = uppe.propagator(dev, mat, a_dev, 1, 0.0, L, L)
        out[key] = chi.cpu().numpy()
        dev.close()
    assert np.array_equal(out["removed"], out["kerr"])
    share = rel_err(out["raman"], out["kerr"])
    print("Raman share of chi", f"{share:.3f}")
    assert share > 0.02


def test_adjoint_refuses_rotator():
    import torch
    from searay_gb300 import uppe
    vd, g, dev, mat = _setup((65, 16, 16), n2_rotator(), ionize=False)
    mat.UpdateMaterial(10.0)
    q = dev.empty_field()
    lam = dev.empty_field()
    out = dev.empty_field()
    q.zero_()
    lam.zero_()
    with pytest.raises(RuntimeError, match="Raman"):
        dev.adjoint_step(q, lam, out, 0.0, 10.0)
    dev.close()
