"""Parity of the GB300 paraxial (envelope) path, through the C ABI, with the reference.

Targets: the golden fixtures made from SeaRay's own paraxial_kernel.track (tests/golden/make_golden.py,
cases par_cart_ion, par_cyl_raman, par_cyl_az_adk) and the FP64 paraxial oracle
(oracle/paraxial_oracle.py).  Metrics and bounds are those of tests/parity.py: with FP32
transverse transforms (Cartesian, and cylindrical in the plain FP32 form) field, fluence and
spectrum within 1e-5, J, chi, ne within 1e-4; with the tensor-core Hankel transform of the mixed
form every output within 1e-4."""
import numpy as np
import pytest

import replay
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


def tensor_core_hankel(vd, precision):
    return vd["wave coordinates"] != "cartesian" and precision == "mixed"


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("name", replay.PARAXIAL_CASE_NAMES)
def test_paraxial_track_matches_reference(name, precision):
    from searay_gb300 import paraxial
    vd, exp = replay.load_case(name)
    vd["precision"] = precision
    A, J, chi, ne, dom4d = paraxial.track(None, None, None, None, vd)
    assert np.array_equal(dom4d, exp["dom4d"])
    errs = field_errors(A[..., 1:], exp["A"])
    for key, arr in (("J", J), ("chi", chi), ("ne", ne)):
        ref = exp[key]
        if np.max(np.abs(ref)) == 0:
            assert np.max(np.abs(arr[..., 1:])) == 0
            continue
        errs[key] = rel_err(arr[..., 1:], ref)
    print(name, precision, fmt(errs))
    check_field(errs, tensor_core_hankel(vd, precision))
    for key in ("J", "chi", "ne"):
        if key in errs:
            assert errs[key] < DIAG_TOL, (key, errs[key])


def _device(vd, precision="mixed"):
    from oracle import paraxial_oracle as PO
    from searay_gb300 import grid, ionization, paraxial, uppe
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") else None
    dev = uppe.DeviceGrid(g, vd, rates, precision, envelope=True)
    dev.set_rotator(vd.get("rotator"))
    orc = PO.ParaxialOracle(vd)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = paraxial.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                            orc.w0, orc.ngrp, orc.n0, vd["density lambda"])
    return g, dev, mat, orc


@pytest.mark.parametrize("name", replay.PARAXIAL_CASE_NAMES)
def test_paraxial_load_and_rhs_vs_oracle(name):
    """One kspacex of the incoming field and one load_source evaluation, against FP64."""
    import torch
    vd, _ = replay.load_case(name)
    g, dev, mat, orc = _device(vd)
    z = 1234.5
    mat.UpdateMaterial(z)
    orc.mat.update(z)
    a = np.fft.ifftshift(vd["incoming wave"](g.w, g.x1, g.x2), axes=0)
    dev.load_field(torch.from_numpy(a.astype(np.complex64)).cuda())
    q = dev.empty_field()
    dev.get_field(q)
    q_ref = orc.g.kspace(a)
    tc = tensor_core_hankel(vd, "mixed")
    eq = rel_err(q.cpu().numpy(), q_ref)
    S = dev.empty_field()
    dev.eval_rhs(q, z, S)
    S_ref = orc.load_source(q_ref, z)
    es = rel_err(S.cpu().numpy(), S_ref)
    print(name, f"load {eq:.2e} rhs {es:.2e}")
    assert eq < (5e-5 if tc else 2e-6)
    assert es < (1e-4 if tc else 2e-5)
    dev.close()


def test_paraxial_rk4_step_64x64_vs_oracle():
    """One adaptive RK4 step and the finish on a 256 x 64 x 64 Cartesian grid with ionization (the
    generic slice kernels at a larger slice), against FP64."""
    import torch
    import cases
    from oracle import paraxial_oracle as PO
    from searay_gb300 import dispersion, paraxial
    c = cases.PARAXIAL_CASES["par_cart_ion"]
    vd = dict(c["keys"])
    vd.update({"wave grid": (256, 64, 64, 2), "size": (1600.0, 1600.0, 1.5e4), "ionizer": None,
               "dispersion inside": dispersion.SimpleAir(cases.MKS_LENGTH),
               "density lambda": cases.density_lambda(c["density"])})
    from searay_gb300 import ionization as ion
    from searay_gb300.workloads import Units
    vd["ionizer"] = ion.PPT_Tunneling(cases.MKS_LENGTH, False, Units(cases.MKS_LENGTH).eV(12.07), 0.53)
    vd["incoming wave"] = cases.make_wave(c["wave"], vd["size"][0])
    g, dev, mat, orc = _device(vd)
    L = 300.0
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    A_ref, J_ref, chi_ref, ne_ref, nsteps = orc.propagator(a, 0.0, L, 1)
    a_dev = torch.from_numpy(np.fft.ifftshift(a, axes=0).astype(np.complex64)).cuda()
    A, J, chi, ne, evals = paraxial.propagator(dev, mat, a_dev, 1, 0.0, L)
    assert evals == 4 * nsteps
    sh = lambda t: np.fft.fftshift(t.cpu().numpy(), axes=0)
    errs = field_errors(sh(A), A_ref)
    errs.update({"J": rel_err(sh(J), J_ref), "chi": rel_err(sh(chi), chi_ref), "ne": rel_err(sh(ne), ne_ref)})
    print("256x64x64", nsteps, fmt(errs))
    check_field(errs, False)
    assert errs["J"] < DIAG_TOL and errs["chi"] < DIAG_TOL and errs["ne"] < DIAG_TOL
    dev.close()


def test_paraxial_adjoint_refused():
    vd, _ = replay.load_case("par_cart_ion")
    g, dev, mat, orc = _device(vd)
    mat.UpdateMaterial(10.0)
    q = dev.empty_field()
    q.zero_()
    lam = dev.empty_field()
    lam.zero_()
    out = dev.empty_field()
    with pytest.raises(RuntimeError, match="paraxial"):
        dev.adjoint_step(q, lam, out, 0.0, 10.0)
    dev.close()
