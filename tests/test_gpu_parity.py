"""Parity of the GB300 CUDA path (through the C ABI) with the reference on the same inputs.

Targets are the golden fixtures made from SeaRay's own UPPE path (tests/golden/make_golden.py) and
the FP64 oracle.  Error metric: max |x - x_ref| / max |x_ref| over an output array.
Tolerances: the field A within 2e-5 (plain FP32 form) and 2e-5 (mixed form); the diagnostic
outputs J, chi, ne within 1e-4 (they pass through the exponentially stiff rate)."""
import numpy as np
import pytest

import replay

pytestmark = pytest.mark.gpu

TOL = {"A": 2e-5, "J": 1e-4, "chi": 1e-4, "ne": 1e-4}


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


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("name", replay.CASE_NAMES)
def test_track_matches_reference(name, precision):
    from searay_gb300 import uppe
    vd, exp = replay.load_case(name)
    vd["precision"] = precision
    A, J, chi, ne, dom4d = uppe.track(None, None, None, None, vd)
    assert np.array_equal(dom4d, exp["dom4d"])
    errs = {}
    for key, arr in (("A", A), ("J", J), ("chi", chi), ("ne", ne)):
        ref = exp[key]
        if np.max(np.abs(ref)) == 0:
            assert np.max(np.abs(arr[..., 1:])) == 0
            continue
        errs[key] = rel_err(arr[..., 1:], ref)
    print(name, precision, {k: f"{v:.2e}" for k, v in errs.items()})
    for key, e in errs.items():
        assert e < TOL[key], (key, e)


def _device_case(name, precision="mixed"):
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe
    vd, _ = replay.load_case(name)
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") else None
    dev = uppe.DeviceGrid(g, vd, rates, precision)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                        vd.get("window speed", 1.0), vd["density lambda"])
    orc = O.Oracle(vd)
    return vd, g, dev, mat, orc


@pytest.mark.parametrize("name", replay.CASE_NAMES)
def test_transform_and_rhs_vs_oracle(name):
    """One kspacex of the incoming field and one load_source evaluation, against FP64."""
    import torch
    vd, g, dev, mat, orc = _device_case(name)
    z = 1234.5
    mat.UpdateMaterial(z)
    orc.mat.update(z)
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    a_dev = torch.from_numpy(a.astype(np.complex64)).cuda()
    dev.load_field(a_dev)
    q_dev = dev.empty_field()
    dev.get_field(q_dev)
    q_ref = orc.g.kspace(a)
    assert rel_err(q_dev.cpu().numpy(), q_ref) < 2e-6
    S_dev = dev.empty_field()
    dev.eval_rhs(q_dev, z, S_dev)
    S_ref = orc.load_source(q_ref, z)
    S = S_dev.cpu().numpy()
    # w-bins 0-3 are zeroed by the DC conditioner after every stage (uppe_kernel.py:127-137); there
    # Re kz ~ w is small and S amplifies rounding, so they are reported but not held to the bound
    e_all = rel_err(S, S_ref)
    e = rel_err(S[4:], S_ref[4:])
    print(name, f"rhs {e:.2e} (all bins {e_all:.2e})")
    assert e < 1e-5
    dev.close()


def test_long_z_phase_mixed_vs_fp32():
    """The float-float phase keeps the RHS accurate at z ~ 4e5 (about 5 cm); report the FP32 form."""
    import torch
    errs = {}
    for precision in ("mixed", "fp32"):
        vd, g, dev, mat, orc = _device_case("cart_ion", precision)
        z = 4.0e5
        mat.UpdateMaterial(1.0)
        orc.mat.update(1.0)
        a = vd["incoming wave"](g.w, g.x1, g.x2)
        q_ref = orc.g.kspace(a)
        q_dev = torch.from_numpy(q_ref.astype(np.complex64)).cuda()
        S_dev = dev.empty_field()
        dev.eval_rhs(q_dev, z, S_dev)
        errs[precision] = rel_err(S_dev.cpu().numpy()[4:], orc.load_source(q_ref, z)[4:])
        dev.close()
    print("long z rhs", errs)
    assert errs["mixed"] < 2e-5


def test_gaussian_known_answer_gpu():
    """test/gaussian_test.py:110-154 through the GPU path."""
    from searay_gb300 import uppe
    from test_oracle_golden import _gaussian_case, check_gaussian_expansion
    vd, r00 = _gaussian_case()
    A, J, chi, ne, dom4d = uppe.track(None, None, None, None, vd)
    check_gaussian_expansion(A, dom4d, r00)


def test_nonfinite_input_is_flagged():
    """A NaN in the incoming field is reported by the device non-finite check (no trap)."""
    import torch
    vd, g, dev, mat, orc = _device_case("cart_ion")
    mat.UpdateMaterial(0.0)
    a = vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)
    a[10, 3, 3] = np.nan
    dev.load_field(torch.from_numpy(a).cuda())
    assert dev.nonfinite()
    dev.close()
