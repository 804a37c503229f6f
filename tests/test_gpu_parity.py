"""Parity of the GB300 CUDA path (through the C ABI) with the reference on the same inputs.

Targets are the golden fixtures made from SeaRay's own UPPE path (tests/golden/make_golden.py) and
the FP64 oracle.  Metrics and bounds are those of tests/parity.py: max |x - x_ref| / max |x_ref|
per output array, plus the fluence (sum over w of |A|^2 per transverse point) and the spectrum (sum
over the transverse points of |A|^2 per w) of the field.
  * FP32 transverse transforms (every Cartesian run, and cylindrical runs in the plain FP32 form):
    field, fluence and spectrum within 1e-5; diagnostics J, chi, ne within 1e-4 (they pass
    through the stiff rate);
  * the tensor-core Hankel transform of the mixed form (split-BF16x3, about 1e-5 per transform):
    every output within 1e-4, the bound stated for the mixed-precision form."""
import numpy as np
import pytest

import replay
from parity import DIAG_TOL, check_field, field_errors, field_tol, fmt, rel_err

pytestmark = pytest.mark.gpu


def tensor_core_hankel(vd, precision):
    return vd["wave coordinates"] != "cartesian" and precision == "mixed"


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()
    return True


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("name", replay.CASE_NAMES)
def test_track_matches_reference(name, precision):
    from searay_gb300 import uppe
    vd, exp = replay.load_case(name)
    vd["precision"] = precision
    A, J, chi, ne, dom4d = uppe.track(None, None, None, None, vd)
    assert np.array_equal(dom4d, exp["dom4d"])
    errs = field_errors(A[..., 1:], exp["A"])
    for key, arr in (("J", J), ("chi", chi), ("ne", ne)):
        ref = exp[key]
        if np.max(np.abs(ref)) == 0:
            assert np.max(np.abs(arr[..., 1:])) == 0
            continue
        errs[key] = rel_err(arr[..., 1:], ref)
    print(name, precision, fmt(errs))
    tc = tensor_core_hankel(vd, precision)
    check_field(errs, tc)
    for key in ("J", "chi", "ne"):
        if key in errs:
            assert errs[key] < DIAG_TOL, (key, errs[key])


def _device_case(name, precision="mixed"):
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe
    vd, _ = replay.load_case(name)
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") else None
    dev = uppe.DeviceGrid(g, vd, rates, precision)
    dev.set_rotator(vd.get("rotator"))
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                        vd.get("window speed", 1.0), vd["density lambda"])
    orc = O.Oracle(vd)
    return vd, g, dev, mat, orc


def test_tensor_core_and_simt_hankel_agree():
    """The split-BF16x3 tensor-core Hankel transform against the FP32 SIMT one on the same field."""
    import torch
    out = {}
    for precision in ("fp32", "mixed"):
        vd, g, dev, mat, orc = _device_case("cyl_az_adk", precision)
        mat.UpdateMaterial(50.0)
        a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        dev.load_field(a)
        q = dev.empty_field()
        dev.get_field(q)
        S = dev.empty_field()
        dev.eval_rhs(q, 50.0, S)
        out[precision] = (q.cpu().numpy(), S.cpu().numpy())
        assert not dev.nonfinite()
        dev.close()
    eq = rel_err(out["mixed"][0], out["fp32"][0])
    es = rel_err(out["mixed"][1][4:], out["fp32"][1][4:])
    print("tensor vs simt", f"q {eq:.2e} S {es:.2e}")
    assert eq < 5e-5 and es < 1e-4


@pytest.mark.parametrize("name", ["cyl_kerr", "cyl_raman"])
def test_stage_update_writes_next_transform_operand(name, monkeypatch):
    """Mixed form, one azimuthal node: the time pass writes J straight into the split operand tiles
    of the forward tensor-core transform, and the spectral update of RK stages 1-3 writes those of
    the next inverse transform (k_spec_point); both transforms then skip their pre-pass
    (k_hankel_tc_prep); the step's final update also writes the operand of the next step's first
    inverse transform, used when that step starts at the same z (bit for bit) with nothing called in
    between.  Against SEARAY_UPPE_TC_NEXT=0 (every transform forms its operand itself) over three
    fixed steps: the same arithmetic on the same values, so the field, J and the held q agree bit
    for bit, with seven launches fewer per step (four forward, three inverse) and one more for each
    step whose start z matches the previous step's end exactly (the z's are summed on the host)."""
    import torch
    from searay_gb300 import uppe
    out, launches = {}, {}
    for form in ("fused", "prepass"):
        if form == "prepass":
            monkeypatch.setenv("SEARAY_UPPE_TC_NEXT", "0")
        else:
            monkeypatch.delenv("SEARAY_UPPE_TC_NEXT", raising=False)
        vd, g, dev, mat, orc = _device_case(name, "mixed")
        L = vd["size"][2] / 20
        a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        l0 = dev.launches()
        A, J, chi, ne, evals = uppe.propagator(dev, mat, a, 3, 0.0, 3 * L, L)
        assert evals == 12 and not dev.nonfinite()
        launches[form] = dev.launches() - l0
        q = dev.empty_field()
        dev.get_field(q)
        out[form] = (A.cpu().numpy(), J.cpu().numpy(), q.cpu().numpy())
        dev.close()
    print(name, launches)
    assert 3 * 7 <= launches["prepass"] - launches["fused"] <= 3 * 7 + 2, launches
    for x, y in zip(out["fused"], out["prepass"]):
        assert np.array_equal(x, y)


def test_operand_carried_between_steps_is_dropped_by_other_calls(monkeypatch):
    """The tiles a step leaves for the next step's first inverse transform are only used by an
    immediately following uppe_rk4_step: here a step, then uppe_set_field with another field (same
    z), then a step from it, in the fused and the pre-pass forms.  A stale operand would transform
    the old field; both forms must give the same result bit for bit."""
    import torch
    out = {}
    for form in ("fused", "prepass"):
        if form == "prepass":
            monkeypatch.setenv("SEARAY_UPPE_TC_NEXT", "0")
        else:
            monkeypatch.delenv("SEARAY_UPPE_TC_NEXT", raising=False)
        vd, g, dev, mat, orc = _device_case("cyl_kerr", "mixed")
        L = vd["size"][2] / 20
        mat.UpdateMaterial(0.5 * L)
        a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        dev.load_field(a)
        dev.rk4_step(0.0, L, 0.0, L)
        q = dev.empty_field()
        dev.get_field(q)
        dev.set_field(0.5 * q)
        dev.rk4_step(L, L, 0.0, L)
        dev.get_field(q)
        out[form] = q.cpu().numpy()
        assert not dev.nonfinite()
        dev.close()
    assert np.array_equal(out["fused"], out["prepass"])


def test_adjoint_time_pass_writes_transform_operand(monkeypatch):
    """Mixed form, one azimuthal node: in the vector-Jacobian product of a step the adjoint time
    pass writes the cotangent of E straight into the operand tiles of the Minv^T transform that
    follows (its pre-pass skipped).  Against SEARAY_UPPE_TC_NEXT=0: the same arithmetic on the same
    values, so the cotangent of q agrees bit for bit and the chi3 derivative to its summation order,
    with at least four launches fewer (one per stage)."""
    import torch
    out, launches = {}, {}
    for form in ("fused", "prepass"):
        if form == "prepass":
            monkeypatch.setenv("SEARAY_UPPE_TC_NEXT", "0")
        else:
            monkeypatch.delenv("SEARAY_UPPE_TC_NEXT", raising=False)
        vd, g, dev, mat, orc = _device_case("cyl_kerr", "mixed")
        L = vd["size"][2] / 20
        mat.UpdateMaterial(0.5 * L)
        a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        dev.load_field(a)
        q = dev.empty_field()
        dev.get_field(q)
        rng = np.random.default_rng(5)
        qn = q.cpu().numpy()
        lam = torch.from_numpy(((rng.standard_normal(qn.shape) + 1j * rng.standard_normal(qn.shape)) *
                                np.abs(qn)).astype(np.complex64)).cuda()
        gq = dev.empty_field()
        l0 = dev.launches()
        dred = dev.adjoint_step(q, lam, gq, 0.0, L)
        launches[form] = dev.launches() - l0
        out[form] = (gq.cpu().numpy(), dred)
        assert not dev.nonfinite()
        dev.close()
    print("adjoint launches", launches)
    assert launches["prepass"] - launches["fused"] >= 4, launches
    assert np.array_equal(out["fused"][0], out["prepass"][0])
    # (the chi3 derivative is summed by atomics in a run-dependent order)
    assert abs(out["fused"][1] - out["prepass"][1]) <= 1e-12 * abs(out["prepass"][1])


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
    tc = tensor_core_hankel(vd, "mixed")
    assert rel_err(q_dev.cpu().numpy(), q_ref) < (5e-5 if tc else 2e-6)
    S_dev = dev.empty_field()
    dev.eval_rhs(q_dev, z, S_dev)
    S_ref = orc.load_source(q_ref, z)
    S = S_dev.cpu().numpy()
    # w-bins 0-3 are zeroed by the DC conditioner after every stage (uppe_kernel.py:127-137); there
    # Re kz ~ w is small and S amplifies rounding, so they are reported but not held to the bound
    e_all = rel_err(S, S_ref)
    e = rel_err(S[4:], S_ref[4:])
    print(name, f"rhs {e:.2e} (all bins {e_all:.2e})")
    assert e < (1e-4 if tc else 1e-5)
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
    assert errs["mixed"] < 1e-5


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


def test_kerr_collapse_long_run():
    """cyl_kerr_64 (the config-1 beam: about twice the critical power of air, Kerr only, 100 fixed
    steps over 10 cm) through 80 steps, on the GPU in both forms and in the FP64 oracle: the fields
    agree after 80 steps (the peak has grown by about 11 %), and carried on to step 100 both have
    overflowed, the unarrested self-focusing collapse near the end of the 10 cm (about step 88 in
    the oracle).  Bounds after 80 steps: the forms' field bounds, 1e-4 with the split-BF16
    tensor-core transforms of the mixed form and 1e-5 for the plain FP32 form, applied to the field,
    its fluence and its spectrum."""
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, uppe, workloads
    vd = workloads.cyl_kerr_64(steps=100)
    g = grid.VolumeGrid(vd)
    L = vd["size"][2]
    dz = L / 100
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    orc = O.Oracle(vd)
    A80, _, _, _, n80 = orc.propagator(a, 0.0, 80 * dz, 80, dz)
    assert n80 == 80 and np.isfinite(A80).all()
    with np.errstate(all="ignore"):
        A100, _, _, _, _ = orc.propagator(A80, 80 * dz, 100 * dz, 20, dz)
    assert not np.isfinite(A100).all()
    for precision in ("mixed", "fp32"):
        dev = uppe.DeviceGrid(g, vd, None, precision)
        chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
        mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd["chi3"], vd["density reference"],
                            vd["window speed"], vd["density lambda"])
        A, _, _, _, ev = uppe.propagator(dev, mat, torch.from_numpy(a.astype(np.complex64)).cuda(), 80, 0.0,
                                         80 * dz, dz)
        assert ev == 4 * 80
        A = A.cpu().numpy()
        errs = field_errors(A, A80)
        B, _, _, _, _ = uppe.propagator(dev, mat, torch.from_numpy(A.astype(np.complex64)).cuda(), 20, 80 * dz,
                                        100 * dz, dz)
        finite100 = bool(np.isfinite(B.cpu().numpy()).all())
        print(precision, "80 steps", fmt(errs), "finite at 100:", finite100, "peak growth",
              float(np.abs(A80).max() / np.abs(a).max()))
        check_field(errs, precision == "mixed")
        assert not finite100
        dev.close()
