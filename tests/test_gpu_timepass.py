"""The time-axis pass at the frequency grids of the benchmark configurations (N0 = 257, 513, 1025,
2049), where it runs with compile-time sizes (searay_gb300/csrc/timepass.cu), and at the longest
time axis the library accepts (N0 = 4097, Nt = 8192: one transverse point per block, the
runtime-size kernel): one fixed RK4 step and the finish against the FP64 oracle, on a 16 x 16
Cartesian grid with the filamentation medium and a pulse strong enough to ionize.  Bounds: those of
tests/parity.py for FP32 transverse transforms (field, fluence and spectrum 1e-5; J, chi, ne
1e-4)."""
import numpy as np
import pytest

from parity import DIAG_TOL, check_field, field_errors, fmt

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


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("n0", [257, 513, 1025, 2049, 4097])
def test_time_pass_rk4_step_vs_oracle(n0, precision):
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=16)
    vd["wave grid"] = (n0, 16, 16, 2)
    vd["frequency band"] = (0.0, 4.0 * (n0 - 1) / 512)
    vd["nonlinear band"] = (0.0, 3.5 * (n0 - 1) / 512)
    wave = vd["incoming wave"]
    vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, ionization.RateCoefficients(vd["ionizer"]), precision)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    L = vd["size"][2] / 400
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    A_ref, J_ref, chi_ref, ne_ref, nsteps = O.Oracle(vd).propagator(a, 0.0, L, 1, L)
    A, J, chi_w, ne, evals = uppe.propagator(dev, mat, torch.from_numpy(a.astype(np.complex64)).cuda(), 1, 0.0, L, L)
    assert nsteps == 1 and evals == 4
    errs = field_errors(A.cpu().numpy(), A_ref)
    errs.update({"J": rel_err(J.cpu().numpy(), J_ref), "chi": rel_err(chi_w.cpu().numpy(), chi_ref),
                 "ne": rel_err(ne.cpu().numpy(), ne_ref)})
    print(n0, precision, fmt(errs))
    assert np.max(np.abs(ne_ref)) > 0
    check_field(errs, False)
    assert errs["J"] < DIAG_TOL and errs["chi"] < DIAG_TOL and errs["ne"] < DIAG_TOL
    dev.close()


@pytest.mark.parametrize("n0,n_perp", [(257, 16), (513, 32), (1025, 16)])
def test_register_time_pass_matches_shared_memory_form(n0, n_perp, monkeypatch):
    """The register-resident time pass (M = 256, 512, 1024) against the shared-memory Stockham form
    (SEARAY_UPPE_TIME=smem) on the same field: one RHS evaluation, ionizing columns included.  Both are
    FP32 transforms of the same sums, each within about 2e-6 of the FP64 RHS on these grids; they are
    held to the RHS bound of the oracle comparisons, 1e-5 (w-bins 4 and up)."""
    import torch
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=n_perp)
    vd["wave grid"] = (n0, n_perp, n_perp, 2)
    vd["frequency band"] = (0.0, 4.0 * (n0 - 1) / 512)
    vd["nonlinear band"] = (0.0, 3.5 * (n0 - 1) / 512)
    wave = vd["incoming wave"]
    vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    g = grid.VolumeGrid(vd)
    a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
    out = {}
    for form in ("reg", "smem"):
        if form == "smem":
            monkeypatch.setenv("SEARAY_UPPE_TIME", "smem")
        else:
            monkeypatch.delenv("SEARAY_UPPE_TIME", raising=False)
        dev = uppe.DeviceGrid(g, vd, ionization.RateCoefficients(vd["ionizer"]), "mixed")
        chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
        mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                            vd["density lambda"])
        mat.UpdateMaterial(100.0)
        dev.load_field(a)
        q = dev.empty_field()
        dev.get_field(q)
        S = dev.empty_field()
        dev.eval_rhs(q, 50.0, S)
        out[form] = S.cpu().numpy()
        dev.close()
    e = rel_err(out["reg"][4:], out["smem"][4:])
    print(n0, n_perp, f"register vs shared-memory time pass: {e:.2e}")
    assert np.max(np.abs(out["smem"][4:])) > 0 and e < 1e-5


def _adjoint_step(vd, g, a, lam, form, ionizing, chi3, monkeypatch):
    """(cotangent of q, chi3 derivative, kernel launches) of one RK4 step's VJP in the given form."""
    import torch
    from searay_gb300 import ionization, uppe
    if form == "smem":
        monkeypatch.setenv("SEARAY_UPPE_TIME", "smem")
    else:
        monkeypatch.delenv("SEARAY_UPPE_TIME", raising=False)
    rates = ionization.RateCoefficients(vd["ionizer"]) if ionizing else None
    dev = uppe.DeviceGrid(g, vd, rates, "mixed")
    dev.set_chi3(chi3 / vd["density reference"])
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, chi3, vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    mat.UpdateMaterial(100.0)
    dev.load_field(torch.from_numpy(a.astype(np.complex64)).cuda())
    q = dev.empty_field()
    dev.get_field(q)
    gq = dev.empty_field()
    l0 = dev.launches()
    dred = dev.adjoint_step(q, torch.from_numpy(lam.astype(np.complex64)).cuda(), gq, 50.0, 100.0)
    launches = dev.launches() - l0
    assert not dev.nonfinite()
    out = gq.cpu().numpy()
    dev.close()
    return out, dred, launches


@pytest.mark.parametrize("ionizing", [True, False], ids=["ionizing", "kerr"])
@pytest.mark.parametrize("n0,n_perp", [(257, 64), (513, 64), (1025, 64)])
def test_register_adjoint_time_pass_matches_shared_memory_form(n0, n_perp, ionizing, monkeypatch):
    """The vector-Jacobian product of one RK4 step with the register-resident adjoint time pass
    (timepass_adj_reg.cu: the column groups without ionization; the groups with a nonzero rate go to
    the shared-memory kernel from its list) against the shared-memory form alone
    (SEARAY_UPPE_TIME=smem) on the same field and cotangent.  The time pass gives the nonlinear
    part of the cotangent of q, so the error is measured on that part: the difference of the two
    forms over max |g - g_lin|, g_lin the cotangent with chi3 = 0 and no ionization (time pass
    output zero).  Both are FP32 forms of the same sums: held to 1e-4 there, and to 1e-3 relative
    on the chi3 derivative, a sum of some 10^7 terms of both signs over the grid whose total is far
    below the sum of their magnitudes (measured 1e-6 to 2e-4 between the forms; its accuracy against
    FP64 autograd is held in test_gpu_adjoint.py and test_gpu_bigslice.py).  Kerr coefficient at 30x the workload's, so that the nonlinear part is
    a measurable share of the cotangent (the linear part is the same code, bit for bit, in both
    forms).  With ionization the register form launches one more kernel per
    stage (the listed groups), which shows both kernels ran.  64 x 64 columns: the register pass takes
    grids whose blocks fill the multiprocessors."""
    from searay_gb300 import grid, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=n_perp)
    vd["wave grid"] = (n0, n_perp, n_perp, 2)
    vd["frequency band"] = (0.0, 4.0 * (n0 - 1) / 512)
    vd["nonlinear band"] = (0.0, 3.5 * (n0 - 1) / 512)
    wave = vd["incoming wave"]
    vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    g = grid.VolumeGrid(vd)
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    rng = np.random.default_rng(11)
    lam = (rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)) * (np.abs(a) + 1e-3 * np.abs(a).max())
    chi3 = 30.0 * vd["chi3"]
    g_lin, _, _ = _adjoint_step(vd, g, a, lam, "reg", False, 0.0, monkeypatch)
    out, launches = {}, {}
    for form in ("reg", "smem"):
        gq, dred, launches[form] = _adjoint_step(vd, g, a, lam, form, ionizing, chi3, monkeypatch)
        out[form] = (gq, dred)
    nl = np.max(np.abs(out["smem"][0] - g_lin))
    share = nl / np.max(np.abs(out["smem"][0]))
    e = float(np.max(np.abs(out["reg"][0] - out["smem"][0])) / nl)
    ed = abs(out["reg"][1] - out["smem"][1]) / abs(out["smem"][1])
    print(n0, n_perp, "ionizing" if ionizing else "kerr", f"nonlinear share {share:.2e}",
          f"register vs shared-memory adjoint time pass: {e:.2e}, chi3 derivative {ed:.2e}", launches)
    assert share > 1e-4
    assert e < 1e-4
    assert ed < 1e-3
    if ionizing:
        assert launches["reg"] - launches["smem"] == 4, launches
