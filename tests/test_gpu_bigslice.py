"""Cartesian slices above 128 x 128 (row and column passes, searay_gb300/csrc/slice_big.cu):
256 x 256 (the 1025 x 256 x 256 filament configuration's slice), 128 x 256 and 256 x 128.

* the spectral load, one RHS evaluation and one fixed RK4 step with the finish against the FP64
  oracle (q 2e-6, RHS 1e-5 on bins >= 4; field, fluence and spectrum 1e-5, J, chi and ne 1e-4:
  the bounds of tests/parity.py for FP32 transverse transforms);
* the vector-Jacobian products of the step, the load and the finish against FP64 torch autograd
  of the same functions (2e-4, as the adjoint tests of the other slice kernels).

Inputs: the 800 nm filamentation medium of the bench workload (air, Kerr, O2 tunnelling, plasma
current), the pulse at 3x field so that the plasma terms matter, on 33 frequencies."""
import numpy as np
import pytest

from parity import DIAG_TOL, check_field, field_errors, fmt

pytestmark = pytest.mark.gpu
SHAPES = [(33, 256, 256), (33, 128, 256), (33, 256, 128)]


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()


def rel_err(x, ref):
    return float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))


def _setup(shape, precision="mixed"):
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=shape[1])
    vd["wave grid"] = (shape[0], shape[1], shape[2], 2)
    wave = vd["incoming wave"]
    vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, ionization.RateCoefficients(vd["ionizer"]), precision)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    return vd, g, dev, mat, O.Oracle(vd)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_big_slice_vs_oracle(shape):
    import torch
    from searay_gb300 import uppe
    vd, g, dev, mat, orc = _setup(shape)
    L = vd["size"][2] / 400
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    a_dev = torch.from_numpy(a.astype(np.complex64)).cuda()
    z = 0.5 * L
    mat.UpdateMaterial(z)
    orc.mat.update(z)
    dev.load_field(a_dev)
    q = dev.empty_field()
    dev.get_field(q)
    q_ref = orc.g.kspace(a)
    S = dev.empty_field()
    dev.eval_rhs(q, 0.25 * L, S)
    S_ref = orc.load_source(q_ref, 0.25 * L)
    errs = {"q": rel_err(q.cpu().numpy(), q_ref), "S": rel_err(S.cpu().numpy()[4:], S_ref[4:])}
    A_ref, J_ref, chi_ref, ne_ref, nsteps = orc.propagator(a, 0.0, L, 1, L)
    A, J, chi, ne, evals = uppe.propagator(dev, mat, a_dev, 1, 0.0, L, L)
    assert nsteps == 1 and evals == 4
    errs.update(field_errors(A.cpu().numpy(), A_ref))
    errs.update({"J": rel_err(J.cpu().numpy(), J_ref), "chi": rel_err(chi.cpu().numpy(), chi_ref),
                 "ne": rel_err(ne.cpu().numpy(), ne_ref)})
    print(shape, fmt(errs))
    assert np.max(np.abs(ne_ref)) > 0
    assert errs["q"] < 2e-6 and errs["S"] < 1e-5
    check_field(errs, False)
    assert errs["J"] < DIAG_TOL and errs["chi"] < DIAG_TOL and errs["ne"] < DIAG_TOL
    assert not dev.nonfinite()
    dev.close()


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_big_slice_adjoints_match_torch_fp64(shape):
    import torch
    from torch_reference import TorchStep
    vd, g, dev, mat, orc = _setup(shape)
    zmat = 3000.0
    mat.UpdateMaterial(zmat)
    orc.mat.update(zmat)
    ts = TorchStep(orc)
    redchi3 = vd["chi3"] / vd["density reference"]
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    q0 = orc.g.kspace(a)
    rng = np.random.default_rng(3)
    lam = (rng.standard_normal(q0.shape) + 1j * rng.standard_normal(q0.shape)) * (np.abs(q0) + 1e-3 * np.abs(q0).max())
    z, dz = 1500.0, 2500.0
    errs = {}
    x = torch.tensor(q0.real, requires_grad=True)
    y = torch.tensor(q0.imag, requires_grad=True)
    c3 = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
    q1 = ts.step(torch.complex(x, y), z, dz, c3)
    (torch.as_tensor(lam).conj() * q1).real.sum().backward()
    g_ref = x.grad.numpy() + 1j * y.grad.numpy()
    q0d = torch.from_numpy(q0.astype(np.complex64)).cuda()
    lamd = torch.from_numpy(lam.astype(np.complex64)).cuda()
    out = dev.empty_field()
    dred = dev.adjoint_step(q0d, lamd, out, z, dz)
    errs["step"] = rel_err(out.cpu().numpy(), g_ref)
    errs["dchi3"] = abs(dred - float(c3.grad)) / abs(float(c3.grad))
    x = torch.tensor(q0.real, requires_grad=True)
    y = torch.tensor(q0.imag, requires_grad=True)
    A = ts.finish_field(torch.complex(x, y), z)
    (torch.as_tensor(lam).conj() * A).real.sum().backward()
    g_ref = x.grad.numpy() + 1j * y.grad.numpy()
    dev.adjoint_finish(z, lamd, out)
    errs["finish"] = rel_err(out.cpu().numpy(), g_ref)
    x = torch.tensor(a.real, requires_grad=True)
    y = torch.tensor(a.imag, requires_grad=True)
    qk = ts.kspace(torch.complex(x, y))
    (torch.as_tensor(lam).conj() * qk).real.sum().backward()
    g_ref = x.grad.numpy() + 1j * y.grad.numpy()
    dev.adjoint_load(lamd, out)
    errs["load"] = rel_err(out.cpu().numpy(), g_ref)
    print({k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < 2e-4, (k, e)
    dev.close()


def test_cluster_tail_matches_three_passes(monkeypatch):
    """256 x 256 slices: the fused evaluation tail on a cluster of 8 CTAs (slice_cluster.cu: the slice
    in distributed shared memory, one launch) against the three-pass form (rows, columns, inverse
    rows through HBM, the default) on the same field: three fixed RK4 steps (every stage
    mode, the slices above the nonlinear cut included) and the finish.  Both run the same line
    transforms and pointwise arithmetic, so they agree to rounding (1e-6 of the maximum)."""
    import torch
    from searay_gb300 import uppe
    out, launches = {}, {}
    for form in ("cluster", "passes"):
        if form == "cluster":
            monkeypatch.setenv("SEARAY_UPPE_CLUSTER", "1")
        else:
            monkeypatch.delenv("SEARAY_UPPE_CLUSTER", raising=False)
        vd, g, dev, mat, orc = _setup((65, 256, 256))
        L = vd["size"][2] / 400
        a_dev = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
        l0 = dev.launches()
        A, J, chi, ne, evals = uppe.propagator(dev, mat, a_dev, 3, 0.0, 3 * L, L)
        assert evals == 12 and not dev.nonfinite()
        q = dev.empty_field()
        dev.get_field(q)
        out[form] = (A.cpu().numpy(), J.cpu().numpy(), q.cpu().numpy())
        launches[form] = dev.launches() - l0
        dev.close()
    # one launch per evaluation tail instead of three: the cluster form really ran
    assert launches["passes"] - launches["cluster"] == 2 * 12, launches
    errs = {k: rel_err(out["cluster"][n], out["passes"][n]) for n, k in enumerate(("A", "J", "q"))}
    print("cluster vs three passes", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < 1e-6, (k, e)
