"""Register-resident Cartesian slice kernels (searay_gb300/csrc/slice_reg.cuh) at slice sizes the
golden cases do not reach.

* Against the generic shared-memory Stockham kernels (``SEARAY_UPPE_SLICE=generic``) on the same
  inputs: the spectral field after loading, one RHS evaluation, two fixed RK4 steps and the finish
  (every kernel family: spectral load, inverse, fused tail, finish); max |a - b| / max |b| below
  1e-5 (1e-4 for the current).
* At the bench's 128 x 128 slice: one fixed RK4 step and the finish against the FP64 oracle; field,
  fluence and spectrum within 1e-5 and current within 1e-4 (tests/parity.py).

Inputs: the 800 nm filamentation medium of the bench workload (air, Kerr, O2 tunnelling, plasma
current) with its seeded transverse phase screen, on smaller frequency grids."""
import os

import numpy as np
import pytest

from parity import DIAG_TOL, check_field, field_errors, fmt

pytestmark = pytest.mark.gpu

SHAPES = [(129, 128, 128), (65, 64, 32), (65, 16, 128), (65, 32, 16), (65, 16, 16)]


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


def _setup(shape, generic, precision="mixed"):
    from searay_gb300 import grid, ionization, uppe, workloads
    vd = workloads.cart_filament_128(steps=400, n_perp=shape[1])
    vd["wave grid"] = (shape[0], shape[1], shape[2], 2)
    if generic:
        os.environ["SEARAY_UPPE_SLICE"] = "generic"
    try:
        g = grid.VolumeGrid(vd)
        rates = ionization.RateCoefficients(vd["ionizer"])
        dev = uppe.DeviceGrid(g, vd, rates, precision)
    finally:
        os.environ.pop("SEARAY_UPPE_SLICE", None)
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    return vd, g, dev, mat


def _run(vd, g, dev, mat):
    import torch
    L = vd["size"][2] / 400
    mat.UpdateMaterial(0.5 * L)
    a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
    dev.load_field(a)
    out = {}
    q = dev.empty_field()
    dev.get_field(q)
    out["q0"] = q.cpu().numpy()
    S = dev.empty_field()
    dev.eval_rhs(q, 0.25 * L, S)
    out["S"] = S.cpu().numpy()[4:]
    for n in range(2):
        assert dev.rk4_step(n * L, L, 0.0, L) == pytest.approx(L)
    dev.get_field(q)
    out["q2"] = q.cpu().numpy()
    A, J, chi, ne = (dev.empty_field() for _ in range(4))
    dev.finish(2 * L, A, J, chi, ne)
    out["A"] = A.cpu().numpy()
    out["J"] = J.cpu().numpy()
    assert not dev.nonfinite()
    dev.close()
    return out


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_register_slices_match_generic(shape):
    res = {}
    for generic in (False, True):
        res[generic] = _run(*_setup(shape, generic))
    tol = {"q0": 1e-5, "S": 1e-5, "q2": 1e-5, "A": 1e-5, "J": 1e-4}
    errs = {k: rel_err(res[False][k], res[True][k]) for k in tol}
    print(shape, {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < tol[k], (k, e)


def test_register_slices_rk4_step_vs_oracle_128():
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import uppe
    vd, g, dev, mat = _setup((129, 128, 128), generic=False)
    L = vd["size"][2] / 400
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    orc = O.Oracle(vd)
    A_ref, J_ref, _, _, nsteps = orc.propagator(a, 0.0, L, 1, L)
    assert nsteps == 1
    a_dev = torch.from_numpy(a.astype(np.complex64)).cuda()
    A, J, _, _, evals = uppe.propagator(dev, mat, a_dev, 1, 0.0, L, L)
    assert evals == 4
    errs = field_errors(A.cpu().numpy(), A_ref)
    errs["J"] = rel_err(J.cpu().numpy(), J_ref)
    print("128x128 one step:", fmt(errs))
    check_field(errs, False)
    assert errs["J"] < DIAG_TOL
    dev.close()
