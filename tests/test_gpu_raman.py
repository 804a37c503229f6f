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


@pytest.mark.parametrize("shape,precision", [((129, 16, 16), "mixed"), ((1025, 16, 8), "fp32"), ((4097, 4, 4), "mixed")],
                         ids=["129x16x16", "1025x16x8", "4097x4x4"])
def test_adjoint_with_rotator_matches_torch_fp64(shape, precision):
    """The vector-Jacobian product of one RK4 step with the rotational Raman response (the transpose
    of AddChiUPPE, rotations.cl:85-129, in the adjoint time pass) and ionization, against FP64 torch
    autograd of the same step (tests/torch_reference.py, which carries the oracle's raman_chi), at
    16, 4 and 1 transverse points per block of the adjoint time pass.  The rotator's polarizability
    difference is raised 100-fold (the Raman chi grows with its square) so that the Raman response
    carries a measurable part of the VJP.  Checked: the VJP (2e-4, the tolerance of the FP32
    transforms) and, separately, the Raman part of it, the difference between the VJPs with and
    without the rotator, on the GPU and in torch (2e-3 of its maximum)."""
    import torch
    from oracle import uppe_oracle as O
    from torch_reference import TorchStep
    rot = n2_rotator()
    rot.dalpha *= 100.0
    vd, g, dev, mat = _setup(shape, rot, precision=precision)
    zmat = 100.0
    mat.UpdateMaterial(zmat)
    orc = O.Oracle(vd)
    assert orc.rotator is rot
    orc.mat.update(zmat)
    ts = TorchStep(orc)
    redchi3 = vd["chi3"] / vd["density reference"]
    q0 = orc.g.kspace(vd["incoming wave"](g.w, g.x1, g.x2))
    rng = np.random.default_rng(13)
    lam = (rng.standard_normal(q0.shape) + 1j * rng.standard_normal(q0.shape)) * (np.abs(q0) + 1e-3 * np.abs(q0).max())
    z, dz = 50.0, vd["size"][2] / 400
    q0d = torch.from_numpy(q0.astype(np.complex64)).cuda()
    lamd = torch.from_numpy(lam.astype(np.complex64)).cuda()
    ref, gpu = {}, {}
    for with_raman in (True, False):
        ts.rotator = rot if with_raman else None
        x = torch.tensor(q0.real, requires_grad=True)
        y = torch.tensor(q0.imag, requires_grad=True)
        c3 = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
        q1 = ts.step(torch.complex(x, y), z, dz, c3)
        (torch.as_tensor(lam).conj() * q1).real.sum().backward()
        ref[with_raman] = (x.grad.numpy() + 1j * y.grad.numpy(), float(c3.grad))
        dev.set_rotator(rot if with_raman else None)
        out = dev.empty_field()
        dred = dev.adjoint_step(q0d, lamd, out, z, dz)
        gpu[with_raman] = (out.cpu().numpy(), dred)
    e = rel_err(gpu[True][0], ref[True][0])
    ed = abs(gpu[True][1] - ref[True][1]) / abs(ref[True][1])
    d_ref = ref[True][0] - ref[False][0]
    d_gpu = gpu[True][0].astype(np.complex128) - gpu[False][0]
    share = np.max(np.abs(d_ref)) / np.max(np.abs(ref[True][0]))
    er = rel_err(d_gpu, d_ref)
    print(shape, precision, f"vjp {e:.2e} dchi3 {ed:.2e}; Raman part {er:.2e} (share of the VJP {share:.2e})")
    assert e < 2e-4 and ed < 2e-4
    assert share > 5e-3 and er < 2e-3
    dev.close()
