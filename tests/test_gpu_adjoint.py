"""The hand-written adjoint of the UPPE step (through the C ABI) against a plain-PyTorch FP64
autograd of the same step (tests/torch_reference.py), and gradients of a loss through the
checkpointed torch.autograd.Function against central finite differences."""
import numpy as np
import pytest

import replay

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


def _setup(name, precision, zmat):
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
    mat.UpdateMaterial(zmat)
    orc = O.Oracle(vd)
    orc.mat.update(zmat)
    return vd, g, dev, orc


# tolerance of the VJP: FP32 transforms 2e-4, the tensor-core Hankel transform of the mixed form 2e-3
@pytest.mark.parametrize("name,precision", [("cart_ion", "mixed"), ("cart_series", "fp32"), ("cyl_kerr", "fp32"),
                                            ("cyl_kerr", "mixed"), ("cyl_raman", "fp32"), ("cyl_raman", "mixed")])
def test_vjp_of_rk4_step_matches_torch_fp64(name, precision):
    import torch
    from torch_reference import TorchStep
    vd, g, dev, orc = _setup(name, precision, 3000.0)
    redchi3 = vd.get("chi3", 0.0) / vd["density reference"]
    ts = TorchStep(orc)
    q0 = orc.g.kspace(vd["incoming wave"](g.w, g.x1, g.x2))
    rng = np.random.default_rng(7)
    lam = (rng.standard_normal(q0.shape) + 1j * rng.standard_normal(q0.shape)) * (np.abs(q0) + 1e-3 * np.abs(q0).max())
    z, dz = 1500.0, 2500.0
    # torch FP64 autograd of the same step
    x = torch.tensor(q0.real, requires_grad=True)
    y = torch.tensor(q0.imag, requires_grad=True)
    c3 = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
    q1 = ts.step(torch.complex(x, y), z, dz, c3)
    L = (torch.as_tensor(lam).conj() * q1).real.sum()
    L.backward()
    g_ref = x.grad.numpy() + 1j * y.grad.numpy()
    dred_ref = float(c3.grad)
    # the CUDA adjoint
    q0d = torch.from_numpy(q0.astype(np.complex64)).cuda()
    lamd = torch.from_numpy(lam.astype(np.complex64)).cuda()
    out = dev.empty_field()
    dred = dev.adjoint_step(q0d, lamd, out, z, dz)
    g_gpu = out.cpu().numpy()
    e = rel_err(g_gpu, g_ref)
    ed = abs(dred - dred_ref) / abs(dred_ref)
    # the forward step itself
    dev.set_field(q0d)
    dev.rk4_step(z, dz, 0.0, dz)
    qd = dev.empty_field()
    dev.get_field(qd)
    ef = rel_err(qd.cpu().numpy(), q1.detach().numpy())
    print(name, precision, f"vjp {e:.2e} dchi3 {ed:.2e} forward {ef:.2e}")
    tol = 2e-3 if (precision == "mixed" and not g.cartesian) else 2e-4
    assert e < tol and ed < tol
    dev.close()


@pytest.mark.parametrize("name", ["cart_ion", "cyl_kerr"])
def test_gradient_matches_finite_differences(name):
    """L = the on-axis spectral energy in the self-phase-modulation wing 1.15 < w < 1.4 after 6 steps
    (FP64 accumulation); gradient with respect to a Legendre spectral-phase coefficient and chi3,
    against central differences."""
    import torch
    from searay_gb300 import adjoint
    vd, g, dev, orc = _setup(name, "fp32", 0.0)
    redchi3 = vd.get("chi3", 0.0) / vd["density reference"]
    a_base = vd["incoming wave"](g.w, g.x1, g.x2)
    xi = 2 * (g.w - g.w[0]) / (g.w[-1] - g.w[0]) - 1
    P2 = torch.tensor(0.5 * (3 * xi ** 2 - 1))[:, None, None]
    base = torch.tensor(a_base)
    band = (g.w > 1.15) & (g.w < 1.4)
    ax = (0, 0) if not g.cartesian else (g.N[1] // 2, g.N[2] // 2)
    nsteps, dz = 6, 1500.0

    def loss(theta, chi):
        a0 = (base * torch.exp(1j * theta * P2)).to(torch.complex64).cuda()
        A = adjoint.propagate(dev, a0, chi, dz, nsteps, checkpoint_every=4)
        sel = A[torch.as_tensor(band), ax[0], ax[1]].to(torch.complex128)
        return (sel.abs() ** 2).sum()

    theta = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    chi = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
    L = loss(theta, chi)
    L.backward()
    ht, hc = 1e-2, 1e-2 * redchi3
    with torch.no_grad():
        fd_t = (loss(theta + ht, chi) - loss(theta - ht, chi)).item() / (2 * ht)
        fd_c = (loss(theta, chi + hc) - loss(theta, chi - hc)).item() / (2 * hc)
    et = abs(theta.grad.item() - fd_t) / abs(fd_t)
    ec = abs(chi.grad.item() - fd_c) / abs(fd_c)
    print(name, f"dtheta {theta.grad.item():.6e} fd {fd_t:.6e} ({et:.1e}); dchi3 {chi.grad.item():.6e} fd {fd_c:.6e} ({ec:.1e})")
    assert et < 2e-2 and ec < 2e-2
    dev.close()


@pytest.mark.parametrize("n0", [513, 1025, 2049])
def test_vjp_at_benchmark_time_axes(n0):
    """The adjoint time pass with compile-time sizes (2048 complex elements per block: 4, 2 and 1
    transverse points per block at N0 = 513, 1025, 2049) in one VJP of an RK4 step on a 16 x 16
    Cartesian grid with the filamentation medium and an ionizing pulse, against the FP64 torch
    autograd.  Bound: the VJP tolerance of the FP32 transforms, 2e-4."""
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe, workloads
    from torch_reference import TorchStep
    vd = workloads.cart_filament_128(steps=400, n_perp=16)
    vd["wave grid"] = (n0, 16, 16, 2)
    vd["frequency band"] = (0.0, 4.0 * (n0 - 1) / 512)
    vd["nonlinear band"] = (0.0, 3.5 * (n0 - 1) / 512)
    wave = vd["incoming wave"]
    vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, ionization.RateCoefficients(vd["ionizer"]), "mixed")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    zmat = 100.0
    mat.UpdateMaterial(zmat)
    orc = O.Oracle(vd)
    orc.mat.update(zmat)
    redchi3 = vd["chi3"] / vd["density reference"]
    ts = TorchStep(orc)
    q0 = orc.g.kspace(vd["incoming wave"](g.w, g.x1, g.x2))
    rng = np.random.default_rng(11)
    lam = (rng.standard_normal(q0.shape) + 1j * rng.standard_normal(q0.shape)) * (np.abs(q0) + 1e-3 * np.abs(q0).max())
    z, dz = 50.0, vd["size"][2] / 400
    x = torch.tensor(q0.real, requires_grad=True)
    y = torch.tensor(q0.imag, requires_grad=True)
    c3 = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
    q1 = ts.step(torch.complex(x, y), z, dz, c3)
    L = (torch.as_tensor(lam).conj() * q1).real.sum()
    L.backward()
    g_ref = x.grad.numpy() + 1j * y.grad.numpy()
    dred_ref = float(c3.grad)
    out = dev.empty_field()
    dred = dev.adjoint_step(torch.from_numpy(q0.astype(np.complex64)).cuda(),
                            torch.from_numpy(lam.astype(np.complex64)).cuda(), out, z, dz)
    e = rel_err(out.cpu().numpy(), g_ref)
    ed = abs(dred - dred_ref) / abs(dred_ref)
    print(n0, f"vjp {e:.2e} dchi3 {ed:.2e}")
    assert e < 2e-4 and ed < 2e-4
    dev.close()


@pytest.mark.parametrize("case", ["129x16x16", "33x256x128", "cart_series", "cyl_kerr"])
def test_kept_step_matches_recompute(case):
    """rk4_step_keep + adjoint_step_kept (the stage fields kept by the forward step) against rk4_step
    + adjoint_step (the stage states recomputed): the same step result and the same VJP, on the
    register-resident (16 x 16) and big-slice (256 x 128) passes with ionization and the slices above
    the nonlinear cut, on the generic Cartesian slices (8 x 16) and on a cylindrical grid (the
    tensor-core transforms).  Bound 1e-6 relative (the same kernels; only the order of launches
    differs)."""
    import torch
    from oracle import uppe_oracle as O
    from searay_gb300 import grid, ionization, uppe, workloads
    if "x" in case:
        shape = tuple(int(v) for v in case.split("x"))
        vd = workloads.cart_filament_128(steps=400, n_perp=shape[1])
        vd["wave grid"] = (shape[0], shape[1], shape[2], 2)
        wave = vd["incoming wave"]
        vd["incoming wave"] = lambda w, x1, x2: 3.0 * wave(w, x1, x2)
    else:
        vd, _ = replay.load_case(case)
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") else None
    dev = uppe.DeviceGrid(g, vd, rates, "mixed")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                        vd.get("window speed", 1.0), vd["density lambda"])
    mat.UpdateMaterial(100.0)
    q0 = O.Oracle(vd).g.kspace(vd["incoming wave"](g.w, g.x1, g.x2))
    rng = np.random.default_rng(5)
    lam = (rng.standard_normal(q0.shape) + 1j * rng.standard_normal(q0.shape)) * (np.abs(q0) + 1e-3 * np.abs(q0).max())
    q0d = torch.from_numpy(q0.astype(np.complex64)).cuda()
    lamd = torch.from_numpy(lam.astype(np.complex64)).cuda()
    z, dz = 50.0, 1500.0
    dev.set_field(q0d)
    dev.rk4_step(z, dz, 0.0, dz)
    q1 = dev.empty_field()
    dev.get_field(q1)
    g_rec = dev.empty_field()
    d_rec = dev.adjoint_step(q0d, lamd, g_rec, z, dz)
    dev.set_field(q0d)
    dev.rk4_step_keep(z, dz)
    q1k = dev.empty_field()
    dev.get_field(q1k)
    g_kept = dev.empty_field()
    d_kept = dev.adjoint_step_kept(lamd, g_kept)
    eq = rel_err(q1k.cpu().numpy(), q1.cpu().numpy())
    eg = rel_err(g_kept.cpu().numpy(), g_rec.cpu().numpy())
    ed = abs(d_kept - d_rec) / abs(d_rec)
    print(case, f"step {eq:.1e} vjp {eg:.1e} dchi3 {ed:.1e}")
    assert eq < 1e-6 and eg < 1e-6 and ed < 1e-6
    # the kept fields belong to one step: a plain step ends them
    dev.rk4_step(z + dz, dz, 0.0, dz)
    with pytest.raises(RuntimeError):
        dev.adjoint_step_kept(lamd, g_kept)
    dev.close()


def test_legendre_phase_gradient_1025x256():
    """The gradient of the adjoint workload (config 4): 1025 x 256 cylindrical, the config-1 beam,
    the on-axis spectral energy in the 700-750 nm band as the loss, 64 Legendre spectral-phase
    coefficients ~ N(0, 0.1) rad (numpy default_rng(1)) and chi3 as the parameters, checkpoints
    every 20 steps.  100 steps of 0.5 mm (5 cm: the beam of twice the critical power collapses near
    8.7 cm, so 200 such steps overflow), in the plain FP32 form.  The FP32 loss carries rounding
    noise of about 1e-6 of itself, and the loss moves little with any one coefficient (the largest
    component of the gradient is about 6e-3 of the loss per radian), so the central differences take
    h = 1e-2 rad (at h = 1e-4 they are noise: they grow as 1/h) on the two coefficients with the
    largest gradient, and h = 1e-4 of chi3 for chi3; 3e-2 relative.  The gradient of the constant
    (global-phase) coefficient, which the loss does not depend on, stays below 2e-2 of the largest
    component (a cancellation over 1025 frequencies in FP32)."""
    import torch
    from numpy.polynomial import legendre
    from searay_gb300 import adjoint, grid, uppe, workloads
    vd = workloads.cyl_adjoint_256()
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, None, "fp32")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd["chi3"], vd["density reference"],
                        vd["window speed"], vd["density lambda"])
    mat.UpdateMaterial(0.0)
    redchi3 = vd["chi3"] / vd["density reference"]
    dz = vd["size"][2] / vd["subcycles"]
    nsteps = 100
    xi = 2 * (g.w - g.w[0]) / (g.w[-1] - g.w[0]) - 1
    Pl = torch.tensor(legendre.legvander(xi, 63))  # (N0, 64)
    base = torch.tensor(vd["incoming wave"](g.w, g.x1, g.x2))
    band = torch.as_tensor((g.w > 0.8 / 0.75) & (g.w < 0.8 / 0.70))
    c0 = torch.tensor(np.random.default_rng(1).normal(0.0, 0.1, 64))

    def loss(c, chi3):
        phase = (Pl @ c)[:, None, None]
        a0 = (base * torch.exp(1j * phase)).to(torch.complex64).cuda()
        A = adjoint.propagate(dev, a0, chi3, dz, nsteps, checkpoint_every=20)
        return (A[band, 0, 0].to(torch.complex128).abs() ** 2).sum()

    c = c0.clone().requires_grad_(True)
    x3 = torch.tensor(redchi3, dtype=torch.float64, requires_grad=True)
    L = loss(c, x3)
    L.backward()
    gc, g3 = c.grad.numpy(), float(x3.grad)
    top = [int(n) for n in np.argsort(-np.abs(gc[1:]))[:2] + 1]
    h = 1e-2
    errs = {}
    with torch.no_grad():
        for n in top:
            e = torch.zeros(64, dtype=torch.float64)
            e[n] = h
            fd = (loss(c0 + e, x3.detach()) - loss(c0 - e, x3.detach())).item() / (2 * h)
            errs[f"c{n}"] = (gc[n], fd)
        hc = 1e-4 * redchi3
        fd3 = (loss(c0, torch.tensor(redchi3 + hc)) - loss(c0, torch.tensor(redchi3 - hc))).item() / (2 * hc)
        errs["chi3"] = (g3, fd3)
    print(f"L {L.item():.4e}", {k: f"{a:.6e} fd {b:.6e}" for k, (a, b) in errs.items()},
          f"|g0|/max {abs(gc[0]) / np.abs(gc).max():.1e}")
    for k, (a, b) in errs.items():
        assert abs(a - b) < 3e-2 * abs(b), (k, a, b)
    assert abs(gc[0]) < 2e-2 * np.abs(gc).max()
    dev.close()


def test_transverse_phase_gradient_large_filament():
    """The gradient of the large-filament workload's forward+adjoint objective: 1025 x 256 x 256
    Cartesian, 800 nm 40 fs at 10 critical powers in air with Kerr, O2 tunnelling and the plasma
    current, mixed precision, checkpoints every 50 steps; the loss is the energy of the central
    32 x 32 points in the band 0.9 < w < 1.1 after 100 steps (1 cm of the 10 cm), and the parameter
    the 256 x 256 input transverse phase phi(x, y) (a0 = a e^{i phi}).  The gradient is checked along
    two smooth directions of phi against central differences of the FP32 forward: centred Gaussian
    bumps of the beam's radius and of half of it (weak lenses of two widths), h = 0.05 rad, within
    3e-2.  The loss responds to a lens of 1 rad by a few percent over 1 cm (the Rayleigh length is
    about 35 cm), so h is large against the FP32 rounding noise (about 1e-6 of the loss) and small
    enough that the O(h^2) error stays below 1e-2."""
    import torch
    from searay_gb300 import adjoint, grid, ionization, uppe, workloads
    vd = workloads.cart_filament_256()
    g = grid.VolumeGrid(vd)
    dev = uppe.DeviceGrid(g, vd, ionization.RateCoefficients(vd["ionizer"]), "mixed")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, "cartesian", None, chi, vd["chi3"], vd["density reference"], vd["window speed"],
                        vd["density lambda"])
    dz = vd["size"][2] / vd["subcycles"]
    mat.UpdateMaterial(0.5 * dz)
    redchi3 = vd["chi3"] / vd["density reference"]
    nsteps = 100
    base = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
    band = torch.as_tensor((g.w > 0.9) & (g.w < 1.1)).cuda()
    c = g.N[1] // 2

    def loss(phi):
        a0 = base * torch.exp(1j * phi.to(torch.float32))[None]
        A = adjoint.propagate(dev, a0, redchi3, dz, nsteps, checkpoint_every=50)
        sel = A[band][:, c - 16:c + 16, c - 16:c + 16].to(torch.complex128)
        return (sel.abs() ** 2).sum()

    phi = torch.zeros(g.N[1], g.N[2], dtype=torch.float64, device="cuda", requires_grad=True)
    L = loss(phi)
    L.backward()
    grad = phi.grad.detach()
    X, Y = np.meshgrid(g.x1, g.x2, indexing="ij")
    r0 = 0.3e-3 / (0.8e-6 / (2 * np.pi))  # the beam radius, simulation units
    gauss = np.exp(-(X ** 2 + Y ** 2) / r0 ** 2)
    dirs = {"lens": gauss, "narrow lens": np.exp(-4 * (X ** 2 + Y ** 2) / r0 ** 2)}
    h = 0.05
    res = {}
    with torch.no_grad():
        for name, u in dirs.items():
            ut = torch.from_numpy(u).cuda()
            ad = float((grad * ut).sum())
            fd = (loss(h * ut) - loss(-h * ut)).item() / (2 * h)
            res[name] = (ad, fd)
    print(f"L {L.item():.6e}", {k: f"adjoint {a:.6e} fd {b:.6e}" for k, (a, b) in res.items()})
    for k, (a, b) in res.items():
        assert abs(b) > 1e-3 * L.item(), (k, b)  # the direction moves the loss measurably
        assert abs(a - b) < 3e-2 * abs(b), (k, a, b)
    dev.close()
