"""The FP64 oracle against the reference's own outputs (fixtures made by tests/golden/make_golden.py,
which runs SeaRay's unmodified modules/uppe_kernel.py with its own OpenCL kernels on host cores)
and against the known answer of the reference's test/gaussian_test.py:110-154."""
import numpy as np
import pytest

import replay
from oracle import uppe_oracle as O


@pytest.mark.parametrize("name", replay.CASE_NAMES)
def test_oracle_matches_reference(name):
    vd, exp = replay.load_case(name)
    orc = O.Oracle(vd)
    A, J, chi, ne, dom4d = orc.track()
    for key, arr in (("A", A), ("J", J), ("chi", chi), ("ne", ne)):
        ref = exp[key]
        scale = max(np.max(np.abs(ref)), 1e-300)
        err = np.max(np.abs(arr[..., 1:] - ref)) / scale
        assert err < 1e-12, (key, err)
    assert np.array_equal(dom4d, exp["dom4d"])
    # same number of RHS evaluations in the last diagnostic interval (adaptive steps agree)
    n_ref = int(exp["evals_log"].split()[-4])
    assert 4 * orc.rk_steps[-1] == n_ref


def test_hankel_basis_matches_reference():
    d = np.load(replay.HERE / "hankel_bases.npz")
    for (Nr, dr, mmax, Nk) in ((32, 25.0, 0, 24), (16, 37.5, 2, 12)):
        key = f"Nr{Nr}_mmax{mmax}_Nk{Nk}"
        H, vals, lam = O.hankel_basis(Nr, dr, mmax, Nk)
        np.testing.assert_allclose(H, d[key + "_H"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(vals, d[key + "_vals"], rtol=1e-13, atol=0)
        np.testing.assert_allclose(lam, d[key + "_Lambda"], rtol=1e-15)


def test_plasma_density_serial_scan():
    """The vectorised scan equals the reference's serial loop (ionization.cl:144-154) bit for bit."""
    rng = np.random.default_rng(3)
    rate = rng.random((37, 3, 2)) * 1e-3
    ng = rng.random((3, 2))
    dt = 0.7
    got = O.plasma_density(rate, ng, dt)
    ne = rate.copy()
    for i in range(3):
        for j in range(2):
            prev = 0.0
            S = 0.0
            ne[-1, i, j] = 0.0
            for k in range(36, -1, -1):
                cur = ne[k, i, j]
                S += 0.5 * (cur + prev) * dt
                ne[k, i, j] = ng[i, j] * (1.0 - np.exp(-S))
                prev = cur
    assert np.array_equal(got, ne)


def _gaussian_case(N=(65, 128, 128, 3)):
    mks_length = 0.8e-6 / (2 * np.pi)
    cm = 100 * mks_length
    r00 = .01 / cm
    zR = 0.5 * r00 ** 2

    def incoming(w, x, y):
        f = lambda x, x0, dx: np.exp(-(x - x0) ** 2 / dx ** 2)
        return np.einsum("i,j,k", f(w, 1.0, 0.1), f(x, 0, r00), f(y, 0, r00))

    class Vacuum:
        def chi(self, w):
            return np.zeros(w.shape)

    vd = {"density reference": 1.0, "density lambda": lambda x, y, z, r2: np.ones(x.shape),
          "incoming wave": incoming, "frequency band": (0.0, 2.0), "nonlinear band": (0.0, 2.0),
          "wave grid": N, "wave coordinates": "cartesian", "dispersion inside": Vacuum(),
          "size": (36 * r00, 36 * r00, 4 * zR), "subcycles": 1, "minimum step": 1}
    return vd, r00


def check_gaussian_expansion(A, dom4d, r00):
    """The assertions of test/gaussian_test.py:133-155 (waist growth by 5 and 17 in area)."""
    dw = (dom4d[1] - dom4d[0]) / A.shape[0]
    dx = (dom4d[3] - dom4d[2]) / A.shape[1]
    dy = (dom4d[5] - dom4d[4]) / A.shape[2]
    w_nodes = np.linspace(dom4d[0] + 0.5 * dw, dom4d[1] - 0.5 * dw, A.shape[0])
    x_nodes = np.linspace(dom4d[2] + 0.5 * dx, dom4d[3] - 0.5 * dx, A.shape[1])
    y_nodes = np.linspace(dom4d[4] + 0.5 * dy, dom4d[5] - 0.5 * dy, A.shape[2])
    for k, f in ((1, 5), (2, 17)):
        xl = np.abs(A[32, :, 64, k])
        wfac = np.exp(-(w_nodes[32] - 1.0) ** 2 / .1 ** 2)
        yfac = np.exp(-y_nodes[64] ** 2 / r00 ** 2 / f)
        expct = wfac * yfac * np.exp(-x_nodes ** 2 / r00 ** 2 / f) / f ** 0.5
        assert np.allclose(xl, expct, .02, .01)


def test_oracle_gaussian_known_answer():
    vd, r00 = _gaussian_case()
    A, J, chi, ne, dom4d = O.track(vd)
    assert A.shape == (65, 128, 128, 3)
    check_gaussian_expansion(A, dom4d, r00)


def test_grid_checks():
    vd, _ = _gaussian_case((64, 128, 128, 3))
    with pytest.raises(ValueError, match="2\\*\\*n\\+1 w-nodes"):
        O.Oracle(vd)
    vd, _ = _gaussian_case((65, 100, 128, 3))
    with pytest.raises(ValueError, match="x-nodes"):
        O.Oracle(vd)


def test_torch_reference_step_matches_oracle():
    """The PyTorch FP64 step used to check the adjoint equals the oracle's RK4 step (with the
    rotational Raman response on cyl_raman)."""
    import torch
    from torch_reference import TorchStep
    for name in ("cart_ion", "cyl_kerr", "cyl_raman"):
        vd, _ = replay.load_case(name)
        orc = O.Oracle(vd)
        orc.mat.update(3000.0)
        g = orc.g
        q0 = g.kspace(vd["incoming wave"](g.w, g.x1, g.x2))
        z, dz = 1500.0, 2500.0
        q1t = TorchStep(orc).step(torch.tensor(q0), z, dz, vd.get("chi3", 0.0) / vd["density reference"]).numpy()
        cond = orc.conditioner[:, None, None]
        k1 = orc.load_source(q0, z)
        qf = q0 + dz / 6 * k1
        k2 = orc.load_source((q0 + dz / 2 * k1) * cond, z + dz / 2)
        qf = qf + dz / 3 * k2
        k3 = orc.load_source((q0 + dz / 2 * k2) * cond, z + dz / 2)
        qf = qf + dz / 3 * k3
        k4 = orc.load_source((q0 + dz * k3) * cond, z + dz)
        q1o = (qf + dz / 6 * k4) * cond
        assert np.max(np.abs(q1t - q1o)) / np.max(np.abs(q1o)) < 1e-13


@pytest.mark.parametrize("name", replay.PARAXIAL_CASE_NAMES)
def test_paraxial_oracle_matches_reference(name):
    """The paraxial oracle against the reference's own paraxial_kernel.track on the same inputs."""
    from oracle import paraxial_oracle as PO
    vd, exp = replay.load_case(name)
    orc = PO.ParaxialOracle(vd)
    A, J, chi, ne, dom4d = orc.track()
    for key, arr in (("A", A), ("J", J), ("chi", chi), ("ne", ne)):
        ref = exp[key]
        scale = max(np.max(np.abs(ref)), 1e-300)
        err = np.max(np.abs(arr[..., 1:] - ref)) / scale
        print(name, key, f"{err:.2e}")
        assert err < 1e-12, (key, err)
    assert np.array_equal(dom4d, exp["dom4d"])
    n_ref = int(exp["evals_log"].split()[-4])
    assert 4 * orc.rk_steps[-1] == n_ref
