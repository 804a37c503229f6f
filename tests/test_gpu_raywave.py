"""SeaRay's ray-started UPPE volume through the GB300 track(): rays -> boundary field -> RK4
propagation on the GPU -> ray relaunch, against the reference's own ``uppe_kernel.track`` on the
same rays (``tests/golden/raywave_track_cart.npz``, made by ``make_raywave.py``).

Bounds: the first plane is host FP64 arithmetic (1e-10); the propagated planes are held to the
bounds of tests/parity.py (field, fluence and spectrum 1e-5, J and chi 1e-4 of their maxima); the relaunched ray positions, times
and velocities follow from the rays and the medium alone (1e-12); the relaunched amplitude is
sampled from the GPU's last plane (1e-5 of its maximum), and so is the phase, compared where the
amplitude is above 1 % of its maximum (1e-4 rad)."""
import pathlib

import numpy as np
import pytest

from parity import check_field, field_errors, fmt

pytestmark = pytest.mark.gpu
GOLD = pathlib.Path(__file__).resolve().parent / "golden"


class StoredMedium:
    """chi at the grid's frequency nodes and the group velocity at the rays' frequencies, as the
    reference's SimpleAir gave them."""

    def __init__(self, w_nodes, chi_w, vg_w, vg_v):
        self.w_nodes, self.chi_w, self.vg_w, self.vg_v = w_nodes, chi_w, vg_w, vg_v

    def chi(self, w):
        assert np.allclose(w, self.w_nodes, rtol=0, atol=1e-12)
        return self.chi_w.copy()

    def GroupVelocityMagnitude(self, w):
        return np.interp(w, self.vg_w, self.vg_v)


@pytest.fixture(scope="module", autouse=True)
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import build
    build.build()
    return True


def rel(x, ref):
    return np.max(np.abs(x - ref)) / np.max(np.abs(ref))


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_track_from_rays_matches_reference(precision):
    from searay_gb300 import grid, uppe
    d = np.load(GOLD / "raywave_track_cart.npz")
    N = tuple(int(n) for n in d["N"])
    vd = {"wave grid": N, "wave coordinates": "cartesian", "frequency band": (0.0, 2.5), "nonlinear band": (0.0, 2.2),
          "size": (1200.0, 1200.0, 4000.0), "subcycles": 2, "minimum step": 1000.0, "chi3": 0.6,
          "density reference": 1.0, "window speed": 1.0, "ionizer": None,
          "density lambda": lambda x, y, z, r2: np.ones(x.shape), "full relaunch": False, "precision": precision}
    w = grid.VolumeGrid(vd).w
    vd["dispersion inside"] = StoredMedium(w, d["chi_w"], d["vg_w"], d["vg_v"])
    xp, eik, vg = d["xp"].copy(), d["eik"].copy(), d["vg"].copy()
    A, J, chi, ne, dom4d = uppe.track(None, xp, eik, vg, vd)
    assert np.allclose(dom4d, d["dom4d"], rtol=1e-12)
    errs = {"A0": rel(A[..., 0], d["A0"]), **field_errors(A[..., 1:], d["A"]), "J": rel(J[..., 1:], d["J"]),
            "chi": rel(chi[..., 1:], d["chiNL"])}
    amp_ref = d["eik_out"][:, 1]
    errs["amp"] = np.max(np.abs(eik[:, 1] - amp_ref)) / np.max(np.abs(amp_ref))
    strong = np.abs(amp_ref) > 0.01 * np.max(np.abs(amp_ref))
    dphi = np.angle(np.exp(1j * (eik[strong, 0] - d["eik_out"][strong, 0])))
    errs["phase"] = np.max(np.abs(dphi))
    print(precision, fmt(errs))
    assert errs["A0"] < 1e-10
    check_field(errs, False)
    assert errs["J"] < 1e-4 and errs["chi"] < 1e-4
    assert errs["amp"] < 1e-5 and errs["phase"] < 1e-4
    assert np.allclose(xp, d["xp_out"], rtol=1e-12, atol=1e-12)
    assert np.allclose(vg, d["vg_out"], rtol=1e-12, atol=1e-12)
    assert np.max(np.abs(ne[..., 1:])) == 0


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_paraxial_track_from_rays_matches_reference(precision):
    """The reference's ray-started paraxial volume (raywave_paraxial_cart.npz: envelope band
    0.5-1.5, 64 x 16 x 16, Kerr) through searay_gb300.paraxial.track, same bounds as above."""
    from searay_gb300 import grid, paraxial
    d = np.load(GOLD / "raywave_paraxial_cart.npz")
    N = tuple(int(n) for n in d["N"])
    vd = {"wave grid": N, "wave coordinates": "cartesian", "frequency band": tuple(d["band"]),
          "size": (1200.0, 1200.0, 4000.0), "subcycles": 2, "chi3": 0.6, "density reference": 1.0,
          "window speed": 1.0, "ionizer": None, "density lambda": lambda x, y, z, r2: np.ones(x.shape),
          "full relaunch": False, "precision": precision}
    w = grid.VolumeGrid(vd).w
    vd["dispersion inside"] = StoredMedium(w, d["chi_w"], d["vg_w"], d["vg_v"])
    xp, eik, vg = d["xp"].copy(), d["eik"].copy(), d["vg"].copy()
    A, J, chi, ne, dom4d = paraxial.track(None, xp, eik, vg, vd)
    assert np.allclose(dom4d, d["dom4d"], rtol=1e-12)
    errs = {"A0": rel(A[..., 0], d["A0"]), **field_errors(A[..., 1:], d["A"]), "J": rel(J[..., 1:], d["J"]),
            "chi": rel(chi[..., 1:], d["chiNL"])}
    amp_ref = d["eik_out"][:, 1]
    errs["amp"] = np.max(np.abs(eik[:, 1] - amp_ref)) / np.max(np.abs(amp_ref))
    strong = np.abs(amp_ref) > 0.01 * np.max(np.abs(amp_ref))
    dphi = np.angle(np.exp(1j * (eik[strong, 0] - d["eik_out"][strong, 0])))
    errs["phase"] = np.max(np.abs(dphi))
    print("paraxial", precision, fmt(errs))
    assert errs["A0"] < 1e-10
    check_field(errs, False)
    assert errs["J"] < 1e-4 and errs["chi"] < 1e-4
    assert errs["amp"] < 1e-5 and errs["phase"] < 1e-4
    assert np.allclose(xp, d["xp_out"], rtol=1e-12, atol=1e-12)
    assert np.allclose(vg, d["vg_out"], rtol=1e-12, atol=1e-12)
    assert np.max(np.abs(ne[..., 1:])) == 0
