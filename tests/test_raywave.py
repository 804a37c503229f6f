"""Ray <-> wave coupling (searay_gb300/raywave.py) against SeaRay's own field tools.

Fixtures ``tests/golden/raywave_*.npz`` hold seeded synthetic ray sets on three field grids
(Cartesian, cylindrical, cylindrical with azimuthal modes) and what the reference's
``caustic_tools`` made of them (``make_raywave.py``): ``GetBoundaryFields``, ``RelaunchRays`` and
``RelaunchRays1``.  The host restatement runs the same FP64 algorithms, so the bound is 1e-9
relative (interpolation libraries are the same; only the order of a few sums differs)."""
import pathlib

import numpy as np
import pytest

from searay_gb300 import dispersion, grid, raywave

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
NAMES = ("cart", "cyl", "cyl_az")


class TableMedium:
    """Group velocity at the stored ray frequencies (the reference medium's own values)."""

    def __init__(self, w, v):
        self.w, self.v = w, v

    def GroupVelocityMagnitude(self, w):
        return np.interp(w, self.w, self.v)


def _load(name):
    d = np.load(GOLD / f"raywave_{name}.npz")
    N = tuple(int(n) for n in d["N"])
    vd = {"wave grid": N, "wave coordinates": "cartesian" if int(d["modes"]) < 0 else "cylindrical",
          "frequency band": tuple(d["band"]), "size": tuple(d["size"])}
    if int(d["modes"]) > 0:
        vd["radial modes"] = int(d["modes"])
    return d, raywave.FieldGrid(grid.VolumeGrid(vd))


def close(a, b, tol=1e-9):
    s = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) / s < tol


@pytest.mark.parametrize("name", NAMES)
def test_boundary_fields(name):
    d, fg = _load(name)
    bf = raywave.boundary_fields(fg, d["xp"][:, 0, :], d["eik"], 1)
    assert bf.shape == d["bf"].shape
    assert close(bf, d["bf"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("full", [False, True])
def test_relaunch(name, full):
    d, fg = _load(name)
    xp, eik, vg = d["xp"].copy(), d["eik"].copy(), d["vg"].copy()
    fn = raywave.relaunch_rays_full if full else raywave.relaunch_rays
    fn(fg, xp, eik, vg, d["a"], float(d["L"]), TableMedium(d["vg_w"], d["vg_v"]))
    tag = "f" if full else "s"
    for got, ref in ((xp, d["xp_" + tag]), (eik, d["eik_" + tag]), (vg, d["vg_" + tag])):
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        assert close(np.nan_to_num(got), np.nan_to_num(ref))


def test_relaunch_moves_rays():
    """The relaunch changes the rays on the grid and leaves the others alone."""
    d, fg = _load("cart")
    xp = d["xp"].copy()
    raywave.relaunch_rays(fg, xp, d["eik"].copy(), d["vg"].copy(), d["a"], float(d["L"]),
                          TableMedium(d["vg_w"], d["vg_v"]))
    moved = np.any(xp != d["xp"], axis=(1, 2))
    hit = fg.clip_rays(d["xp"])
    assert np.array_equal(np.where(moved)[0], hit) and 0 < hit.shape[0] < xp.shape[0]


def test_simple_air_group_velocity_matches_reference():
    d, _ = _load("cart")
    air = dispersion.SimpleAir(0.8e-6 / (2 * np.pi))
    assert np.allclose(air.GroupVelocityMagnitude(d["vg_w"][1:]), d["vg_v"][1:], rtol=1e-12, atol=0)


def test_missing_frequency_bin_raises():
    d, fg = _load("cart")
    xps = d["xp"][:, 0, :]
    keep = xps[:, 4] > 0.5  # no rays in the low bins
    with pytest.raises(ValueError, match="no rays found in frequency bin"):
        raywave.boundary_fields(fg, xps[keep], d["eik"][keep], 1)


def _paraxial_grid(d):
    vd = {"wave grid": tuple(int(n) for n in d["N"]), "wave coordinates": "cartesian",
          "frequency band": tuple(d["band"]), "size": (1200.0, 1200.0, 4000.0)}
    return raywave.FieldGrid(grid.VolumeGrid(vd))


def test_paraxial_boundary_field_and_relaunch():
    """The host ray <-> wave steps of the reference's ray-started paraxial volume (envelope band
    0.5-1.5, raywave_paraxial_cart.npz): the first plane from the rays, and the relaunch from the
    reference's own last plane."""
    d = np.load(GOLD / "raywave_paraxial_cart.npz")
    fg = _paraxial_grid(d)
    bf = raywave.boundary_fields(fg, d["xp"][:, 0, :], d["eik"], 1)
    assert close(bf, d["A0"], 1e-10)
    xp, eik, vg = d["xp"].copy(), d["eik"].copy(), d["vg"].copy()
    raywave.relaunch_rays(fg, xp, eik, vg, d["A"][..., -1], 4000.0, TableMedium(d["vg_w"], d["vg_v"]))
    for got, ref in ((xp, d["xp_out"]), (eik, d["eik_out"]), (vg, d["vg_out"])):
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        assert close(np.nan_to_num(got), np.nan_to_num(ref))
