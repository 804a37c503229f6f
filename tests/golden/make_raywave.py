"""Generate the ray <-> wave coupling fixtures (``raywave_*.npz``) from the reference itself.

For three field grids (Cartesian 33x16x16, cylindrical 33x32x1, cylindrical with azimuthal modes
33x16x4) it runs SeaRay's own ``caustic_tools`` field tools on seeded synthetic rays:
``GetBoundaryFields`` (component 1), ``RelaunchRays`` and ``RelaunchRays1``, and stores inputs and
outputs.  It also runs the reference's whole ``uppe_kernel.track`` from rays (no ``incoming
wave``) on a small Cartesian Kerr volume (``raywave_track_cart.npz``), and its paraxial
``paraxial_kernel.track`` on such a volume with an envelope band (``raywave_paraxial_cart.npz``).

The reference's cylindrical ``RelaunchRays1`` calls ``scipy.integrate.cumtrapz``, which SciPy has
since renamed ``cumulative_trapezoid`` (same trapezoid rule); the name is supplied before the call.
Needs the reference source tree, given by ``--reference PATH`` (or ``SEARAY_REF``)::

    python tests/golden/make_raywave.py --reference PATH [paraxial]
"""
import pathlib
import sys

import numpy as np
import scipy.integrate

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

from oracle.refshim import runner  # noqa: E402
import cases  # noqa: E402

if not hasattr(scipy.integrate, "cumtrapz"):
    scipy.integrate.cumtrapz = scipy.integrate.cumulative_trapezoid

BAND = (0.0, 2.5)
TOOLS = {
    "cart": dict(N=(33, 16, 16, 2), size=(1200.0, 1200.0, 1.0e4), modes=None),
    "cyl": dict(N=(33, 32, 1, 2), size=(1200.0, 1200.0, 1.0e4), modes=24),
    "cyl_az": dict(N=(33, 16, 4, 2), size=(1200.0, 1200.0, 1.0e4), modes=16),
}


def make_rays(wn, cartesian, half_width, rng, per_bin=40, nudge_first=True):
    """Bundles of 4 rays: primaries at every frequency node (the first node nudged above w = 0 when
    nudge_first), spread over the grid and a little beyond; satellites displaced by 0.5 in x, y, x+y."""
    dw = wn[1] - wn[0]
    prim = []
    for i, w in enumerate(wn):
        wv = w if (i > 0 or not nudge_first) else 0.25 * dw
        if cartesian:
            r = 1.03 * half_width
            corners = np.array([[-r, -r], [-r, r], [r, -r], [r, r]])
            pts = np.concatenate((corners, rng.uniform(-r, r, (per_bin - 4, 2))))
        else:
            rho = rng.uniform(0.0, 1.05 * half_width, per_bin)
            phi = rng.uniform(-np.pi, np.pi, per_bin)
            pts = np.stack((rho * np.cos(phi), rho * np.sin(phi)), axis=-1)
        for x, y in pts:
            prim.append((wv, x, y))
    prim = np.array(prim)
    nb = prim.shape[0]
    xp = np.zeros((nb, 4, 8))
    off = np.array([[0, 0], [0.5, 0], [0, 0.5], [0.5, 0.5]])
    for r in range(4):
        xp[:, r, 1] = prim[:, 1] + off[r, 0]
        xp[:, r, 2] = prim[:, 2] + off[r, 1]
    xp[..., 4] = prim[:, :1]
    xp[..., 0] = 5.0 + 0.01 * xp[..., 1]
    xp[..., 7] = xp[..., 4]
    x, y, w = prim[:, 1], prim[:, 2], prim[:, 0]
    eik = np.zeros((nb, 4))
    r2 = x ** 2 + y ** 2
    eik[:, 0] = w * xp[:, 0, 0] + 2e-5 * w * r2
    eik[:, 1] = np.exp(-r2 / 400.0 ** 2) * np.exp(-((w - 1.0) / 0.4) ** 2)
    eik[:, 2] = 0.3 * eik[:, 1]
    vg = np.zeros((nb, 4, 4))
    return xp, eik, vg


def wave_on_grid(wn, xn, yn, cartesian):
    if cartesian:
        X, Y = np.meshgrid(xn, yn, indexing="ij")
    else:
        R, P = np.meshgrid(xn, yn, indexing="ij")
        X, Y = R * np.cos(P), R * np.sin(P)
    r2 = X ** 2 + Y ** 2
    w = wn[:, None, None]
    return (np.exp(-r2 / 350.0 ** 2)[None] * np.exp(-((w - 1.0) / 0.4) ** 2)
            * np.exp(1j * (3e-5 * w * r2[None] + 0.002 * X[None])))


def tool_fixture(name, m, cl, rng):
    t = TOOLS[name]
    ct = m["caustic_tools"]
    cart = t["modes"] is None
    if cart:
        tool = ct.FourierTool(t["N"], BAND, (0, 0, 0), t["size"], cl)
    else:
        tool = ct.BesselBeamTool(t["N"], BAND, (0, 0, 0), t["size"], cl, t["modes"])
    wn, xn, yn, _ = tool.GetGridInfo()
    xp, eik, vg = make_rays(wn, cart, 0.5 * t["size"][0], rng)
    bf = tool.GetBoundaryFields(xp[:, 0, :], eik, 1)
    a = wave_on_grid(wn, xn, yn, cart)
    L = t["size"][2]
    medium = m["dispersion"].SimpleAir(cases.MKS_LENGTH)
    out = {}
    for tag, fn in (("s", tool.RelaunchRays), ("f", tool.RelaunchRays1)):
        x2, e2, v2 = xp.copy(), eik.copy(), vg.copy()
        fn(x2, e2, v2, a, L, medium)
        out["xp_" + tag], out["eik_" + tag], out["vg_" + tag] = x2, e2, v2
    wu = np.unique(xp[..., 4])
    np.savez_compressed(HERE / f"raywave_{name}.npz", N=np.array(t["N"]), band=np.array(BAND),
                        size=np.array(t["size"]), modes=np.array(-1 if cart else t["modes"]), xp=xp, eik=eik, vg=vg,
                        a=a, L=np.array(L), bf=bf, vg_w=wu, vg_v=medium.GroupVelocityMagnitude(wu), **out)
    print(name, "bundles", xp.shape[0], "max |bf|", np.abs(bf).max())


def track_fixture(m, cl, rng):
    medium = m["dispersion"].SimpleAir(cases.MKS_LENGTH)
    N = (65, 16, 16, 2)
    vd = {"wave grid": N, "wave coordinates": "cartesian", "frequency band": BAND, "nonlinear band": (0.0, 2.2),
          "size": (1200.0, 1200.0, 4000.0), "subcycles": 2, "minimum step": 1000.0, "chi3": 0.6,
          "density reference": 1.0, "window speed": 1.0, "dispersion inside": medium, "ionizer": None,
          "density lambda": lambda x, y, z, r2: np.ones(x.shape), "full relaunch": False}
    ft = m["caustic_tools"].FourierTool(N, BAND, (0, 0, 0), vd["size"], cl)
    wn = ft.GetGridInfo()[0]
    xp, eik, vg = make_rays(wn, True, 600.0, rng, per_bin=32)
    eik[:, 1:3] *= 0.02  # field strength of the Kerr cases
    A, J, chi, ne, dom4d, xp2, eik2, vg2 = runner.reference_track_rays(vd, xp, eik, vg)
    wu = np.unique(xp[..., 4])
    np.savez_compressed(HERE / "raywave_track_cart.npz", N=np.array(N), xp=xp, eik=eik, vg=vg, chi_w=medium.chi(wn),
                        A=A[..., 1:], J=J[..., 1:], chiNL=chi[..., 1:], ne=ne[..., 1:], A0=A[..., 0], dom4d=dom4d,
                        xp_out=xp2, eik_out=eik2, vg_out=vg2, vg_w=wu, vg_v=medium.GroupVelocityMagnitude(wu))
    print("track from rays: max |A0|", np.abs(A[..., 0]).max(), "max |A|", np.abs(A[..., 1]).max())


def paraxial_fixture(m, cl, rng):
    medium = m["dispersion"].SimpleAir(cases.MKS_LENGTH)
    N = (64, 16, 16, 2)
    band = (0.5, 1.5)
    vd = {"wave grid": N, "wave coordinates": "cartesian", "frequency band": band,
          "size": (1200.0, 1200.0, 4000.0), "subcycles": 2, "chi3": 0.6,
          "density reference": 1.0, "window speed": 1.0, "dispersion inside": medium, "ionizer": None,
          "density lambda": lambda x, y, z, r2: np.ones(x.shape), "full relaunch": False}
    ft = m["caustic_tools"].FourierTool(N, band, (0, 0, 0), vd["size"], cl)
    wn = ft.GetGridInfo()[0]
    xp, eik, vg = make_rays(wn, True, 600.0, rng, per_bin=32, nudge_first=False)
    eik[:, 1:3] *= 0.02
    A, J, chi, ne, dom4d, xp2, eik2, vg2 = runner.reference_paraxial_rays(vd, xp, eik, vg)
    wu = np.unique(xp[..., 4])
    np.savez_compressed(HERE / "raywave_paraxial_cart.npz", N=np.array(N), band=np.array(band), xp=xp, eik=eik,
                        vg=vg, chi_w=medium.chi(wn), A=A[..., 1:], J=J[..., 1:], chiNL=chi[..., 1:], ne=ne[..., 1:],
                        A0=A[..., 0], dom4d=dom4d, xp_out=xp2, eik_out=eik2, vg_out=vg2, vg_w=wu,
                        vg_v=medium.GroupVelocityMagnitude(wu))
    print("paraxial track from rays: max |A0|", np.abs(A[..., 0]).max(), "max |A|", np.abs(A[..., 1]).max())


def main(names=None):
    if not runner.available():
        raise SystemExit("reference tree not found")
    cl = runner.cl_refs()
    m = runner.modules()
    rng = np.random.default_rng(7)
    if names:  # only the named fixtures ("paraxial"), with their own seed
        if "paraxial" in names:
            paraxial_fixture(m, cl, np.random.default_rng(11))
        return
    for name in TOOLS:
        tool_fixture(name, m, cl, rng)
    track_fixture(m, cl, rng)
    paraxial_fixture(m, cl, np.random.default_rng(11))


def _args(argv):
    """Strip ``--reference PATH`` from the arguments and point the reference runner at PATH."""
    argv = list(argv)
    if "--reference" in argv:
        i = argv.index("--reference")
        runner.set_reference(argv[i + 1])
        del argv[i:i + 2]
    return argv


if __name__ == "__main__":
    main(_args(sys.argv[1:]))
