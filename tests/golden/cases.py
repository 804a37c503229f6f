"""Parity cases for the UPPE z-step: small volumes whose reference outputs are stored as fixtures.

Each case is a SeaRay volume input dictionary (the keys ``uppe_kernel.track`` reads,
``modules/uppe_kernel.py:341-403``) described by plain numbers, so the same case can be built from
the reference's own dispersion/ionization classes (when generating fixtures) or replayed from the
stored arrays (at test time, where the reference tree is absent).

Units are SeaRay simulation units with ``mks_length = 0.8 um / 2 pi`` (so the 800 nm carrier has
w = 1).
"""
import numpy as np

MKS_LENGTH = 0.8e-6 / (2 * np.pi)


def gaussian_wave(E0, w0, dw, r0, t_shift=0.0, cylindrical=False, phase_noise=None):
    """Incoming-wave callable (w, x1, x2) -> complex (N0, N1, N2): a Gaussian in w and in the
    transverse plane, with an optional transverse phase screen phase_noise(x1, x2).  The spectral
    amplitude is set so that the time-domain field irfft(i*w*A) peaks near E0 on axis."""
    def wave(w, x1, x2):
        dwn = w[1] - w[0]
        Nt = 2 * w.shape[0] - 2
        amp = E0 * Nt / (2.0 * np.sqrt(np.pi) * (dw / dwn) * w0)
        spec = np.exp(-(w - w0) ** 2 / dw ** 2) * np.exp(1j * w * t_shift)
        if cylindrical:
            tr = np.exp(-(x1[:, None] ** 2) / r0 ** 2) * np.ones((1, x2.shape[0]))
        else:
            tr = np.exp(-(x1[:, None] ** 2 + x2[None, :] ** 2) / r0 ** 2)
        if phase_noise is not None:
            tr = tr * np.exp(1j * phase_noise(x1, x2))
        return amp * spec[:, None, None] * tr[None, :, :]
    return wave


def seeded_phase(n_modes, amp, size, seed):
    """Sum of n_modes cosine gratings with random directions/phases (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    kx = rng.uniform(-3, 3, n_modes) * 2 * np.pi / size
    ky = rng.uniform(-3, 3, n_modes) * 2 * np.pi / size
    ph = rng.uniform(0, 2 * np.pi, n_modes)

    def screen(x1, x2):
        X = x1[:, None]
        Y = x2[None, :]
        out = np.zeros((x1.shape[0], x2.shape[0]))
        for i in range(n_modes):
            out += amp * np.cos(kx[i] * X + ky[i] * Y + ph[i])
        return out
    return screen


# Each case: the scalar volume keys, the medium and ionizer descriptions, the incoming wave and the
# relative density expression (a NumPy expression of x, y, z, r2).
CASES = {
    # cylindrical, Kerr only, fixed steps (config-1 physics on a small grid)
    "cyl_kerr": dict(
        keys={"wave grid": (129, 32, 1, 3), "wave coordinates": "cylindrical", "radial modes": 24,
              "frequency band": (0.0, 2.5), "nonlinear band": (0.0, 2.2),
              "size": (1600.0, 1600.0, 2.0e4), "subcycles": 4, "minimum step": 5.0e3 / 2,
              "chi3": 0.9, "density reference": 1.0, "window speed": 1.0},
        medium="SimpleAir", ionizer=None,
        wave=dict(E0=0.007, w0=1.0, dw=0.12, r0=220.0, cylindrical=True),
        density="np.ones(x.shape)"),
    # Cartesian, Kerr + explicit-form tunneling rate + plasma current, adaptive steps
    "cart_ion": dict(
        keys={"wave grid": (129, 16, 16, 2), "wave coordinates": "cartesian",
              "frequency band": (0.0, 2.5), "nonlinear band": (0.0, 2.2),
              "size": (1200.0, 1200.0, 1.5e4), "subcycles": 3, "minimum step": 200.0,
              "chi3": 0.6, "density reference": 3.1e-3, "window speed": 1.0},
        medium="SimpleAir", ionizer=dict(kind="PPT_Tunneling", Uion_eV=12.07, Z=0.53),
        wave=dict(E0=0.0095, w0=1.0, dw=0.12, r0=200.0, phase=dict(n_modes=8, amp=0.05, seed=0)),
        density="np.ones(x.shape)"),
    # cylindrical with azimuthal modes, z- and r-dependent density, ADK rate, group-velocity frame
    "cyl_az_adk": dict(
        keys={"wave grid": (65, 16, 4, 2), "wave coordinates": "cylindrical", "radial modes": 16,
              "frequency band": (0.0, 3.0), "nonlinear band": (0.1, 2.8),
              "size": (1200.0, 1200.0, 8.0e3), "subcycles": 2, "minimum step": 400.0,
              "chi3": 0.5, "density reference": 2.0e-3, "window speed": "vg"},
        medium="SimpleAir", ionizer=dict(kind="ADK", Uion_eV=12.13, Z=1.0),
        wave=dict(E0=0.008, w0=1.0, dw=0.2, r0=180.0, cylindrical=True),
        density="(1.0 + 0.3*np.exp(-r2/300.0**2))*(1.0 + 0.2*np.cos(z*3e-4))"),
    # Cartesian, series-form (curve-fit) rate from PPT, NL band cut above 0
    "cart_series": dict(
        keys={"wave grid": (129, 8, 16, 2), "wave coordinates": "cartesian",
              "frequency band": (0.0, 2.5), "nonlinear band": (0.05, 2.0),
              "size": (1000.0, 1400.0, 6.0e3), "subcycles": 2, "minimum step": 300.0,
              "chi3": 0.4, "density reference": 3.1e-3, "window speed": 1.0},
        medium="SimpleAir", ionizer=dict(kind="PPT", Uion_eV=12.07, Z=0.53, terms=40),
        wave=dict(E0=0.0085, w0=1.0, dw=0.15, r0=180.0),
        density="np.ones(x.shape)"),
    # cylindrical, Kerr + rotational Raman of N2 (32 states, 100 ps dephasing, 90 Torr), no ionization
    "cyl_raman": dict(
        keys={"wave grid": (257, 32, 1, 2), "wave coordinates": "cylindrical", "radial modes": 24,
              "frequency band": (0.0, 4.0), "nonlinear band": (0.0, 3.5),
              "size": (1600.0, 1600.0, 2.0e4), "subcycles": 4, "minimum step": 2.5e3,
              "chi3": 0.8437031382441211, "density reference": 0.015499784379078858, "window speed": 1.0},
        medium="SimpleAir", ionizer=None,
        rotator=dict(B=2.5464790894703257e-05, dalpha=0.014666374631675184, kT=4.892377952275014e-08,
                     damp=4.247069967100916e-06, hbar=3.032887794225397e-06, states=32),
        wave=dict(E0=0.0046, w0=1.0, dw=0.03, r0=400.0, cylindrical=True),
        density="0.1184*np.ones(x.shape)"),
}


# Paraxial (envelope) cases: 2^n frequency nodes over a band around the carrier, run through the
# reference's paraxial_kernel.track.
PARAXIAL_CASES = {
    # Cartesian, Kerr + explicit-form tunneling rate + plasma current, adaptive steps
    "par_cart_ion": dict(
        keys={"wave grid": (128, 16, 16, 2), "wave coordinates": "cartesian",
              "frequency band": (0.6, 1.4), "size": (1200.0, 1200.0, 1.5e4), "subcycles": 3,
              "chi3": 0.6, "density reference": 3.1e-3, "window speed": 1.0},
        medium="SimpleAir", ionizer=dict(kind="PPT_Tunneling", Uion_eV=12.07, Z=0.53),
        wave=dict(E0=0.0095, w0=1.0, dw=0.03, r0=200.0, envelope=True, phase=dict(n_modes=8, amp=0.05, seed=0)),
        density="np.ones(x.shape)"),
    # cylindrical, Kerr + the N2 rotator of cyl_raman
    "par_cyl_raman": dict(
        keys={"wave grid": (256, 32, 1, 2), "wave coordinates": "cylindrical", "radial modes": 24,
              "frequency band": (0.5, 1.5), "size": (1600.0, 1600.0, 2.0e4), "subcycles": 4,
              "chi3": 0.8437031382441211, "density reference": 0.015499784379078858, "window speed": 1.0},
        medium="SimpleAir", ionizer=None,
        rotator=dict(B=2.5464790894703257e-05, dalpha=0.014666374631675184, kT=4.892377952275014e-08,
                     damp=4.247069967100916e-06, hbar=3.032887794225397e-06, states=32),
        wave=dict(E0=0.0046, w0=1.0, dw=0.03, r0=400.0, cylindrical=True, envelope=True),
        density="0.1184*np.ones(x.shape)"),
    # cylindrical with azimuthal modes, z- and r-dependent density, ADK, group-velocity frame
    "par_cyl_az_adk": dict(
        keys={"wave grid": (64, 16, 4, 2), "wave coordinates": "cylindrical", "radial modes": 16,
              "frequency band": (0.7, 1.3), "size": (1200.0, 1200.0, 8.0e3), "subcycles": 2,
              "chi3": 0.5, "density reference": 2.0e-3, "window speed": "vg"},
        medium="SimpleAir", ionizer=dict(kind="ADK", Uion_eV=12.13, Z=1.0),
        wave=dict(E0=0.008, w0=1.0, dw=0.05, r0=180.0, cylindrical=True, envelope=True),
        density="(1.0 + 0.3*np.exp(-r2/300.0**2))*(1.0 + 0.2*np.cos(z*3e-4))"),
}


def envelope_wave(E0, w0, dw, r0, cylindrical=False, phase_noise=None):
    """Incoming-wave callable (w, x1, x2) -> complex (N0, N1, N2) for the paraxial solver: a Gaussian
    spectrum on the band's absolute frequencies, centred in the time window, whose envelope field
    ifft(i w A) (FFT order) has its crest near E0; Gaussian transverse profile, optional phase screen."""
    def wave(w, x1, x2):
        dwn = w[1] - w[0]
        N0 = w.shape[0]
        amp = E0 * N0 * dwn / (np.sqrt(np.pi) * dw * w0)
        spec = amp * np.exp(-(w - w0) ** 2 / dw ** 2) * np.exp(-1j * (w - w[N0 // 2]) * np.pi / dwn)
        if cylindrical:
            tr = np.exp(-(x1[:, None] ** 2) / r0 ** 2) * np.ones((1, x2.shape[0]))
        else:
            tr = np.exp(-(x1[:, None] ** 2 + x2[None, :] ** 2) / r0 ** 2)
        if phase_noise is not None:
            tr = tr * np.exp(1j * phase_noise(x1, x2))
        return spec[:, None, None] * tr[None, :, :]
    return wave


def rotator_args(spec):
    """Arguments of the Rotator constructor (B, dalpha, kT, dnuc, damp, hbar) for a rotator spec: N2
    nuclear degeneracy 6 for even j and 3 for odd j, one damping for every level."""
    j = np.arange(spec["states"])
    dnuc = 6.0 - 3.0 * (j % 2)
    damp = spec["damp"] * np.ones(spec["states"])
    return spec["B"], spec["dalpha"], spec["kT"], dnuc, damp, spec["hbar"]


def density_lambda(expr):
    code = compile(expr, "<density>", "eval")
    return lambda x, y, z, r2: eval(code, {"np": np}, {"x": x, "y": y, "z": z, "r2": r2})


def make_wave(spec, size):
    screen = None
    if "phase" in spec:
        p = spec["phase"]
        screen = seeded_phase(p["n_modes"], p["amp"], size, p["seed"])
    if spec.get("envelope", False):
        return envelope_wave(spec["E0"], spec["w0"], spec["dw"], spec["r0"],
                             cylindrical=spec.get("cylindrical", False), phase_noise=screen)
    return gaussian_wave(spec["E0"], spec["w0"], spec["dw"], spec["r0"],
                         cylindrical=spec.get("cylindrical", False), phase_noise=screen)
