"""UPPE volumes for the benchmark workloads, built from synthetic analytic inputs.

No public dataset is involved: every input is an analytic pulse in a dispersive, Kerr and
ionizing medium.  Units follow SeaRay: lengths in mks_length = lambda0 / (2 pi), so the carrier
has w = 1.  Unit conversions restate SeaRay's ``InputHelper.dnum`` (``modules/input_tools.py:5-61``).

Workloads (sizes as the reference's volume dictionaries spell them, ``'wave grid' = (N0, N1, N2, N3)``
with N0 = 2^n + 1 frequency nodes):

* ``cyl_kerr_64``: cylindrical, N0 = 257 (Nt = 512, 400 fs window), Nr = Nk = 64 over R = 1 mm,
  800 nm 50 fs Gaussian, w0 = 200 um, 1e13 W/cm^2, two-term air, n2 = 3e-19 cm^2/W, Kerr only,
  100 RK4 steps over 10 cm.
* ``cart_filament_128``: Cartesian 128 x 128 over 2 mm, N0 = 513 (band 0-4 w0), 800 nm 35 fs pulse
  at 5 critical powers, 8-mode seeded transverse phase (0.05 rad, numpy default_rng(0)), Kerr
  (n2 = 3e-19 cm^2/W) + O2 tunneling ionization (PPT, Ip = 12.07 eV, Z = 0.53) at 5.4e18 cm^-3 +
  plasma current, 400 RK4 steps over 10 cm.
* ``cart_filament_256``: Cartesian 256 x 256 over 3 mm, N0 = 1025 (band 0-4 w0), 800 nm 40 fs pulse at
  10 critical powers, the 8-mode seeded transverse phase of ``cart_filament_128`` (scaled to the
  box), the same medium, 1000 RK4 steps over 10 cm.
* ``cyl_adjoint_256``: the physics of ``cyl_kerr_64`` on N0 = 1025 (Nt = 2048, band 0-6.9 w0),
  Nr = Nk = 256, 200 RK4 steps over 10 cm; the forward + adjoint workload.
* ``cyl_silica_512``: cylindrical Nr = Nk = 512 over R = 1 mm, N0 = 2049 (band 0-4 w0, nonlinear
  band 0.3-3.5 w0), 1 um 100 fs pulse of 60 um radius at 1e13 W/cm^2 in fused silica (Malitson
  Sellmeier, n2 = 2.5e-16 cm^2/W), PPT tunneling with Ip = 9 eV (Z = 1 assumed) at 2.2e22 cm^-3,
  100 RK4 steps over 20 um.  The intensity, the radius of the grid and the lower edge of the
  nonlinear band keep the explicit RK4 step stable: at 2e13 W/cm^2 and above this rate model
  ionizes the glass past ten times the critical density within the pulse, and the plasma current
  of an overdense plasma needs steps below a nanometre; the Sellmeier fit has a pole at 9.9 um
  (w = 0.10 w0) with n^2 crossing zero just below it, and with R = 0.5 mm the Hankel modes reach
  transverse wavenumbers near k(w) for w < 0.35 w0 (near-cutoff modes, where the source is divided
  by a vanishing Re kz).
* ``cyl_raman_2049``: rotational Raman (N2, 32 states) with Kerr, cylindrical N0 = 2049 (band 0-8 w0),
  Nr = Nk = 256 over R = 1 mm, 800 nm 40 fs pulse at 4.5e13 W/cm^2, 100 RK4 steps over 0.441 cm.
* ``cyl_raman_paraxial_256``: the same physics with the paraxial envelope propagator (``'propagator':
  'paraxial'``): N0 = 256 over the band 0.5-1.5 w0, Nr = Nk = 256, 100 RK4 steps over 0.441 cm.
"""
import numpy as np
from scipy import constants as C

from . import dispersion, ionization


class Units:
    """Simulation-unit conversions (input_tools.py:5-61)."""

    def __init__(self, mks_length):
        self.x1 = mks_length
        self.t1 = mks_length / C.c
        self.w1 = 1 / self.t1
        self.E1 = C.m_e * C.c * self.w1 / C.e
        self.n1 = C.epsilon_0 * C.m_e * self.w1 ** 2 / C.e ** 2
        self.u1 = C.m_e * C.c ** 2
        self.N1 = self.n1 * self.x1 ** 3

    def fs(self, v):
        return v * 1e-15 / self.t1

    def um(self, v):
        return v * 1e-6 / self.x1

    def mm(self, v):
        return v * 1e-3 / self.x1

    def cm(self, v):
        return v * 1e-2 / self.x1

    def W_cm2(self, v):
        return v * 1e4 * self.t1 * self.x1 ** 2 / self.N1 / self.u1

    def m2_W(self, v):
        return v * self.N1 * self.u1 / self.x1 ** 2 / self.t1

    def eV(self, v):
        return v * C.e / self.u1

    def cm3(self, v):
        return v * 1e6 / self.n1

    def chi3(self, n0, n2_m2_W):
        """chi3 = (4/3) n0^2 n2 (input_tools.py:110-111)."""
        return (4 / 3) * n0 ** 2 * self.m2_W(n2_m2_W)


def seeded_phase_screen(n_modes, amp, size, seed):
    """Transverse phase: sum of n_modes cosine gratings, random directions and phases from
    numpy default_rng(seed), wavenumbers up to 3 cycles across the box."""
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


def gaussian_pulse(E0, tau, r0, cylindrical=False, screen=None, w0=1.0):
    """Incoming wave (w, x1, x2) -> complex (N0, N1, N2): a transform-limited Gaussian pulse
    E(t) = E0 exp(-t^2/tau^2) cos(w0 t) centred in the time window, Gaussian transverse profile of
    1/e field radius r0, optional transverse phase screen."""
    def wave(w, x1, x2):
        dwn = w[1] - w[0]
        Nt = 2 * w.shape[0] - 2
        dw = 2.0 / tau
        amp = E0 * Nt / (2.0 * np.sqrt(np.pi) * (dw / dwn) * w0)
        T = 2 * np.pi / dwn
        spec = amp * np.exp(-(w - w0) ** 2 / dw ** 2) * np.exp(1j * w * 0.5 * T)
        if cylindrical:
            tr = np.exp(-(x1[:, None] ** 2) / r0 ** 2) * np.ones((1, x2.shape[0]))
        else:
            tr = np.exp(-(x1[:, None] ** 2 + x2[None, :] ** 2) / r0 ** 2)
        if screen is not None:
            tr = tr * np.exp(1j * screen(x1, x2))
        return spec[:, None, None] * tr[None, :, :]
    return wave


def envelope_pulse(E0, tau, r0, cylindrical=False, w0=1.0):
    """Incoming wave for the paraxial (envelope) solver: the spectrum on the band's absolute
    frequencies of the pulse E0 exp(-t^2/tau^2) around carrier w0, centred in the time window, so that
    the envelope field ifft(i w A) (FFT order) has its crest near E0; Gaussian transverse profile."""
    def wave(w, x1, x2):
        dwn = w[1] - w[0]
        N0 = w.shape[0]
        dw = 2.0 / tau
        amp = E0 * N0 * dwn / (np.sqrt(np.pi) * dw * w0)
        spec = amp * np.exp(-(w - w0) ** 2 / dw ** 2) * np.exp(-1j * (w - w[N0 // 2]) * np.pi / dwn)
        if cylindrical:
            tr = np.exp(-(x1[:, None] ** 2) / r0 ** 2) * np.ones((1, x2.shape[0]))
        else:
            tr = np.exp(-(x1[:, None] ** 2 + x2[None, :] ** 2) / r0 ** 2)
        return spec[:, None, None] * tr[None, :, :]
    return wave


def field_from_intensity(u, I_W_cm2):
    """Peak field (simulation units) of a linearly polarised wave of intensity I: E = sqrt(2 I)."""
    return np.sqrt(2 * u.W_cm2(I_W_cm2))


def critical_power_W(lam_m, n0, n2_m2_W):
    """Marburger critical power 3.77 lambda^2 / (8 pi n0 n2)."""
    return 3.77 * lam_m ** 2 / (8 * np.pi * n0 * n2_m2_W)


def cyl_kerr_64(steps=100):
    x1 = 0.8e-6 / (2 * np.pi)
    u = Units(x1)
    air = dispersion.SimpleAir(x1)
    N0 = 257
    W = 2 * np.pi * N0 / u.fs(400.0)
    L = u.cm(10.0)
    E0 = field_from_intensity(u, 1e13)
    vd = {
        "wave grid": (N0, 64, 1, 2), "wave coordinates": "cylindrical", "radial modes": 64,
        "frequency band": (0.0, W), "nonlinear band": (0.0, W),
        "size": (2 * u.mm(1.0), 2 * u.mm(1.0), L), "subcycles": steps, "minimum step": L / steps,
        "chi3": u.chi3(1.0, 3e-23), "density reference": 1.0,
        "window speed": air.GroupVelocityMagnitude(1.0),
        "dispersion inside": air, "ionizer": None,
        "density lambda": lambda x, y, z, r2: np.ones(x.shape),
        "incoming wave": gaussian_pulse(E0, u.fs(50.0), u.um(200.0), cylindrical=True),
    }
    return vd


def cart_filament_128(steps=400, n_perp=128):
    x1 = 0.8e-6 / (2 * np.pi)
    u = Units(x1)
    air = dispersion.SimpleAir(x1)
    n2 = 3e-23
    r0 = u.mm(0.3)
    P = 5 * critical_power_W(0.8e-6, 1.0, n2)
    I0 = 2 * P / (np.pi * (0.3e-3) ** 2) * 1e-4  # W/cm^2
    E0 = field_from_intensity(u, I0)
    L = u.cm(10.0)
    box = u.mm(2.0)
    vd = {
        "wave grid": (513, n_perp, n_perp, 2), "wave coordinates": "cartesian",
        "frequency band": (0.0, 4.0), "nonlinear band": (0.0, 3.5),
        "size": (box, box, L), "subcycles": steps, "minimum step": L / steps,
        "chi3": u.chi3(1.0, n2), "density reference": u.cm3(5.4e18),
        "window speed": air.GroupVelocityMagnitude(1.0),
        "dispersion inside": air,
        "ionizer": ionization.PPT_Tunneling(x1, False, u.eV(12.07), 0.53),
        "density lambda": lambda x, y, z, r2: np.ones(x.shape),
        "incoming wave": gaussian_pulse(E0, u.fs(35.0), r0, screen=seeded_phase_screen(8, 0.05, box, 0)),
    }
    return vd


def cart_filament_256(steps=1000):
    x1 = 0.8e-6 / (2 * np.pi)
    u = Units(x1)
    air = dispersion.SimpleAir(x1)
    n2 = 3e-23
    r0 = u.mm(0.3)
    P = 10 * critical_power_W(0.8e-6, 1.0, n2)
    I0 = 2 * P / (np.pi * (0.3e-3) ** 2) * 1e-4  # W/cm^2
    E0 = field_from_intensity(u, I0)
    L = u.cm(10.0)
    box = u.mm(3.0)
    vd = {
        "wave grid": (1025, 256, 256, 2), "wave coordinates": "cartesian",
        "frequency band": (0.0, 4.0), "nonlinear band": (0.0, 3.5),
        "size": (box, box, L), "subcycles": steps, "minimum step": L / steps,
        "chi3": u.chi3(1.0, n2), "density reference": u.cm3(5.4e18),
        "window speed": air.GroupVelocityMagnitude(1.0),
        "dispersion inside": air,
        "ionizer": ionization.PPT_Tunneling(x1, False, u.eV(12.07), 0.53),
        "density lambda": lambda x, y, z, r2: np.ones(x.shape),
        "incoming wave": gaussian_pulse(E0, u.fs(40.0), r0, screen=seeded_phase_screen(8, 0.05, box, 0)),
    }
    return vd


def cyl_silica_512(steps=100):
    x1 = 1.0e-6 / (2 * np.pi)
    u = Units(x1)
    glass = dispersion.FusedSilica(x1)
    n0 = float(np.sqrt(1 + glass.chi(np.array([1.0]))[0]))
    L = u.um(20.0)
    E0 = field_from_intensity(u, 1e13) / np.sqrt(n0)
    vd = {
        "wave grid": (2049, 512, 1, 2), "wave coordinates": "cylindrical", "radial modes": 512,
        "frequency band": (0.0, 4.0), "nonlinear band": (0.3, 3.5),
        "size": (2 * u.mm(1.0), 2 * u.mm(1.0), L), "subcycles": steps, "minimum step": L / steps,
        "chi3": u.chi3(n0, 2.5e-20), "density reference": u.cm3(2.2e22),
        "window speed": glass.GroupVelocityMagnitude(1.0),
        "dispersion inside": glass,
        "ionizer": ionization.PPT_Tunneling(x1, False, u.eV(9.0), 1.0),
        "density lambda": lambda x, y, z, r2: np.ones(x.shape),
        "incoming wave": gaussian_pulse(E0, u.fs(100.0), u.um(60.0), cylindrical=True),
    }
    return vd


def cyl_adjoint_256(steps=200):
    """The adjoint workload: cyl_kerr_64's physics on N0 = 1025 (band scaled with the grid), Nr = 256."""
    vd = cyl_kerr_64(steps)
    W = vd["frequency band"][1] * 1024 / 256
    vd["wave grid"] = (1025, 256, 1, 2)
    vd["radial modes"] = 256
    vd["frequency band"] = (0.0, W)
    vd["nonlinear band"] = (0.0, W)
    return vd


def n2_rotator(u):
    """N2 rotations as SeaRay's rotational Raman example sets them: B = 2 cm^-1, dalpha = 4 pi 6.7e-25
    cm^3, kT = 0.025 eV, 32 states with nuclear degeneracy 6 (even j) and 3 (odd j), 100 ps
    dephasing; hbar in units of m_e c^2 / w1."""
    from .rotations import Rotator
    j = np.arange(32)
    return Rotator(2.0 / u.cm(1.0), 4 * np.pi * 6.7e-25 / u.cm3(1.0), u.eV(0.025), 6 - 3 * (j % 2),
                   np.ones(32) / u.fs(1e5), C.hbar * u.w1 / u.u1)


def cyl_raman_2049(steps=100):
    """Rotational Raman benchmark: SeaRay's example of that name with the UPPE propagator (cylindrical
    N0 = 2049 over the band 0-8 w0, Nr = Nk = 256 over R = 1 mm, nonlinear band 0-4 w0), 800 nm
    40 fs (FWHM intensity) pulse of 150 um radius at 4.5e13 W/cm^2 in N2 at 90 Torr: Kerr
    (n2 = 14.8e-24 m^2/W) and the N2 rotator, no ionization.  Two-term air stands in for the
    example's humid-air dispersion; fixed steps over the example's 0.441 cm."""
    x1 = 0.8e-6 / (2 * np.pi)
    u = Units(x1)
    air = dispersion.SimpleAir(x1)
    L = u.cm(0.441)
    E0 = field_from_intensity(u, 4.5e13)
    tau = u.fs(40.0) / np.sqrt(2 * np.log(2))
    rel = 90.0 / 760.0
    vd = {
        "wave grid": (2049, 256, 1, 2), "wave coordinates": "cylindrical", "radial modes": 256,
        "frequency band": (0.0, 8.0), "nonlinear band": (0.0, 4.0),
        "size": (2 * u.mm(1.0), 2 * u.mm(1.0), L), "subcycles": steps, "minimum step": L / steps,
        "chi3": u.chi3(1.0, 14.8e-24), "density reference": u.cm3(2.7e19),
        "window speed": air.GroupVelocityMagnitude(1.0),
        "dispersion inside": air, "ionizer": None, "rotator": n2_rotator(u),
        "density lambda": lambda x, y, z, r2: rel * np.ones(x.shape),
        "incoming wave": gaussian_pulse(E0, tau, u.um(150.0), cylindrical=True),
    }
    return vd


def cyl_raman_paraxial_256(steps=100):
    """Rotational Raman benchmark with the paraxial (envelope) propagator, SeaRay's default for that
    example: N0 = 256 frequencies over the band 0.5-1.5 w0, cylindrical Nr = Nk = 256 over R = 1 mm,
    the pulse, medium and N2 rotator of ``cyl_raman_2049``; fixed steps over 0.441 cm."""
    vd = cyl_raman_2049(steps)
    vd["propagator"] = "paraxial"
    vd["wave grid"] = (256, 256, 1, 2)
    vd["frequency band"] = (0.5, 1.5)
    x1 = 0.8e-6 / (2 * np.pi)
    u = Units(x1)
    E0 = field_from_intensity(u, 4.5e13)
    tau = u.fs(40.0) / np.sqrt(2 * np.log(2))
    vd["incoming wave"] = envelope_pulse(E0, tau, u.um(150.0), cylindrical=True)
    del vd["nonlinear band"]
    return vd


WORKLOADS = {"cyl_kerr_64": cyl_kerr_64, "cart_filament_128": cart_filament_128, "cart_filament_256": cart_filament_256,
             "cyl_silica_512": cyl_silica_512, "cyl_adjoint_256": cyl_adjoint_256, "cyl_raman_2049": cyl_raman_2049,
             "cyl_raman_paraxial_256": cyl_raman_paraxial_256}
