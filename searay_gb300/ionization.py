"""Photoionization models on the host: coefficients of the device rate evaluation.

The propagator takes the reference's rate-model objects unchanged (anything with ``GetCoeff()``,
``Rate(E)`` in atomic units and ``get_mks_length()``, e.g. SeaRay's ``ionization.PPT_Tunneling``).
:class:`RateCoefficients` turns such an object into the numbers the device kernel needs, as
SeaRay's ``ionization.Ionizer`` does (``modules/ionization.py:36-60,88-150``): the closed form
rate = rate_conv * C_pre * E^C_pow * exp(C_exp/E) when C_pre > 0, else a 5th-order polynomial
fit of log(rate) against log(E).

Closed-form rate models (``Hydrogen``, ``ADK``, ``PPT_Tunneling``) are restated here from
``modules/photoionization_base.py:183-335`` so that runs on machines without the reference can
build inputs; their constructors take simulation units like the reference's wrappers
(``modules/ionization.py:65-86``).
"""
import math

import numpy as np
import scipy.optimize
from scipy import constants as C


class AtomicUnits:
    """Atomic units in SI (photoionization_base.py:183-195)."""

    def __init__(self):
        self.xa = C.hbar / (C.m_e * C.c * C.alpha)
        self.ta = C.hbar / (C.m_e * C.c ** 2 * C.alpha ** 2)
        self.ua = C.m_e * C.c ** 2 * C.alpha ** 2
        self.ea = self.ua / self.xa / C.e

    def energy_to_au(self, u_eV):
        return u_eV * C.e / self.ua


class SimulationUnits(AtomicUnits):
    """Conversions between simulation units (length mks_length) and atomic units (ionization.py:36-59)."""

    def __init__(self, mks_length):
        super().__init__()
        self.xs = mks_length
        self.ts = mks_length / C.c
        self.us = C.m_e * C.c ** 2
        self.es = self.us / self.xs / C.e

    def rate_sim_to_au(self, r):
        return r * self.ta / self.ts

    def rate_au_to_sim(self, r):
        return r * self.ts / self.ta

    def field_sim_to_au(self, f):
        return f * self.es / self.ea

    def energy_sim_to_au(self, u):
        return u * self.us / self.ua


class ClosedFormRate(AtomicUnits):
    """Rate C_pre * E^C_pow * exp(C_exp/E), E = |E| + cutoff, in atomic units
    (photoionization_base.py:198-258).  ``averaging`` selects the cycle-averaged form."""

    cutoff_field = 1e-3

    def __init__(self, averaging, Uion, Z, lstar=0, l=0, m=0, w0=0, terms=1):
        super().__init__()
        self.avg = averaging
        self.Uion = Uion
        self.Z = Z
        self.lstar = lstar
        self.l = l
        self.m = m
        self.w0 = w0
        self.terms = terms
        self.C_pre = 0.0
        self.C_pow = 0.0
        self.C_exp = 0.0

    def GetCoeff(self):
        return self.C_pre, self.C_pow, self.C_exp

    def ToAverage(self):
        self.C_pre *= np.sqrt(3.0 / np.pi) / (2 * self.Uion) ** 0.75
        self.C_pow += 0.5

    def ToStatic(self):
        self.C_pre *= (2 * self.Uion) ** 0.75 / np.sqrt(3.0 / np.pi)
        self.C_pow -= 0.5

    def Rate(self, Es):
        E = np.abs(Es) + self.cutoff_field
        return self.C_pre * E ** self.C_pow * np.exp(self.C_exp / E)


class HydrogenAU(ClosedFormRate):
    """Landau-Lifshitz hydrogen rate (photoionization_base.py:260-268)."""

    def __init__(self, averaging, Uion, Z, *a, **k):
        super().__init__(averaging, Uion, Z)
        self.C_pre, self.C_pow, self.C_exp = 4.0, -1.0, -2.0 / 3.0
        if averaging:
            self.ToAverage()


class ADKAU(ClosedFormRate):
    """ADK rate for arbitrary states (photoionization_base.py:270-286)."""

    def __init__(self, averaging, Uion, Z, lstar=0, l=0, m=0, w0=0, terms=1):
        super().__init__(averaging, Uion, Z, lstar, l, m)
        nstar = Z / np.sqrt(2 * Uion)
        m = abs(m)
        e = math.e
        sn2l2 = np.sqrt(nstar ** 2 - lstar ** 2)
        cp = np.sqrt(3 / np.pi ** 3) * (2 * l + 1) * math.factorial(l + m) / math.factorial(m) / math.factorial(l - m)
        cp *= (e / sn2l2) ** (m + 1.5)
        cp *= ((nstar + lstar) / (nstar - lstar)) ** (lstar + 0.5)
        cp *= Z ** 2 / nstar ** 3
        cp *= (4 * e * Z ** 3 / nstar ** 3 / sn2l2) ** (2 * nstar - m - 1.5)
        self.C_pre = cp
        self.C_pow = m + 1.5 - 2 * nstar
        self.C_exp = -2 * Z ** 3 / (3 * nstar ** 3)
        if not averaging:
            self.ToStatic()


class PPTTunnelingAU(ClosedFormRate):
    """PPT in the tunneling limit with the Coulomb factor (photoionization_base.py:314-335)."""

    def __init__(self, averaging, Uion, Z, lstar=0, l=0, m=0, w0=0, terms=1):
        super().__init__(averaging, Uion, Z, lstar, l, m, w0, terms)
        from scipy import special as spsf
        nstar = Z / np.sqrt(2 * Uion)
        m = abs(m)
        F0 = Z ** 3 / nstar ** 3
        cp = Uion
        cp *= 2 ** (2 * nstar) / (nstar * spsf.gamma(nstar + lstar + 1) * spsf.gamma(nstar - lstar))
        cp *= np.sqrt(6 / np.pi)
        cp *= (2 * l + 1) * math.factorial(l + m) / 2 ** m / math.factorial(m) / math.factorial(l - m)
        cp *= (0.5 / F0) ** (m + 1.5)
        self.C_pow = m + 1.5
        self.C_exp = -2 * F0 / 3
        cp *= (2 * F0) ** (2 * nstar)
        self.C_pow -= 2 * nstar
        self.C_pre = cp
        if not averaging:
            self.ToStatic()


class _SimUnitsWrapper:
    """Construct a rate model from simulation units (ionization.py:65-71)."""

    def __init__(self, mks_length, averaging, Uion, Z, lstar=0, l=0, m=0, w0=0, terms=1):
        self.mks_length = mks_length
        uc = SimulationUnits(mks_length)
        super().__init__(averaging, uc.energy_sim_to_au(Uion), Z, lstar, l, m, uc.rate_sim_to_au(w0), terms)

    def get_mks_length(self):
        return self.mks_length


class ADK(_SimUnitsWrapper, ADKAU):
    pass


class PPT_Tunneling(_SimUnitsWrapper, PPTTunnelingAU):
    pass


class Hydrogen(_SimUnitsWrapper, HydrogenAU):
    pass


class RateCoefficients:
    """Device-rate coefficients from a rate model (ionization.py:88-109,131-150)."""

    def __init__(self, rate_gen, pts=256, mks_length=0.0):
        xs = rate_gen.get_mks_length() if mks_length == 0.0 else mks_length
        units = SimulationUnits(xs)
        self.field_conv = units.field_sim_to_au(1.0)
        self.rate_conv = units.rate_au_to_sim(1.0)
        self.cutoff = 1e-3
        self.C1, self.C2, self.C3 = rate_gen.GetCoeff()
        self.clog = np.zeros(6)
        self.explicit = self.C1 > 0.0
        if self.C1 == 0.0:
            def model(x, c0, c1, c2, c3, c4, c5):
                return c0 + c1 * x + c2 * x ** 2 + c3 * x ** 3 + c4 * x ** 4 + c5 * x ** 5
            E = np.logspace(np.log10(self.cutoff * 2), np.log10(1), pts)
            r = rate_gen.Rate(E)
            self.clog, _ = scipy.optimize.curve_fit(model, np.log(E), np.log(r))
