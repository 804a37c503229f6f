"""Linear susceptibility chi(w) of a few media, for building UPPE inputs without the reference.

The propagator accepts any object with ``chi(w)`` (SeaRay's ``dispersion`` classes included).
These restate the two Sellmeier families of SeaRay's ``modules/dispersion.py`` (``sellmeier_medium``
:178-234, ``sellmeier_medium_alt1`` :236-294, ``SimpleAir`` :371-377) and the group velocity
used for the pulse frame (``Vacuum.GroupVelocityMagnitude`` :70-81 with ``isotropic_medium.vg``
:166-176).  Frequencies are in simulation units (w = 1 at the wavelength 2 pi mks_length).
"""
import numpy as np


class Vacuum:
    def chi(self, w):
        return np.zeros(np.shape(w))

    def dchidw(self, w):
        return np.zeros(np.shape(w))

    def GroupVelocityMagnitude(self, w):
        return np.ones(np.shape(w)) if np.ndim(w) else 1.0


class _Isotropic(Vacuum):
    def GroupVelocityMagnitude(self, w):
        w = np.asarray(w, dtype=float)
        k = w * np.real(np.sqrt(1 + self.chi(w)))
        denom = w * (1.0 + self.chi(w) + 0.5 * w * self.dchidw(w))
        v = np.abs(np.real(k / denom))
        return float(v) if v.ndim == 0 else v


class Sellmeier(_Isotropic):
    """chi = sum_i A_i lambda^2 / (lambda^2 - L_i), L_i in um^2 (dispersion.py:178-234)."""

    def __init__(self, mks_length, A, L):
        self.mks_length = mks_length
        self.A = np.asarray(A, dtype=float)
        self.D = np.asarray(L, dtype=float) * 1e-12 / mks_length ** 2 / (2 * np.pi) ** 2

    def chi(self, w):
        w = np.asarray(w, dtype=float)
        return np.sum(self.A / (1 - np.multiply.outer(w ** 2, self.D)), axis=-1)

    def dchidw(self, w):
        w = np.asarray(w, dtype=float)
        return np.sum(np.multiply.outer(2 * w, self.A * self.D) / (1.0 - np.multiply.outer(w ** 2, self.D)) ** 2, axis=-1)


class SellmeierAlt1(_Isotropic):
    """chi = sum_i B_i / (C_i - lambda^-2), B and C in um^-2 (dispersion.py:236-294)."""

    def __init__(self, mks_length, B, Cc):
        self.mks_length = mks_length
        self.Bn = (2.0 * np.pi) ** 2 * mks_length ** 2 * 1e12 * np.asarray(B, dtype=float)
        self.Cn = (2.0 * np.pi) ** 2 * mks_length ** 2 * 1e12 * np.asarray(Cc, dtype=float)

    def chi(self, w):
        w = np.asarray(w, dtype=float)
        return np.sum(self.Bn / (self.Cn - np.multiply.outer(w ** 2, np.ones_like(self.Cn))), axis=-1)

    def dchidw(self, w):
        w = np.asarray(w, dtype=float)
        return np.sum(np.multiply.outer(2 * w, self.Bn) / (self.Cn - np.multiply.outer(w ** 2, np.ones_like(self.Cn))) ** 2, axis=-1)


class SimpleAir(SellmeierAlt1):
    """Two-term air fit valid from 0.2 to 1.0 um (dispersion.py:371-377)."""

    def __init__(self, mks_length):
        super().__init__(mks_length, B=2 * np.array([0.05792105, 0.00167917]), Cc=np.array([238.0185, 57.362]))


class FusedSilica(Sellmeier):
    """Fused silica, three-term Sellmeier fit of I. H. Malitson, J. Opt. Soc. Am. 55, 1205 (1965)
    (A_i dimensionless, L_i in um^2).  Not part of SeaRay; used for the solid-state workload."""

    def __init__(self, mks_length):
        super().__init__(mks_length,
                         A=[0.6961663, 0.4079426, 0.8974794],
                         L=[0.0684043 ** 2, 0.1162414 ** 2, 9.896161 ** 2])
