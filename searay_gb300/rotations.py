"""Molecular rotations for the rotational Raman response (SeaRay ``modules/rotations.py``).

``Rotator`` takes the reference's constructor arguments and derives the same per-state tables
(``rotations.py:15-44``): level frequencies w_j = 2 pi B j (j+1), thermal populations
rho0_j = dnuc_j exp(-hbar w_j / kT) / Z with Z = sum (2j+1) dnuc_j exp(-hbar w_j / kT), and for
each j -> j-2 transition the complex frequency W_j = w_j - w_(j-2) + i damp_j and the population
difference T_j = rho0_j - rho0_(j-2).  The propagator reads ``Wj``, ``Tj``, ``dalpha`` and ``hbar``,
so SeaRay's own ``Rotator`` objects work as well.
"""
import numpy as np


class Rotator:
    def __init__(self, B, dalpha, kT, dnuc, damp, hbar):
        """:param B: rotational constant (inverse length, simulation units)
        :param dalpha: polarizability difference (volume, simulation units)
        :param kT: temperature as an energy
        :param dnuc: nuclear degeneracy per state j (its length is the number of states)
        :param damp: damping rate per state
        :param hbar: reduced Planck constant in simulation units"""
        dnuc = np.asarray(dnuc, dtype=float)
        damp = np.asarray(damp, dtype=float)
        n = dnuc.shape[0]
        j = np.arange(n)
        self.dalpha = dalpha
        self.hbar = hbar
        self.wj = 2 * np.pi * B * j * (j + 1)
        X = dnuc * np.exp(-hbar * self.wj / kT)
        Z = np.sum((2 * j + 1) * X)
        self.rho0jm = X / Z if Z > 0 else np.zeros(n)
        self.Wj = np.zeros(n, dtype=np.cdouble)
        self.Tj = np.zeros(n)
        self.Wj[2:] = self.wj[2:] - self.wj[:-2] + 1j * damp[2:]
        self.Tj[2:] = self.rho0jm[2:] - self.rho0jm[:-2]
