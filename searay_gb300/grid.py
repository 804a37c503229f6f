"""Frequency and transverse grids of a UPPE volume, and the transverse eigenbases.

Host-side set-up, run once per volume (FP64, NumPy/SciPy).  Restates SeaRay's node helpers
(``modules/grid_tools.py:25-49``), the grid construction of ``FourierTool``/``BesselBeamTool``
(``modules/caustic_tools.py:27-38,88-96,207-229``), the finite-difference transverse wavenumbers
(``grid_tools.py:236-250``) and the Hankel eigenbasis (``grid_tools.py:252-298``).
"""
import numpy as np
import scipy.linalg


def cyclic_nodes(lo, hi, n):
    """Nodes of a periodic axis, low end included (grid_tools.py:25-34)."""
    if n == 1:
        return np.array([0.5 * lo + 0.5 * hi])
    d = (hi - lo) / n
    return np.linspace(lo, hi - d, n)


def cell_centers(lo, hi, n):
    """n cell-centred nodes between two walls (grid_tools.py:36-40)."""
    d = (hi - lo) / n
    return np.linspace(lo + 0.5 * d, hi - 0.5 * d, n)


def cell_walls(lo, hi, n, default_width=1000.0):
    """Walls bracketing n nodes (grid_tools.py:42-49)."""
    d = default_width if n == 1 else (hi - lo) / (n - 1)
    return np.linspace(lo - 0.5 * d, hi + 0.5 * d, n + 1)


def fd_wavenumber(num, dx):
    """Wavenumber whose square is the eigenvalue of the 3-point FD Laplacian (grid_tools.py:236-244)."""
    i = np.arange(num)
    sgn = np.ones(num)
    sgn[int(num / 2) + 1:] = -1.0
    return sgn * np.sqrt(2.0 * (1.0 - np.cos(2.0 * np.pi * i / num))) / dx


def hankel_eigenbasis(Nr, dr, mmax, Nk=None):
    """Radial modes of the root-volume-symmetrised FD Laplacian on Nr cell-centred nodes.

    For every azimuthal mode m the tridiagonal operator (grid_tools.py:274-287) is symmetrised by
    the root cell volumes and its Nk largest eigenpairs are taken with LAPACK's banded solver.
    Returns H (Nk, Nr, Nm), eigenvalues (Nr, Nm) zero-padded past Nk, and Lambda (Nr,).
    Negative azimuthal modes reuse the positive ones (FFT packing, grid_tools.py:289-293)."""
    if Nk is None:
        Nk = Nr
    r = cell_centers(0.0, Nr * dr, Nr)
    inner = 2 * np.pi * (r - 0.5 * dr)
    outer = 2 * np.pi * (r + 0.5 * dr)
    vol = np.pi * ((r + 0.5 * dr) ** 2 - (r - 0.5 * dr) ** 2)
    lam = np.sqrt(vol)
    Nm = 1 if mmax == 0 else 2 * mmax
    vals = np.zeros((Nr, Nm))
    basis = np.zeros((Nr, Nk, Nm))
    for m in range(mmax + 1):
        lower = inner / (dr * vol)
        diag = -(inner + outer) / (dr * vol) - (m / r) ** 2
        upper = outer / (dr * vol)
        diag[0] += lower[0]
        diag[Nr - 1] -= upper[Nr - 1]
        lower[1:] *= lam[1:] / lam[:-1]
        upper[:-1] *= lam[:-1] / lam[1:]
        band = np.zeros((2, Nr))
        band[0, :] = lower
        band[1, :] = diag
        vals[:Nk, m], basis[:, :, m] = scipy.linalg.eig_banded(band, select="i", select_range=(Nr - Nk, Nr - 1))
    for m in range(1, mmax):
        vals[:Nk, -m] = vals[:Nk, m]
        basis[:, :, -m] = basis[:, :, m]
    return np.ascontiguousarray(basis.swapaxes(0, 1)), vals, lam


class VolumeGrid:
    """Grids of one UPPE volume from its input dictionary (uppe_kernel.py:341-378)."""

    def __init__(self, vol_dict):
        band = vol_dict["frequency band"]
        size = (band[1] - band[0],) + tuple(vol_dict["size"])
        N = tuple(vol_dict["wave grid"])
        self.N = N
        self.band = band
        self.size = size
        self.cartesian = vol_dict["wave coordinates"] == "cartesian"
        center, width = 0.5 * (band[0] + band[1]), band[1] - band[0]
        self.w = center + cyclic_nodes(-width / 2, width / 2, N[0])
        w_walls = cell_walls(self.w[0], self.w[-1], N[0], size[1])
        if self.cartesian:
            self.x1 = cell_centers(-size[1] / 2, size[1] / 2, N[1])
            self.x2 = cell_centers(-size[2] / 2, size[2] / 2, N[2])
            kx = fd_wavenumber(N[1], size[1] / N[1])
            ky = fd_wavenumber(N[2], size[2] / N[2])
            self.kr2 = np.outer(kx ** 2, np.ones(N[2])) + np.outer(np.ones(N[1]), ky ** 2)
            self.H = None
            self.Lambda = None
            self.Nk = N[1]
        else:
            self.x1 = cell_centers(0.0, size[1] / 2, N[1])
            self.x2 = cyclic_nodes(-np.pi, np.pi, N[2])
            Nk = vol_dict.get("radial modes", None)
            self.Nk = N[1] if Nk is None else int(Nk)
            self.H, vals, self.Lambda = hankel_eigenbasis(N[1], 0.5 * size[1] / N[1], int(N[2] / 2), self.Nk)
            self.kr2 = -vals
        x1w = cell_walls(self.x1[0], self.x1[-1], N[1])
        x2w = cell_walls(self.x2[0], self.x2[-1], N[2])
        self.plot_ext = np.array([w_walls[0], w_walls[-1], x1w[0], x1w[-1], x2w[0], x2w[-1]])
        self.dt = np.pi / np.max(self.w)
        self.dw = self.w[1] - self.w[0]
        self.Nt = 2 * N[0] - 2
