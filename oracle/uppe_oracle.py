"""FP64 CPU oracle for the UPPE z-step — TEST INFRASTRUCTURE, never part of the product path.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
this module, and only to check results against / as the timed CPU baseline.  The CUDA path in ``searay_gb300``
does not import it and has no CPU fallback.

This is a NumPy restatement of SeaRay's UPPE algorithm (``modules/uppe_kernel.py``, kernels
``kernels/uppe.cl``, ``kernels/fft.cl``, ``kernels/ionization.cl``, ``kernels/paraxial.cl:27-58``),
function by function, with every step citing the reference line it follows.  It is pinned against
the reference itself: ``tests/golden/make_golden.py`` runs the reference's own unmodified Python
and OpenCL kernels (compiled as C++, ``oracle/refshim``) and stores the outputs as fixtures, and
``tests/test_oracle_golden.py`` checks this module against them and against the reference test
suite's known answers (``test/gaussian_test.py:110-154``).

Arrays use the reference layout: spectral ``[w][x|r][y|phi]`` complex128, time ``[t][x][y]``
float64, ``Nt = 2*N0 - 2``.
"""
import math
import os

import numpy as np
import scipy.fft
import scipy.linalg
import scipy.optimize
from scipy import constants as C

_WORKERS = int(os.environ.get("ORACLE_FFT_WORKERS", "0")) or (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else 1)


def set_workers(n):
    global _WORKERS
    _WORKERS = max(1, int(n))


# ----------------------------------------------------------------------------------------------
# grids (modules/grid_tools.py:25-49, modules/caustic_tools.py:27-38,88-96,207-229)
# ----------------------------------------------------------------------------------------------

def cyclic_nodes(lo, hi, n):
    """grid_tools.py:25-34"""
    if n == 1:
        return np.array([0.5 * lo + 0.5 * hi])
    d = (hi - lo) / n
    return np.linspace(lo, hi - d, n)


def cell_centers(lo, hi, n):
    """grid_tools.py:36-40"""
    d = (hi - lo) / n
    return np.linspace(lo + 0.5 * d, hi - 0.5 * d, n)


def cell_walls(lo, hi, n, default_width=1000.0):
    """grid_tools.py:42-49"""
    d = default_width if n == 1 else (hi - lo) / (n - 1)
    return np.linspace(lo - 0.5 * d, hi + 0.5 * d, n + 1)


def fd_k(num, dx):
    """Finite-difference wavenumber whose square is the FD Laplacian eigenvalue (grid_tools.py:236-244)."""
    i = np.arange(num)
    sgn = np.ones(num)
    sgn[int(num / 2) + 1:] = -1.0
    return sgn * np.sqrt(2.0 * (1.0 - np.cos(2.0 * np.pi * i / num))) / dx


def hankel_basis(Nr, dr, mmax, Nk):
    """Eigenbasis of the root-volume-symmetrised FD radial Laplacian (grid_tools.py:254-294).

    Returns H with shape (Nk, Nr, Nm), eigenvalues ``vals`` (Nr, Nm) padded with zeros past Nk,
    and the root-volume weights Lambda (Nr,)."""
    if Nk is None:
        Nk = Nr
    r = cell_centers(0.0, Nr * dr, Nr)
    A1 = 2 * np.pi * (r - 0.5 * dr)
    A2 = 2 * np.pi * (r + 0.5 * dr)
    V = np.pi * ((r + 0.5 * dr) ** 2 - (r - 0.5 * dr) ** 2)
    lam = np.sqrt(V)
    Nm = 1 if mmax == 0 else 2 * mmax
    vals = np.zeros((Nr, Nm))
    Hi = np.zeros((Nr, Nk, Nm))
    for m in range(0, mmax + 1):
        T1 = A1 / (dr * V)
        T2 = -(A1 + A2) / (dr * V) - (m / r) ** 2
        T3 = A2 / (dr * V)
        T2[0] += T1[0]
        T2[Nr - 1] -= T3[Nr - 1]
        T1[1:] *= lam[1:] / lam[:-1]
        T3[:-1] *= lam[:-1] / lam[1:]
        band = np.zeros((2, Nr))
        band[0, :] = T1
        band[1, :] = T2
        vals[:Nk, m], Hi[:, :, m] = scipy.linalg.eig_banded(band, select="i", select_range=(Nr - Nk, Nr - 1))
    for m in range(1, mmax):
        vals[:Nk, -m] = vals[:Nk, m]
        Hi[:, :, -m] = Hi[:, :, m]
    H = np.ascontiguousarray(Hi.swapaxes(0, 1))
    return H, vals, lam


class Grid:
    """Frequency and transverse grids of a UPPE volume (uppe_kernel.py:341-378, caustic_tools.py)."""

    def __init__(self, vol_dict):
        band = vol_dict["frequency band"]
        size = (band[1] - band[0],) + tuple(vol_dict["size"])
        N = tuple(vol_dict["wave grid"])
        self.N = N
        self.band = band
        self.size = size
        self.cartesian = vol_dict["wave coordinates"] == "cartesian"
        w0c, dwb = 0.5 * (band[0] + band[1]), band[1] - band[0]
        self.w = w0c + cyclic_nodes(-dwb / 2, dwb / 2, N[0])
        w_walls = cell_walls(self.w[0], self.w[-1], N[0], size[1])
        if self.cartesian:
            self.x1 = cell_centers(-size[1] / 2, size[1] / 2, N[1])
            self.x2 = cell_centers(-size[2] / 2, size[2] / 2, N[2])
            x1w = cell_walls(self.x1[0], self.x1[-1], N[1])
            x2w = cell_walls(self.x2[0], self.x2[-1], N[2])
            dx1 = size[1] / N[1]
            dx2 = size[2] / N[2]
            kx = fd_k(N[1], dx1)
            ky = fd_k(N[2], dx2)
            self.kr2 = np.outer(kx ** 2, np.ones(N[2])) + np.outer(np.ones(N[1]), ky ** 2)
            self.H = None
            self.Nk = N[1]
        else:
            mmax = int(N[2] / 2)
            self.x1 = cell_centers(0.0, size[1] / 2, N[1])
            self.x2 = cyclic_nodes(-np.pi, np.pi, N[2])
            x1w = cell_walls(self.x1[0], self.x1[-1], N[1])
            x2w = cell_walls(self.x2[0], self.x2[-1], N[2])
            dr = 0.5 * size[1] / N[1]
            Nk = vol_dict.get("radial modes", None)
            self.Nk = N[1] if Nk is None else Nk
            self.H, vals, self.Lambda = hankel_basis(N[1], dr, mmax, self.Nk)
            self.kr2 = -vals
        self.plot_ext = np.array([w_walls[0], w_walls[-1], x1w[0], x1w[-1], x2w[0], x2w[-1]])
        self.dt = np.pi / np.max(self.w)
        self.dw = self.w[1] - self.w[0]
        self.Nt = 2 * N[0] - 2

    # transverse transforms (grid_tools.py:220-229, 308-325; fft.cl:363-477)
    def kspace(self, a):
        if self.cartesian:
            return scipy.fft.fft(scipy.fft.fft(a, axis=1, workers=_WORKERS), axis=2, workers=_WORKERS)
        b = scipy.fft.fft(a, axis=2, workers=_WORKERS) * self.Lambda[None, :, None]
        out = np.zeros_like(b)
        out[:, :self.Nk, :] = np.einsum("ijm,fjm->fim", self.H, b)
        out /= self.Lambda[None, :, None]
        return out

    def rspace(self, a):
        if self.cartesian:
            return scipy.fft.ifft(scipy.fft.ifft(a, axis=2, workers=_WORKERS), axis=1, workers=_WORKERS)
        b = a * self.Lambda[None, :, None]
        out = np.einsum("jim,fjm->fim", self.H, b[:, :self.Nk, :])
        out /= self.Lambda[None, :, None]
        return scipy.fft.ifft(out, axis=2, workers=_WORKERS)


# ----------------------------------------------------------------------------------------------
# ionization coefficients (modules/ionization.py:36-150, photoionization_base.py:183-195)
# ----------------------------------------------------------------------------------------------

class RateCoefficients:
    """Host-side coefficients of the rate kernels, from a rate-model object with ``GetCoeff``,
    ``Rate`` (atomic units) and ``get_mks_length`` (ionization.py:88-109,131-150)."""

    def __init__(self, rate_gen, pts=256, mks_length=0.0):
        xs = rate_gen.get_mks_length() if mks_length == 0.0 else mks_length
        xa = C.hbar / (C.m_e * C.c * C.alpha)
        ta = C.hbar / (C.m_e * C.c ** 2 * C.alpha ** 2)
        ua = C.m_e * C.c ** 2 * C.alpha ** 2
        ea = ua / xa / C.e
        ts = xs / C.c
        es = C.m_e * C.c ** 2 / xs / C.e
        self.field_conv = es / ea
        self.rate_conv = ts / ta
        self.cutoff = 1e-3
        self.C1, self.C2, self.C3 = rate_gen.GetCoeff()
        self.explicit = self.C1 > 0.0
        self.clog = np.zeros(6)
        if self.C1 == 0.0:
            model = lambda x, c0, c1, c2, c3, c4, c5: c0 + c1 * x + c2 * x ** 2 + c3 * x ** 3 + c4 * x ** 4 + c5 * x ** 5
            E = np.logspace(np.log10(self.cutoff * 2), np.log10(1), pts)
            r = rate_gen.Rate(E)
            self.clog, _ = scipy.optimize.curve_fit(model, np.log(E), np.log(r))

    def rate(self, Et):
        """ExplicitRate (ionization.cl:22-44) or ExplicitRateSeries (ionization.cl:71-97)."""
        if self.explicit:
            Emag = self.field_conv * np.abs(Et) + self.cutoff
            return self.rate_conv * self.C1 * Emag ** self.C2 * np.exp(self.C3 / Emag)
        logE = np.log(self.field_conv * np.abs(Et) + self.cutoff)
        c = self.clog
        return self.rate_conv * np.exp(c[0] + c[1] * logE + c[2] * logE * logE + c[3] * logE ** 3 + c[4] * logE ** 4 + c[5] * logE ** 5)


# ----------------------------------------------------------------------------------------------
# point operations
# ----------------------------------------------------------------------------------------------

def plasma_density(rate, ng, dt):
    """ComputePlasmaDensity (ionization.cl:127-155): the last time sample's rate is taken as zero and
    the trapezoid sum runs from high to low time index; ne = ng*(1-exp(-S))."""
    r = rate.copy()
    r[-1] = 0.0
    pair = 0.5 * (r[:-1] + r[1:]) * dt
    S = np.zeros_like(r)
    S[:-1] = np.cumsum(pair[::-1], axis=0)[::-1]
    return ng[None, ...] * (1.0 - np.exp(-S))


def soft_time_window(A, cutoff=4, width=64):
    """SoftTimeWindow (fft.cl:331-355), applied along axis 0."""
    Ni = A.shape[0]
    f = np.ones(Ni)
    i = np.arange(Ni)
    f[(i < cutoff) | (i > Ni - cutoff - 1)] = 0.0
    up = (i >= cutoff) & (i < cutoff + width)
    q = (i[up] - cutoff) / width
    f[up] *= 10 * q ** 3 - 15 * q ** 4 + 6 * q ** 5
    dn = (i <= Ni - cutoff - 1) & (i > Ni - cutoff - width - 1)
    q = (Ni - cutoff - 1 - i[dn]) / width
    f[dn] *= 10 * q ** 3 - 15 * q ** 4 + 6 * q ** 5
    return A * f[:, None, None]


def propagator_phase(kz, kg, z):
    """exp(i(kz+kg)z) including the decay from Im kz (uppe.cl:54-71)."""
    return np.exp(-kz.imag * z) * (np.cos((kz.real + kg) * z) + 1j * np.sin((kz.real + kg) * z))


def raman_chi(rotator, Et, ng, dt):
    """Rotational Raman susceptibility, AddChiUPPE (kernels/rotations.cl:85-129), FP64.

    For every j -> j-2 transition (j >= 2) the density-matrix element is driven by the field along the
    reference's time order (index Nt-1 down to 0, step n): with h = exp(i wdt / 2), wdt = W_j dt,
        rho_n = -i dt sum_{m < n} F_m h^(2m+1),   F = (dalpha / hbar) E^2 / 2,
        chi_n += sum_{n' <= n} 2 Im(T_j S_j rho_n' conj(h^(2n')) wdt) ng dalpha,
    S_j = 2 j (j-1) / (15 (2j-1)).  The reference multiplies the phasor by h twice per step; here
    the powers are formed directly, which agrees to rounding."""
    Nt = Et.shape[0]
    Er = Et[::-1]  # processing order n = Nt-1-k
    F = 0.5 * (rotator.dalpha / rotator.hbar) * Er ** 2
    n = np.arange(Nt, dtype=float)[:, None, None]
    chi = np.zeros_like(Et)
    for j in range(2, rotator.Wj.shape[0]):
        wdt = rotator.Wj[j] * dt
        S = 2.0 * j * (j - 1) / (15 * (2 * j - 1))
        h2n = np.exp(1j * wdt * n)            # h^(2n)
        a = F * h2n * np.exp(0.5j * wdt)      # F_m h^(2m+1)
        rho = -1j * dt * (np.cumsum(a, axis=0) - a)  # exclusive prefix
        term = rotator.Tj[j] * S * rho * np.conj(h2n) * wdt
        chi += np.cumsum(2 * term.imag * ng[None] * rotator.dalpha, axis=0)[::-1]
    return chi


class Medium:
    """Material (uppe_kernel.py:32-90): kz, kGalileo and the gas density plane at one z."""

    def __init__(self, grid, vol_dict, window_speed):
        self.g = grid
        self.vd = vol_dict
        self.chi = vol_dict["dispersion inside"].chi(grid.w).astype(np.cdouble)
        self.chi3 = vol_dict.get("chi3", 0.0)
        self.nref = vol_dict["density reference"]
        self.redchi3 = self.chi3 / self.nref
        self.vg = window_speed
        N = grid.N
        self.xp_eff = np.zeros((N[1], N[2], 8))
        if grid.cartesian:
            self.xp_eff[..., 1] = np.outer(grid.x1, np.ones(N[2]))
            self.xp_eff[..., 2] = np.outer(np.ones(N[1]), grid.x2)
        else:
            self.xp_eff[..., 1] = np.outer(grid.x1, np.cos(grid.x2))
            self.xp_eff[..., 2] = np.outer(grid.x1, np.sin(grid.x2))
        obj = vol_dict.get("object", None)
        if obj is not None and hasattr(obj, "GetRelDensity"):
            self.rel_density = obj.GetRelDensity
        else:
            lam = vol_dict["density lambda"]

            def rel(xp):
                r2 = np.einsum("...i,...i", xp[..., 1:3], xp[..., 1:3])
                return lam(xp[..., 1], xp[..., 2], xp[..., 3], r2)
            self.rel_density = rel

    def update(self, z):
        """UpdateMaterial (uppe_kernel.py:67-90)."""
        self.xp_eff[..., 3] = z
        dens = self.rel_density(self.xp_eff)
        chi0 = np.copy(self.chi)
        chi0[np.where(np.real(self.chi) > 0.0)] *= np.min(dens)
        chi0[np.where(np.real(self.chi) < 0.0)] *= np.max(dens)
        w2n2 = self.g.w ** 2 * (1 + chi0)
        kz = np.sqrt(0j + w2n2[..., None, None] - self.g.kr2[None, ...])
        kz[np.where(np.imag(kz) < 0)] *= -1
        kz[np.where(np.real(kz) == 0.0)] = 1.0
        self.kz = kz
        self.kg = -self.g.w[..., None, None] / self.vg
        self.ng = self.nref * dens
        self.chi0 = chi0


class Oracle:
    """One UPPE volume: the reference's ``track`` (uppe_kernel.py:333-424) restated in FP64 NumPy."""

    def __init__(self, vol_dict):
        self.vd = vol_dict
        N = tuple(vol_dict["wave grid"])
        p2 = [2 ** i for i in range(32)]
        if N[0] - 1 not in p2:
            raise ValueError("UPPE propagator requires 2**n+1 w-nodes")
        if N[1] not in p2:
            raise ValueError("UPPE propagator requires 2**n x-nodes")
        if N[2] not in p2:
            raise ValueError("UPPE propagator requires 2**n y-nodes")
        self.g = Grid(vol_dict)
        self.window_speed = vol_dict.get("window speed", 1.0)
        self.mat = Medium(self.g, vol_dict, self.window_speed)
        iz = vol_dict.get("ionizer", None)
        self.rates = RateCoefficients(iz) if iz is not None else None
        self.rotator = vol_dict.get("rotator", None)
        self.dphi = 0.4
        self.rel_amin = 1e-2
        g = self.g
        filt = np.ones(N[0])
        nl = vol_dict["nonlinear band"]
        filt[:int(nl[0] / g.dw)] = 0.0
        filt[int(nl[1] / g.dw):] = 0.0
        self.nl_filter = filt
        cond = np.ones(N[0])
        cond[:4] = 0.0
        self.conditioner = cond
        self.evals = 0

    # -- one right-hand side evaluation -------------------------------------------------------
    def update_current(self, Ew):
        """update_current (uppe_kernel.py:139-186): Ew is the real-space spectral E field."""
        g, mat = self.g, self.mat
        Nt = g.Nt
        Et = scipy.fft.irfft(Ew, n=Nt, axis=0, workers=_WORKERS)
        w = g.w[:, None, None]
        if self.rates is None:
            ne = np.zeros_like(Et)
            Jw = np.zeros(Ew.shape, np.cdouble)
        else:
            rate = self.rates.rate(Et)
            ne = plasma_density(rate, mat.ng, g.dt)
            ne = soft_time_window(ne, 4, 64)
            Jw = scipy.fft.rfft(ne * Et, axis=0, workers=_WORKERS)
            Jw = Jw / (0.1 - 1j * w)
        chi = mat.ng[None, ...] * mat.redchi3 * Et * Et
        if self.rotator is not None:  # uppe_kernel.py:174-176, before the Kerr term
            chi = chi + raman_chi(self.rotator, Et, mat.ng, g.dt)
        P = scipy.fft.rfft(chi * Et, axis=0, workers=_WORKERS)
        Jw = Jw + (-1j * w) * P
        Jw = Jw * self.nl_filter[:, None, None]
        return Jw, chi, ne, Et

    def load_source(self, q, zloc):
        """load_source (uppe_kernel.py:188-216) without the step estimate: returns S(q, z)."""
        mat = self.mat
        E = propagator_phase(mat.kz, mat.kg, zloc) * q
        E = 1j * mat.kz * E
        E = self.g.rspace(E)
        Jw, _, _, _ = self.update_current(E)
        Jw = self.g.kspace(Jw)
        self.evals += 1
        return 0.5j * propagator_phase(mat.kz, mat.kg, -zloc) * Jw / mat.kz.real

    def step_size(self, q, S, L, z, dzmin):
        """LoadModulus/LoadStepSize (paraxial.cl:27-58) and the clamps of uppe_kernel.py:217-232."""
        amin = self.rel_amin * np.max(np.abs(q))
        minRate = 0.5 * self.dphi / L
        den = q.real ** 2 + q.imag ** 2 + amin * amin
        alpha = (q.real * S.real + q.imag * S.imag) / den
        keff = (q.real * S.imag - q.imag * S.real) / den
        K = minRate + np.abs(keff) - alpha * (alpha < 0.0)
        dz = np.min(self.dphi / K)
        if dz < dzmin:
            dz = dzmin
        if z + dz > L:
            dz = L - z
        return dz

    def propagator(self, a, zi, zf, subcycles, dzmin):
        """propagator (uppe_kernel.py:260-331): classic RK4 on q = exp(-i(kz+kg)z) a."""
        g, mat = self.g, self.mat
        if g.w[0] != 0.0:
            raise ValueError("UPPE propagator requires frequency range [0,...]")
        L = (zf - zi) / subcycles
        q = g.kspace(a.astype(np.cdouble))
        cond = self.conditioner[:, None, None]
        steps = 0
        for sub in range(subcycles):
            z0 = zi + sub * L
            z = 0.0
            mat.update(z0 + 0.5 * L)
            while z < L and (z - L) ** 2 > (L / 1e6) ** 2:
                zl = z0 - zi + z
                qi = q
                k1 = self.load_source(q, zl)
                dz = self.step_size(q, k1, L, z, dzmin)
                qf = qi + (dz / 6) * k1
                q = (qi + (dz / 2) * k1) * cond
                k2 = self.load_source(q, zl + 0.5 * dz)
                qf = qf + (dz / 3) * k2
                q = (qi + (dz / 2) * k2) * cond
                k3 = self.load_source(q, zl + 0.5 * dz)
                qf = qf + (dz / 3) * k3
                q = (qi + dz * k3) * cond
                k4 = self.load_source(q, zl + dz)
                q = (qf + (dz / 6) * k4) * cond
                steps += 1
                z += dz
        return self.finish(q, zf - zi) + (steps,)

    def finish(self, q, zloc):
        """finish (uppe_kernel.py:234-258)."""
        mat = self.mat
        a = propagator_phase(mat.kz, mat.kg, zloc) * q
        a = self.g.rspace(a)
        E = 1j * mat.kz * a
        Jw, chi, ne, _ = self.update_current(E)
        return a, Jw, scipy.fft.rfft(chi, axis=0, workers=_WORKERS), scipy.fft.rfft(ne, axis=0, workers=_WORKERS)

    def track(self):
        """track (uppe_kernel.py:333-424) for the ``incoming wave`` route; returns (A, J, chiNL, ne, dom4d)."""
        vd, g = self.vd, self.g
        N = g.N
        A = np.zeros(N, np.cdouble)
        J = np.zeros(N, np.cdouble)
        chiNL = np.zeros(N, np.cdouble)
        ne = np.zeros(N, np.cdouble)
        A[..., 0] = vd["incoming wave"](g.w, g.x1, g.x2)
        subcycles = vd["subcycles"]
        steps = (N[3] - 1) * subcycles
        Lz = g.size[3]
        dens_nodes = cell_centers(-Lz / 2, Lz / 2, steps)
        fw = cell_walls(dens_nodes[0], dens_nodes[-1], steps)
        walls = np.linspace(-Lz / 2, Lz / 2, N[3])
        dom4d = np.concatenate((g.plot_ext, [fw[0], fw[-1]]))
        A0 = np.copy(A[..., 0])
        self.rk_steps = []
        for k in range(N[3] - 1):
            A0, J0, c0, n0, nsteps = self.propagator(A0, walls[k], walls[k + 1], subcycles, vd["minimum step"])
            self.rk_steps.append(nsteps)
            A[..., k + 1] = A0
            J[..., k + 1] = J0
            chiNL[..., k + 1] = c0
            ne[..., k + 1] = n0
        return A, J, chiNL, ne, dom4d


def track(vol_dict):
    return Oracle(vol_dict).track()
