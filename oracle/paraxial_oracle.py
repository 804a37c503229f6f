"""FP64 CPU oracle for the paraxial (envelope) z-step — TEST INFRASTRUCTURE, never part of the
product path.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may import this
module, and only to check results against / as the timed CPU baseline.  The CUDA path in ``searay_gb300`` does
not import it and has no CPU fallback.

A NumPy restatement of SeaRay's paraxial propagator (``modules/paraxial_kernel.py``, kernels
``kernels/paraxial.cl``, the complex strip transforms and ``DtSpectral`` of ``kernels/fft.cl``,
``EnvelopeRate``/``EnvelopeRateSeries`` and ``ComputePlasmaDensity`` of ``kernels/ionization.cl``,
``AddChiParaxial`` of ``kernels/rotations.cl``), each step citing the reference line it follows.
It is pinned against the reference itself: ``tests/golden/make_golden.py`` runs the reference's
own unmodified ``paraxial_kernel.track`` with its OpenCL kernels compiled as C++
(``oracle/refshim``) and stores the outputs; ``tests/test_oracle_golden.py`` checks this module
against them.

Arrays use the reference layout: spectral ``[w][x|r][y|phi]`` complex128 on N0 = 2^n frequency
nodes in ascending order at the interfaces (``track``, ``propagator``) and in FFT order
(``np.fft.ifftshift``) inside, as ``propagator`` keeps them (paraxial_kernel.py:357-361).
"""
import numpy as np
import scipy.fft

from .uppe_oracle import Grid, Medium, RateCoefficients, _WORKERS, cell_centers, cell_walls, plasma_density


def raman_chi_envelope(rotator, Et, ng, dt):
    """Rotational Raman susceptibility of a complex envelope, AddChiParaxial (rotations.cl:30-78),
    FP64: the recurrence of AddChiUPPE with the drive F = (dalpha/hbar) |E|^2 / 4 (the cycle average
    of E^2 / 2), in the reference's time order n = Nt-1-k."""
    Nt = Et.shape[0]
    Er = Et[::-1]
    F = 0.5 * (rotator.dalpha / rotator.hbar) * 0.5 * (Er.real ** 2 + Er.imag ** 2)
    n = np.arange(Nt, dtype=float)[:, None, None]
    chi = np.zeros(Et.shape)
    for j in range(2, rotator.Wj.shape[0]):
        wdt = rotator.Wj[j] * dt
        S = 2.0 * j * (j - 1) / (15 * (2 * j - 1))
        h2n = np.exp(1j * wdt * n)
        a = F * h2n * np.exp(0.5j * wdt)
        rho = -1j * dt * (np.cumsum(a, axis=0) - a)
        term = rotator.Tj[j] * S * rho * np.conj(h2n) * wdt
        chi += np.cumsum(2 * term.imag * ng[None] * rotator.dalpha, axis=0)[::-1]
    return chi


class EnvelopeMedium(Medium):
    """Material of the paraxial solver (paraxial_kernel.py:29-91): the same density plane and chi0
    selection as UPPE's, with kz = (w^2 (1 + chi0 - ng^2) - w0^2 dn^2 - 2 w w0 ng dn - kperp^2) / (2 k0),
    k0 = w0 dn + w ng, dn = n0 - ng, all in FFT frequency order."""

    def __init__(self, grid, vol_dict, w0, ng, n0):
        super().__init__(grid, vol_dict, 1.0)
        self.chi = np.fft.ifftshift(self.chi, axes=0)
        self.wf = np.fft.ifftshift(grid.w, axes=0)
        self.w0, self.ngrp, self.n0 = w0, ng, n0

    def update(self, z):
        """UpdateMaterial (paraxial_kernel.py:67-91)."""
        self.xp_eff[..., 3] = z
        dens = self.rel_density(self.xp_eff)
        chi0 = np.copy(self.chi)
        chi0[np.where(np.real(self.chi) > 0.0)] *= np.min(dens)
        chi0[np.where(np.real(self.chi) < 0.0)] *= np.max(dens)
        w, w0, ng = self.wf, self.w0, self.ngrp
        dn = self.n0 - ng
        fw = w ** 2 * (1 + chi0 - ng ** 2) - w0 ** 2 * dn ** 2 - 2 * w * w0 * ng * dn
        k0 = w0 * dn + w * ng
        self.fw, self.k0 = fw, k0
        self.kz = 0.5 * (fw[:, None, None] - self.g.kr2[None, ...]) / k0[:, None, None]
        self.ng = self.nref * dens
        self.chi0 = chi0


class ParaxialOracle:
    """One paraxial volume: the reference's ``track`` (paraxial_kernel.py:367-443) in FP64 NumPy."""

    def __init__(self, vol_dict):
        self.vd = vol_dict
        N = tuple(vol_dict["wave grid"])
        p2 = [2 ** i for i in range(32)]
        if N[0] not in p2:
            raise ValueError("Paraxial propagator requires 2**n w-nodes")
        if N[1] not in p2:
            raise ValueError("Paraxial propagator requires 2**n x-nodes")
        if N[2] not in p2:
            raise ValueError("Paraxial propagator requires 2**n y-nodes")
        self.g = Grid(vol_dict)
        g = self.g
        ws = vol_dict.get("window speed", 1.0)
        self.w0 = g.w[N[0] // 2]                     # paraxial_kernel.py:407
        self.n0 = 1 / ws
        self.ngrp = 1 / ws
        self.mat = EnvelopeMedium(g, vol_dict, self.w0, self.ngrp, self.n0)
        iz = vol_dict.get("ionizer", None)
        self.rates = RateCoefficients(iz) if iz is not None else None
        self.rotator = vol_dict.get("rotator", None)
        # Source (paraxial_kernel.py:93-111)
        bandwidth = 1.0 if N[0] == 1 else (np.max(g.w) - np.min(g.w)) * (1 + 1 / (N[0] - 1))
        self.dt = 2 * np.pi / bandwidth
        self.dphi = 0.4
        self.rel_amin = 1e-2
        self.evals = 0

    # -- one right-hand side evaluation -------------------------------------------------------
    def update_current(self, Aw):
        """update_current (paraxial_kernel.py:124-172): Aw is the real-space spectral vector potential
        in FFT order; returns J (spectral, FFT order), chi(t), ne(t), E(t)."""
        mat = self.mat
        w = mat.wf[:, None, None]
        Et = scipy.fft.ifft(1j * w * Aw, axis=0, workers=_WORKERS)    # DtSpectral(-1), IFFT
        At = scipy.fft.ifft(Aw, axis=0, workers=_WORKERS)
        ne = np.zeros(Et.shape)
        chi = np.zeros(Et.shape)
        if self.rates is not None:                                   # EnvelopeRate*, ComputePlasmaDensity
            ne = plasma_density(self.rates.rate(Et), mat.ng, self.dt)
        if self.rotator is not None:
            chi = chi + raman_chi_envelope(self.rotator, Et, mat.ng, self.dt)
        chi = chi + 0.75 * mat.ng[None, ...] * mat.redchi3 * (Et.real ** 2 + Et.imag ** 2)   # paraxial.cl:124-138
        P = chi * Et                                                 # SourcePolarization
        J = scipy.fft.fft(P, axis=0, workers=_WORKERS)
        J = -1j * w * J                                              # DtSpectral(+1)
        J = scipy.fft.ifft(J, axis=0, workers=_WORKERS)
        J = J + ne * (0.25 * (At.real ** 2 + At.imag ** 2) - 1.0) * At   # AddPlasmaCurrent (paraxial.cl:110-122)
        J = scipy.fft.fft(J, axis=0, workers=_WORKERS)
        return J, chi, ne, Et

    def load_source(self, q, zloc):
        """load_source (paraxial_kernel.py:174-218) without the step estimate: S(q, z)."""
        mat = self.mat
        A = np.exp(1j * mat.kz * zloc) * q                            # PropagateLinear
        A = self.g.rspace(A)
        J, _, _, _ = self.update_current(A)
        J = self.g.kspace(J)
        self.evals += 1
        return 0.5j * np.exp(-1j * mat.kz * zloc) * J / mat.k0[:, None, None]   # CurrentToODERHS

    def step_size(self, q, S, L, z):
        """LoadModulus/LoadStepSize (paraxial.cl:27-58) and the clamp of paraxial_kernel.py:200-212
        (no minimum step)."""
        amin = self.rel_amin * np.max(np.abs(q))
        minRate = 0.5 * self.dphi / L
        den = q.real ** 2 + q.imag ** 2 + amin * amin
        alpha = (q.real * S.real + q.imag * S.imag) / den
        keff = (q.real * S.imag - q.imag * S.real) / den
        K = minRate + np.abs(keff) - alpha * (alpha < 0.0)
        dz = np.min(self.dphi / K)
        if z + dz > L:
            dz = L - z
        return dz

    def propagator(self, a, zi, zf, subcycles):
        """propagator (paraxial_kernel.py:264-365): classic RK4 on q = exp(-i kz z) a; a and the
        outputs in ascending frequency order."""
        mat = self.mat
        L = (zf - zi) / subcycles
        q = self.g.kspace(np.fft.ifftshift(a.astype(np.cdouble), axes=0))
        steps = 0
        for sub in range(subcycles):
            z0 = zi + sub * L
            z = 0.0
            mat.update(z0 + 0.5 * L)
            while z < L and (z - L) ** 2 > (L / 1e6) ** 2:
                zl = z0 - zi + z
                qi = q
                k1 = self.load_source(q, zl)
                dz = self.step_size(q, k1, L, z)
                qf = qi + (dz / 6) * k1
                q = qi + (dz / 2) * k1
                k2 = self.load_source(q, zl + 0.5 * dz)
                qf = qf + (dz / 3) * k2
                q = qi + (dz / 2) * k2
                k3 = self.load_source(q, zl + 0.5 * dz)
                qf = qf + (dz / 3) * k3
                q = qi + dz * k3
                k4 = self.load_source(q, zl + dz)
                q = qf + (dz / 6) * k4
                steps += 1
                z += dz
        A, J, chi, ne = self.finish(q, zf - zi)
        sh = lambda x: np.fft.fftshift(x, axes=0)
        return sh(A), sh(J), sh(chi), sh(ne), steps

    def finish(self, q, zloc):
        """finish (paraxial_kernel.py:220-262): A, J, fft(chi), fft(ne) in FFT order."""
        A = self.g.rspace(np.exp(1j * self.mat.kz * zloc) * q)
        J, chi, ne, _ = self.update_current(A)
        return A, J, scipy.fft.fft(chi, axis=0, workers=_WORKERS), scipy.fft.fft(ne, axis=0, workers=_WORKERS)

    def track(self):
        """track (paraxial_kernel.py:367-443) for the ``incoming wave`` route."""
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
        fwl = cell_walls(dens_nodes[0], dens_nodes[-1], steps)
        walls = np.linspace(-Lz / 2, Lz / 2, N[3])
        dom4d = np.concatenate((g.plot_ext, [fwl[0], fwl[-1]]))
        A0 = np.copy(A[..., 0])
        self.rk_steps = []
        for k in range(N[3] - 1):
            A0, J0, c0, n0, nsteps = self.propagator(A0, walls[k], walls[k + 1], subcycles)
            self.rk_steps.append(nsteps)
            A[..., k + 1] = A0
            J[..., k + 1] = J0
            chiNL[..., k + 1] = c0
            ne[..., k + 1] = n0
        return A, J, chiNL, ne, dom4d


def track(vol_dict):
    return ParaxialOracle(vol_dict).track()
