"""Host side of the GB300 paraxial (envelope) propagator: a drop-in for SeaRay's
``modules/paraxial_kernel.py``.

``track(cl, xp, eikonal, vg, vol_dict)`` keeps the reference's signature, input-dictionary keys,
checks and return values (``paraxial_kernel.py:367-443``), so ``volume.nonuniform_volume.Propagate``
can call it where the volume's ``'propagator'`` is ``'paraxial'``.  The device work goes through the
same C ABI as the UPPE solver, with ``UppeConfig.envelope = 1`` (``include/searay_uppe.h``): the
transverse transforms, the RK4 bookkeeping and the adaptive step are shared; the operator, the
right-hand-side factor and the time-axis pass are the envelope solver's.  There is no CPU fallback.

The frequency axis holds 2^n absolute frequencies over the band.  As in the reference, the device
keeps it in FFT order (``np.fft.ifftshift``, ``paraxial_kernel.py:294-296``) and the outputs are
returned in ascending order (``:359-363``).

Extra, optional dictionary keys (ignored by the reference): ``'precision'`` as for ``uppe.track``.
"""
import logging

import numpy as np
import torch

from . import raywave
from .grid import VolumeGrid, cell_centers, cell_walls
from .ionization import RateCoefficients
from .uppe import DeviceGrid, TrackOutputs

_POW2 = [2 ** i for i in range(32)]


def _check_grid(N):
    """The grid checks of paraxial_kernel.py:393-398."""
    if N[0] not in _POW2:
        raise ValueError("Paraxial propagator requires 2**n w-nodes")
    if N[1] not in _POW2:
        raise ValueError("Paraxial propagator requires 2**n x-nodes")
    if N[2] not in _POW2:
        raise ValueError("Paraxial propagator requires 2**n y-nodes")


class Material:
    """Material of the paraxial solver (paraxial_kernel.py:29-91): the density plane, chi0(w) and the
    envelope tables f(w) = w^2 (1 + chi0 - ng^2) - w0^2 dn^2 - 2 w w0 ng dn, k0(w) = w0 dn + w ng
    (dn = n0 - ng), in FFT order; kz = (f - kperp^2) / (2 k0) is built on the device."""

    def __init__(self, dev, grid, coords, vol, chi, chi3, nref, w0, ng, n0, density_lambda=None):
        N = grid.N
        self.dev = dev
        self.grid = grid
        self.chi = np.fft.ifftshift(chi, axes=0)
        self.w = np.fft.ifftshift(grid.w, axes=0)
        self.redchi3 = chi3 / nref
        self.n_ref = nref
        self.w0, self.ng, self.n0 = w0, ng, n0
        self.xp_eff = np.zeros((N[1], N[2], 8))
        if coords == "cartesian":
            self.xp_eff[..., 1] = np.outer(grid.x1, np.ones(N[2]))
            self.xp_eff[..., 2] = np.outer(np.ones(N[1]), grid.x2)
        else:
            self.xp_eff[..., 1] = np.outer(grid.x1, np.cos(grid.x2))
            self.xp_eff[..., 2] = np.outer(grid.x1, np.sin(grid.x2))
        if vol is not None and hasattr(vol, "GetRelDensity"):
            self.rel_density = vol.GetRelDensity
        elif density_lambda is not None:
            def rel(xp):
                r2 = np.einsum("...i,...i", xp[..., 1:3], xp[..., 1:3])
                return density_lambda(xp[..., 1], xp[..., 2], xp[..., 3], r2)
            self.rel_density = rel
        else:
            raise ValueError("the volume needs an 'object' with GetRelDensity or a 'density lambda'")
        dn = n0 - ng
        self.k0 = np.ascontiguousarray(w0 * dn + self.w * ng, dtype=np.float64)

    def UpdateMaterial(self, z):
        self.xp_eff[..., 3] = z
        dens = self.rel_density(self.xp_eff)
        chi0 = np.copy(self.chi)
        chi0[np.where(np.real(self.chi) > 0.0)] *= np.min(dens)
        chi0[np.where(np.real(self.chi) < 0.0)] *= np.max(dens)
        w, w0, ng = self.w, self.w0, self.ng
        dn = self.n0 - ng
        fw = w ** 2 * (1 + chi0 - ng ** 2) - w0 ** 2 * dn ** 2 - 2 * w * w0 * ng * dn
        ngas = np.ascontiguousarray(self.n_ref * np.broadcast_to(dens, self.grid.N[1:3]), dtype=np.float64)
        return self.dev.set_material(np.asarray(fw, dtype=np.complex128), self.k0, ngas)


def propagator(dev, mat, a_dev, subcycles, zi, zf, outputs=None):
    """Advance a[w,x,y] (device, FFT frequency order) to the next diagnostic plane
    (paraxial_kernel.py:264-365) with adaptive steps and no minimum step.  Returns device tensors
    (A, J, chiNL_w, ne_w) in FFT order and the number of RHS evaluations."""
    L = (zf - zi) / subcycles
    dev.load_field(a_dev)
    iterations = 0
    for sub in range(subcycles):
        z0 = zi + sub * L
        z = 0.0
        mat.UpdateMaterial(z0 + 0.5 * L)
        while z < L and (z - L) ** 2 > (L / 1e6) ** 2:
            dz = dev.rk4_step(z0 - zi + z, L, z, 0.0)
            iterations += 1
            z += dz
    if outputs is None:
        outputs = tuple(dev.empty_field() for _ in range(4))
    A, J, chi, ne = outputs
    dev.finish(zf - zi, A, J, chi, ne)
    if dev.nonfinite():
        logging.warning("paraxial field holds NaN or Inf after propagating to z=%g", zf)
    return A, J, chi, ne, 4 * iterations


def track(cl, xp, eikonal, vg, vol_dict):
    """Propagate the paraxial volume's wave through its diagnostic planes (paraxial_kernel.py:367-443).

    :param cl: ignored (the reference's OpenCL bundle); the device is the current CUDA device.
    :param numpy.array xp: ray phase space (bundles, rays, 8).  Without an ``incoming wave`` the
        wave starts from the rays; at the end the rays are relaunched from the last plane (both
        modify xp, eikonal and vg in place, as the reference does).  May be None with an incoming wave.
    :param numpy.array eikonal: ray eikonal data (bundles, 4)
    :param numpy.array vg: ray group velocity (bundles, rays, 4)
    :param dict vol_dict: the volume's input dictionary
    :returns: A, J, chiNL, ne (complex128, shape ``wave grid``) and dom4d"""
    band = vol_dict["frequency band"]
    size = (band[1] - band[0],) + tuple(vol_dict["size"])
    N = tuple(vol_dict["wave grid"])
    diagnostic_steps = N[3] - 1
    subcycles = vol_dict["subcycles"]
    steps = diagnostic_steps * subcycles
    _check_grid(N)
    window_speed = vol_dict.get("window speed", 1.0)
    chi3 = vol_dict.get("chi3", 0.0)

    grid = VolumeGrid(vol_dict)
    field_grid = raywave.FieldGrid(grid)
    if "incoming wave" not in vol_dict:
        logging.info("Start paraxial propagation using ray data.")
        logging.warning("Polarization information is lost upon entering paraxial region.")
        first = raywave.boundary_fields(field_grid, xp[:, 0, :], eikonal, 1)
    else:
        logging.info("Start paraxial propagation using wave data")
        first = vol_dict["incoming wave"](grid.w, grid.x1, grid.x2)

    # reference frame of the envelope (paraxial_kernel.py:407-411)
    w0 = grid.w[int(N[0] / 2)]
    n0 = 1 / window_speed
    ng = 1 / window_speed

    chi = vol_dict["dispersion inside"].chi(grid.w).astype(np.cdouble)
    rates = None
    if vol_dict.get("ionizer", None) is not None:
        rates = RateCoefficients(vol_dict["ionizer"])

    dev = DeviceGrid(grid, vol_dict, rates, vol_dict.get("precision", "mixed"), envelope=True)
    try:
        dev.set_rotator(vol_dict.get("rotator", None))
        mat = Material(dev, grid, vol_dict["wave coordinates"], vol_dict.get("object", None), chi, chi3,
                       vol_dict["density reference"], w0, ng, n0, vol_dict.get("density lambda", None))
        dens_nodes = cell_centers(-size[3] / 2, size[3] / 2, steps)
        field_walls = cell_walls(dens_nodes[0], dens_nodes[-1], steps)
        diagnostic_walls = np.linspace(-size[3] / 2, size[3] / 2, N[3])
        dom4d = np.concatenate((grid.plot_ext, [field_walls[0], field_walls[-1]]))

        # the device keeps the frequency axis in FFT order; the outputs go back in ascending order
        res = TrackOutputs(N, first, shift=lambda t: torch.fft.fftshift(t, dim=0))
        a_dev = res.first_plane(order=lambda t: torch.fft.ifftshift(t, dim=0))
        outs = tuple(dev.empty_field() for _ in range(4))
        for k in range(diagnostic_steps):
            zi = diagnostic_walls[k]
            zf = diagnostic_walls[k + 1]
            logging.info("Advancing to diagnostic plane %d", k + 1)
            A0, J0, c0, n0_, evals = propagator(dev, mat, a_dev, subcycles, zi, zf, outs)
            logging.info("%d evaluations of j(w,kx,ky)", evals)
            res.store(k + 1, A0, J0, c0, n0_)
            a_dev, outs = A0, (dev.empty_field(), J0, c0, n0_)
        A, J, chiNL, ne = res.host()
    finally:
        dev.close()
    # relaunch the rays from the last plane (paraxial_kernel.py:438-442)
    if xp is not None:
        relaunch = raywave.relaunch_rays_full if vol_dict.get("full relaunch", False) else raywave.relaunch_rays
        relaunch(field_grid, xp, eikonal, vg, A[..., -1], size[3], vol_dict["dispersion inside"])
    return A, J, chiNL, ne, dom4d
