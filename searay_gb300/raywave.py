"""Coupling between rays and the UPPE wave grid, on the host in FP64 as in SeaRay.

* ``boundary_fields``: the complex amplitude that a set of rays carries onto the first plane of the
  wave grid, SeaRay's ``GetBoundaryFields`` (Cartesian ``modules/caustic_tools.py:98-116``,
  cylindrical ``:237-254``) with ``grid_tools.GridFromInterpolation`` (``modules/grid_tools.py:
  148-177``) and ``CylGridFromInterpolation`` (``:112-146``).
* ``relaunch_rays``: the simplified relaunch, ``RelaunchRays`` (``caustic_tools.py:181-205``,
  ``:311-338``): rays keep frequency and transverse position, leave along z, and take amplitude and
  phase from the last plane.
* ``relaunch_rays_full``: ``RelaunchRays1`` (``:118-179``, ``:256-309``): the transverse wave
  vector from a*grad(a^*), the phase from it (a Poisson solve on Cartesian grids, a radial integral
  on cylindrical grids), both sampled at the rays.

All of them act on small ray sets once per volume, so they run with NumPy and SciPy like the
reference's.  ``xp``, ``eikonal`` and ``vg`` are modified in place, as SeaRay's are.  Layouts:
``xp`` (bundles, 4, 8) = (t, x, y, z, w, kx, ky, kz) per ray, ray 0 the primary of its bundle;
``eikonal`` (bundles, 4) = (phase, a_x, a_y, a_z); ``vg`` (bundles, 4, 4).
"""
import logging

import numpy as np
import scipy.integrate
import scipy.interpolate

from .grid import cell_walls, fd_wavenumber


class FieldGrid:
    """The (w, x1, x2) nodes of one UPPE volume as SeaRay's field tools present them
    (``CausticTool.__init__`` ``caustic_tools.py:26-38``, ``GetGridInfo`` ``:88-97``, ``:222-229``).

    ``grid`` is a :class:`searay_gb300.grid.VolumeGrid`; the tool is centred on the transverse
    origin, as ``uppe_kernel.track`` builds it (``uppe_kernel.py:372-375``)."""

    def __init__(self, grid):
        self.grid = grid
        self.cartesian = grid.cartesian
        self.N = tuple(grid.N)
        band = grid.band
        self.center = np.array([0.5 * (band[0] + band[1]), 0.0, 0.0, 0.0])
        self.band_width = band[1] - band[0]
        self.wn, self.xn, self.yn = grid.w, grid.x1, grid.x2
        # transverse cell sizes of the Fourier tool (caustic_tools.py:36, grid_tools.py:236-244)
        self.dq = (grid.size[1] / self.N[1], grid.size[2] / self.N[2])

    def time_window(self):
        return 2 * np.pi * self.N[0] / self.band_width

    def cyl_coords(self, xp):
        """(rho, phi) of ray positions about the tool's centre (``caustic_tools.py:232-236``)."""
        d = xp[..., 1:4] - self.center[1:4]
        return np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2), np.arctan2(d[..., 1], d[..., 0])

    def clip_rays(self, xp):
        """Bundles whose every ray lies inside the Cartesian grid in (w, x, y)
        (``caustic_tools.py:63-74``)."""
        w, x, y = xp[..., 4], xp[..., 1], xp[..., 2]

        def inside(v, nodes):
            return np.logical_or(np.logical_and(v >= nodes[0], v <= nodes[-1]), nodes.shape[0] == 1)

        ok = inside(w, self.wn) & inside(x, self.xn) & inside(y, self.yn)
        return np.where(np.all(ok, axis=1))[0]


# ---- regular grid <-> scattered data (grid_tools.py:81-177) ----

def _bin_walls(nodes):
    return cell_walls(nodes[0], nodes[-1], nodes.shape[0])


def grid_from_rays_cartesian(w, x, y, vals, wn, xn, yn, fill=0.0):
    """Per frequency bin, cubic interpolation of the scattered (x, y, vals) onto the (xn, yn)
    grid, sampled just inside its nodes (x 0.9999) so that rays on the outer nodes count
    (``GridFromInterpolation``).  Every frequency bin needs rays."""
    ww = _bin_walls(wn)
    xg = 0.9999 * np.outer(xn, np.ones(yn.shape[0]))
    yg = 0.9999 * np.outer(np.ones(xn.shape[0]), yn)
    out = np.zeros((wn.shape[0], xn.shape[0], yn.shape[0]))
    for i in range(wn.shape[0]):
        sel = np.where(np.logical_and(w >= ww[i], w < ww[i + 1]))
        if sel[0].shape[0] == 0:
            # the reference logs this as critical and ends the process
            raise ValueError(f"no rays found in frequency bin {i}: the rays must cover every w node of the grid")
        pts = np.stack((x[sel], y[sel]), axis=-1)
        out[i] = scipy.interpolate.griddata(pts, vals[sel], (xg, yg), method="cubic", fill_value=fill)
    return out


def grid_from_rays_cylindrical(w, rho, phi, vals, wn, rn, pn):
    """Frequency and azimuth binned, linear interpolation in rho inside each bin; below the
    smallest ray radius the value of that ray, beyond the largest zero; empty bins zero
    (``CylGridFromInterpolation``)."""
    ww, wp = _bin_walls(wn), _bin_walls(pn)
    out = np.zeros((wn.shape[0], rn.shape[0], pn.shape[0]))
    for i in range(wn.shape[0]):
        in_w = np.logical_and(w >= ww[i], w < ww[i + 1])
        for j in range(pn.shape[0]):
            sel = np.where(np.logical_and(in_w, np.logical_and(phi >= wp[j], phi < wp[j + 1])))
            if sel[0].shape[0] == 0:
                continue
            r, v = rho[sel], vals[sel]
            inner = v[np.argmin(r)]
            f = scipy.interpolate.interp1d(r, v, kind="linear", bounds_error=False, fill_value=(inner, 0.0))
            out[i, :, j] = f(rn)
    return out


def sample_grid(w, x, y, wn, xn, yn, data):
    """Trilinear sampling of regular (w, x, y) data at scattered points, extrapolating outside;
    a grid with one y node is widened to two identical planes spanning the points' y range
    (``DataFromGrid``)."""
    if wn.shape[0] == 1:
        raise ValueError("Cannot relaunch rays with monochromatic data.")
    if xn.shape[0] == 1:
        raise ValueError("Missing spatial dimension x.")
    if yn.shape[0] == 1:
        ynodes = np.linspace(np.min(y), np.max(y), 2)
        data = np.concatenate((data, data), axis=2)
    else:
        ynodes = yn
    interp = scipy.interpolate.RegularGridInterpolator((wn, xn, ynodes), data, bounds_error=False,
                                                       fill_value=None)
    return interp(np.stack((w, x, y), axis=-1))


def _with_ghost_cell(a, nodes, axis):
    """One cell prepended along ``axis`` (a copy of the first), its node one spacing below
    (``AddGhostCells``)."""
    first = np.take(a, [0], axis=axis)
    return np.concatenate((first, a), axis=axis), np.concatenate(([2 * nodes[0] - nodes[1]], nodes))


# ---- rays -> wave ----

def boundary_fields(fg, xps, eiks, c):
    """Eikonal field component ``c`` (1..3) of the primary rays ``xps`` (bundles, 8) with eikonal
    data ``eiks`` (bundles, 4) on the (w, x1, x2) grid of ``fg`` (a :class:`FieldGrid`): amplitude
    times exp(i psi), with the phase referred to the time of the strongest ray and the centre of the
    time window (``GetBoundaryFields``)."""
    w = xps[:, 4]
    strongest = np.argmax(eiks[:, 1] ** 2 + eiks[:, 2] ** 2)
    psi_rays = eiks[:, 0] - w * (xps[strongest, 0] + 0.5 * fg.time_window())
    if fg.cartesian:
        d = xps[:, 1:4] - fg.center[1:4]
        amp = grid_from_rays_cartesian(w, d[:, 0], d[:, 1], eiks[:, c], fg.wn, fg.xn, fg.yn)
        psi = grid_from_rays_cartesian(w, d[:, 0], d[:, 1], psi_rays, fg.wn, fg.xn, fg.yn)
    else:
        rho, phi = fg.cyl_coords(xps)
        phi = np.where(phi > 0.9999 * np.pi, phi - 2 * np.pi, phi)  # keep -pi rather than +pi
        amp = grid_from_rays_cylindrical(w, rho, phi, eiks[:, c], fg.wn, fg.xn, fg.yn)
        psi = grid_from_rays_cylindrical(w, rho, phi, psi_rays, fg.wn, fg.xn, fg.yn)
    return amp * np.exp(1j * psi)


# ---- wave -> rays ----

def relaunch_rays(fg, xp, eikonal, vg, a, L, material):
    """Simplified relaunch from the last plane's vector potential ``a`` (w, x1, x2): rays on the grid
    keep w and transverse position, point along z, advance by L at the medium's group velocity and
    take |a| and arg(a) there (``RelaunchRays``)."""
    logging.warning("Using simplified ray relaunch; only valid for close couplings.")
    wn, xn, yn = fg.wn, fg.xn, fg.yn
    if fg.cartesian:
        hit = fg.clip_rays(xp)
        w = xp[hit, :, 4]
        x1, x2 = xp[hit, :, 1], xp[hit, :, 2]
    else:
        rho, phi = fg.cyl_coords(xp)
        w_in = np.logical_and(xp[:, 0, 4] >= wn[0], xp[:, 0, 4] <= wn[-1])
        hit = np.where(np.logical_and(rho[:, 0] <= xn[-1], w_in))[0]
        w = xp[hit, :, 4]
        x1, x2 = rho[hit, :], phi[hit, :]
    xp[hit, :, 5] = 0.0
    xp[hit, :, 6] = 0.0
    xp[hit, :, 7] = w
    vg[hit, ...] = xp[hit, ..., 4:8] / xp[hit, ..., 4:5]
    xp[hit, :, 0] += L / material.GroupVelocityMagnitude(w)
    xp[hit, :, 3] += L
    phase = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, np.angle(a))
    if not fg.cartesian:
        phase = w[:, 0] * xp[hit, 0, 0] + phase
    eikonal[hit, 0] = phase
    eikonal[hit, 1] = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, np.abs(a))
    eikonal[hit, 2] = 0.0
    eikonal[hit, 3] = 0.0


def _transverse_k(a, d, axis, eps):
    """Local transverse wave number Re(-i a d(a*)/dq) / |a|^2 without unwrapping the phase."""
    g = a * np.gradient(np.conj(a), d, axis=axis)
    return np.real(0.5j * (g - np.conj(g))) / (eps + np.abs(a)) ** 2


def relaunch_rays_full(fg, xp, eikonal, vg, a, L, material):
    """Relaunch with the wave's local transverse wave vector and phase (``RelaunchRays1``).  The
    medium is taken as vacuum for the ray advance, as in the reference."""
    wn, xn, yn = fg.wn, fg.xn, fg.yn
    eps = np.max(np.abs(a)) * 1e-6
    if fg.cartesian:
        if xn.shape[0] > 1:
            kx = _transverse_k(a, xn[1] - xn[0], 1, eps)
        else:
            kx = np.zeros(a.shape)
        if yn.shape[0] > 1:
            ky = _transverse_k(a, yn[1] - yn[0], 2, eps)
        else:
            ky = np.zeros(a.shape)
        # phase from laplacian(phase) = div(k) in the finite-difference Fourier basis
        ikx = 1j * np.outer(fd_wavenumber(fg.N[1], fg.dq[0]), np.ones(kx.shape[2]))
        iky = 1j * np.outer(np.ones(ky.shape[1]), fd_wavenumber(fg.N[2], fg.dq[1]))
        div = ikx * np.fft.fft(np.fft.fft(kx, axis=1), axis=2) + iky * np.fft.fft(np.fft.fft(ky, axis=1), axis=2)
        lap = ikx ** 2 + iky ** 2
        div[:, 0, 0] = 0.0
        lap[0, 0] = 1.0
        phase = np.real(np.fft.ifft(np.fft.ifft(div / lap, axis=2), axis=1))
        hit = fg.clip_rays(xp)
        w = xp[hit, :, 4]
        x1, x2 = xp[hit, :, 1], xp[hit, :, 2]
        k1 = sample_grid(w, x1, x2, wn, xn, yn, kx)
        k2 = sample_grid(w, x1, x2, wn, xn, yn, ky)
        over = np.where(k1 ** 2 + k2 ** 2 >= w ** 2)
        k1[over] = 0.0
        k2[over] = 0.0
        xp[hit, :, 5] = k1
        xp[hit, :, 6] = k2
    else:
        a, xg = _with_ghost_cell(a, xn, 1)
        if xg.shape[0] > 1:
            dr = xg[1] - xg[0]
            kr_grid = _transverse_k(a, dr, 1, eps)
        else:
            dr = 1.0
            kr_grid = np.zeros(a.shape)
        phase = scipy.integrate.cumulative_trapezoid(kr_grid, dx=dr, axis=1, initial=0.0)
        phase -= 0.25 * kr_grid[:, (0,), :] * dr
        rho, phi = fg.cyl_coords(xp)
        hit = np.where(np.logical_and(rho[:, 0] < xg[-1], xp[:, 0, 4] < wn[-1]))[0]
        w = xp[hit, :, 4]
        x1, x2 = rho[hit, :], phi[hit, :]
        try:
            kr = sample_grid(w, x1, x2, wn, xg, yn, kr_grid)
        except Exception:  # as the reference: a failed sample leaves the rays radial-free
            kr = np.zeros(x2.shape)
        kr[np.where(kr ** 2 >= w ** 2)] = 0.0
        xp[hit, :, 5] = kr * np.cos(x2)
        xp[hit, :, 6] = kr * np.sin(x2)
        xn = xg
    xp[hit, :, 7] = np.sqrt(w ** 2 - xp[hit, :, 5] ** 2 - xp[hit, :, 6] ** 2)
    vg[hit, ...] = xp[hit, ..., 4:8] / xp[hit, ..., 4:5]
    speed = np.sqrt(vg[hit, :, 1] ** 2 + vg[hit, :, 2] ** 2 + vg[hit, :, 3] ** 2)
    xp[hit, :, 0] += L / speed
    xp[hit, :, 3] += L
    if fg.cartesian:
        eikonal[hit, 0] = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, phase)
        eikonal[hit, 1] = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, np.abs(a))
    else:
        try:
            eikonal[hit, 0] = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, phase)
            eikonal[hit, 1] = sample_grid(w[:, 0], x1[:, 0], x2[:, 0], wn, xn, yn, np.abs(a))
        except Exception:  # as the reference: leave the eikonal data as they were
            pass
    eikonal[hit, 2] = 0.0
    eikonal[hit, 3] = 0.0
