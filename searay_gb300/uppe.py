"""Host side of the GB300 UPPE propagator: a drop-in for SeaRay's ``modules/uppe_kernel.py``.

``track(cl, xp, eikonal, vg, vol_dict)`` keeps the reference's signature, input-dictionary keys,
checks and return values (``uppe_kernel.py:333-424``), so ``volume.nonuniform_volume.Propagate``
(``modules/volume.py:606-612``) can call it in place of ``uppe_kernel.track``.  The device work
goes through the C ABI of ``libsearay_uppe.so`` (``include/searay_uppe.h``); there is no CPU
fallback.  Device memory and the stream come from PyTorch.

Extra, optional dictionary keys (ignored by the reference):
  ``'precision'``: ``'mixed'`` (default: FP32 transforms and sources, float-float phase and
  density scan) or ``'fp32'`` (plain FP32 everywhere).
"""
import ctypes
import logging

import numpy as np
import torch

from . import _native, raywave
from .grid import VolumeGrid, cell_centers, cell_walls
from .ionization import RateCoefficients

_POW2 = [2 ** i for i in range(32)]


def _check_grid(N):
    """The grid checks of uppe_kernel.py:354-360."""
    if N[0] - 1 not in _POW2:
        raise ValueError("UPPE propagator requires 2**n+1 w-nodes")
    if N[1] not in _POW2:
        raise ValueError("UPPE propagator requires 2**n x-nodes")
    if N[2] not in _POW2:
        raise ValueError("UPPE propagator requires 2**n y-nodes")


class DeviceGrid:
    """A C handle for one volume grid plus its device field buffers (Source of uppe_kernel.py:92-129).

    envelope=True makes it the paraxial envelope solver's (Source of paraxial_kernel.py:93-122): the
    frequency axis goes to the device in FFT order, dt = 2 pi / bandwidth, no NL band."""

    def __init__(self, grid, vol_dict, rates=None, precision="mixed", stream=None, envelope=False):
        lib = _native.lib()
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 UPPE propagator needs a CUDA device")
        self.grid = grid
        self.N = grid.N
        self.envelope = bool(envelope)
        nl = (0.0, (grid.N[0] + 1) * abs(grid.dw)) if envelope else vol_dict["nonlinear band"]
        cfg = _native.UppeConfig()
        cfg.n0, cfg.n1, cfg.n2 = grid.N[0], grid.N[1], grid.N[2]
        cfg.radial_modes = 0 if grid.cartesian else grid.Nk
        cfg.cylindrical = 0 if grid.cartesian else 1
        if precision not in ("mixed", "fp32"):
            raise ValueError("precision must be 'mixed' or 'fp32'")
        cfg.precision = _native.PREC_MIXED if precision == "mixed" else _native.PREC_FP32
        cfg.dt = grid.dt
        cfg.chi3_over_nref = vol_dict.get("chi3", 0.0) / vol_dict["density reference"]
        cfg.nl_cut_on = int(nl[0] / grid.dw)
        cfg.nl_cut_off = int(nl[1] / grid.dw)
        if envelope:
            N0 = grid.N[0]
            bandwidth = 1.0 if N0 == 1 else (np.max(grid.w) - np.min(grid.w)) * (1 + 1 / (N0 - 1))
            cfg.dt = 2 * np.pi / bandwidth  # paraxial_kernel.py:98-103
            cfg.nl_cut_on, cfg.nl_cut_off = 0, N0
            cfg.envelope = 1
        cfg.damping = 0.1
        cfg.window_cutoff = 4
        cfg.window_width = 64
        cfg.field_cutoff = 1e-3
        if rates is None:
            cfg.rate_form = _native.RATE_NONE
        else:
            cfg.field_conv = rates.field_conv
            cfg.rate_conv = rates.rate_conv
            cfg.field_cutoff = rates.cutoff
            if rates.explicit:
                cfg.rate_form = _native.RATE_EXPLICIT
                cfg.c_pre, cfg.c_pow, cfg.c_exp = rates.C1, rates.C2, rates.C3
            else:
                cfg.rate_form = _native.RATE_SERIES
                for i in range(6):
                    cfg.clog[i] = float(rates.clog[i])
        self.cfg = cfg
        h = ctypes.c_void_p()
        _native.check(lib.uppe_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.lib = lib
        s = torch.cuda.current_stream() if stream is None else stream
        self.stream = s
        self._check(lib.uppe_set_stream(h, ctypes.c_void_p(s.cuda_stream)))
        w = np.ascontiguousarray(np.fft.ifftshift(grid.w) if envelope else grid.w, dtype=np.float64)
        kr2 = np.ascontiguousarray(grid.kr2, dtype=np.float64)
        H = None if grid.H is None else np.ascontiguousarray(grid.H, dtype=np.float64)
        lam = None if grid.Lambda is None else np.ascontiguousarray(grid.Lambda, dtype=np.float64)
        self._check(lib.uppe_set_grid(h, _native.dptr(w), _native.dptr(kr2), _native.dptr(H), _native.dptr(lam)))
        self._last_material = None

    def _check(self, rc):
        return _native.check(rc, self.h)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.uppe_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- device calls ----
    def set_material(self, w2n2, kg, ng):
        key = (w2n2.tobytes(), kg.tobytes(), ng.tobytes())
        if key == self._last_material:
            return False
        w2n2 = np.ascontiguousarray(np.stack([w2n2.real, w2n2.imag], axis=-1).reshape(-1), dtype=np.float64)
        self._check(self.lib.uppe_set_material(self.h, _native.dptr(w2n2), _native.dptr(np.ascontiguousarray(kg, dtype=np.float64)),
                                               _native.dptr(np.ascontiguousarray(ng, dtype=np.float64))))
        self._last_material = key
        return True

    def load_field(self, a_dev):
        assert a_dev.dtype == torch.complex64 and a_dev.is_contiguous() and tuple(a_dev.shape) == tuple(self.N[:3])
        self._check(self.lib.uppe_load_field(self.h, ctypes.c_void_p(a_dev.data_ptr())))

    def rk4_step(self, z_phase, L, z_sub, dzmin):
        dz = ctypes.c_double()
        self._check(self.lib.uppe_rk4_step(self.h, z_phase, L, z_sub, dzmin, ctypes.byref(dz)))
        return dz.value

    def finish(self, z_phase, A=None, J=None, chi=None, ne=None):
        p = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        self._check(self.lib.uppe_finish(self.h, z_phase, p(A), p(J), p(chi), p(ne)))

    def eval_rhs(self, q_dev, z_phase, S_dev):
        self._check(self.lib.uppe_eval_rhs(self.h, ctypes.c_void_p(q_dev.data_ptr()), z_phase, ctypes.c_void_p(S_dev.data_ptr())))

    def get_field(self, q_dev):
        self._check(self.lib.uppe_get_field(self.h, ctypes.c_void_p(q_dev.data_ptr())))

    def nonfinite(self):
        flag = ctypes.c_int()
        self._check(self.lib.uppe_check_finite(self.h, ctypes.byref(flag)))
        return bool(flag.value)

    # ---- adjoint ----
    def set_chi3(self, chi3_over_nref):
        self._check(self.lib.uppe_set_chi3(self.h, float(chi3_over_nref)))

    def set_rotator(self, rotator):
        """Rotational Raman response from a Rotator (this package's or SeaRay's own: the attributes
        Wj, Tj, dalpha, hbar); None removes it."""
        if rotator is None:
            self._check(self.lib.uppe_set_rotator(self.h, 0, None, None, 0.0, 0.0))
            return
        Tj = np.ascontiguousarray(rotator.Tj, dtype=np.float64)
        Wj = np.ascontiguousarray(np.asarray(rotator.Wj, dtype=np.cdouble).view(np.float64))
        if Wj.shape[0] != 2 * Tj.shape[0]:
            raise ValueError("rotator: Wj and Tj differ in length")
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.uppe_set_rotator(self.h, int(Tj.shape[0]), Tj.ctypes.data_as(dp), Wj.ctypes.data_as(dp),
                                              float(rotator.dalpha), float(rotator.hbar)))

    def set_field(self, q_dev):
        self._check(self.lib.uppe_set_field(self.h, ctypes.c_void_p(q_dev.data_ptr())))

    def adjoint_step(self, q0_dev, lam_out_dev, lam_in_dev, z_phase, dz, want_dchi3=True):
        """VJP of one fixed RK4 step; returns d(loss)/d(chi3/nref) of the step (None when not asked,
        which also avoids the host read)."""
        d = ctypes.c_double(0.0)
        self._check(self.lib.uppe_adjoint_rk4_step(self.h, ctypes.c_void_p(q0_dev.data_ptr()),
                                                   ctypes.c_void_p(lam_out_dev.data_ptr()),
                                                   ctypes.c_void_p(lam_in_dev.data_ptr()), z_phase, dz,
                                                   ctypes.byref(d) if want_dchi3 else None))
        return d.value if want_dchi3 else None

    def rk4_step_keep(self, z_phase, dz):
        """One fixed RK4 step of the held field that keeps its stage fields for adjoint_step_kept
        (the result equals rk4_step's with dzmin = L - z_sub = dz)."""
        self._check(self.lib.uppe_rk4_step_keep(self.h, z_phase, dz))

    def adjoint_step_kept(self, lam_out_dev, lam_in_dev, want_dchi3=True):
        """VJP of the step last taken by rk4_step_keep, without recomputing its stage states."""
        d = ctypes.c_double(0.0)
        self._check(self.lib.uppe_adjoint_rk4_step_kept(self.h, ctypes.c_void_p(lam_out_dev.data_ptr()),
                                                        ctypes.c_void_p(lam_in_dev.data_ptr()),
                                                        ctypes.byref(d) if want_dchi3 else None))
        return d.value if want_dchi3 else None

    def adjoint_load(self, lam_q_dev, lam_a_dev):
        self._check(self.lib.uppe_adjoint_load(self.h, ctypes.c_void_p(lam_q_dev.data_ptr()),
                                               ctypes.c_void_p(lam_a_dev.data_ptr())))

    def adjoint_finish(self, z_phase, lam_A_dev, lam_q_dev):
        self._check(self.lib.uppe_adjoint_finish(self.h, z_phase, ctypes.c_void_p(lam_A_dev.data_ptr()),
                                                 ctypes.c_void_p(lam_q_dev.data_ptr())))

    def finish_field(self, z_phase, A_dev):
        """The field output of uppe_finish only (A = T^-1 exp(i(kz+kg)z) q)."""
        self._check(self.lib.uppe_finish(self.h, z_phase, ctypes.c_void_p(A_dev.data_ptr()), None, None, None))

    def profile(self, enable):
        self._check(self.lib.uppe_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self):
        ms = (ctypes.c_double * _native.NCLASS)()
        cnt = (ctypes.c_longlong * _native.NCLASS)()
        self._check(self.lib.uppe_profile_read(self.h, ms, cnt))
        return {self.lib.uppe_class_name(i).decode(): (ms[i], cnt[i]) for i in range(_native.NCLASS)}

    def launches(self):
        n = ctypes.c_longlong()
        self._check(self.lib.uppe_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def empty_field(self):
        return torch.empty(tuple(self.N[:3]), dtype=torch.complex64, device="cuda")


class Material:
    """Medium at one z: chi0(w), kz, kGalileo and the gas density plane (uppe_kernel.py:32-90).
    The host computes the density plane and chi0; kz is built on the device (uppe_set_material)."""

    def __init__(self, dev, grid, coords, vol, chi, chi3, nref, vg, density_lambda=None):
        N = grid.N
        self.dev = dev
        self.grid = grid
        self.chi = chi
        self.w = grid.w
        self.redchi3 = chi3 / nref
        self.n_ref = nref
        self.vg = vg
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
        self.kg = np.ascontiguousarray(-self.w / self.vg, dtype=np.float64)

    def UpdateMaterial(self, z):
        self.xp_eff[..., 3] = z
        dens = self.rel_density(self.xp_eff)
        chi0 = np.copy(self.chi)
        chi0[np.where(np.real(self.chi) > 0.0)] *= np.min(dens)
        chi0[np.where(np.real(self.chi) < 0.0)] *= np.max(dens)
        w2n2 = self.w ** 2 * (1 + chi0)
        ng = np.ascontiguousarray(self.n_ref * np.broadcast_to(dens, self.grid.N[1:3]), dtype=np.float64)
        return self.dev.set_material(np.asarray(w2n2, dtype=np.complex128), self.kg, ng)


def propagator(dev, mat, a_dev, subcycles, zi, zf, dzmin, outputs=None):
    """Advance the real-space field a to the next diagnostic plane (uppe_kernel.py:260-331).
    Returns device tensors (A, J, chiNL_w, ne_w) and the number of RHS evaluations."""
    if dev.grid.w[0] != 0.0:
        raise ValueError("UPPE propagator requires frequency range [0,...]")
    if dev.N[0] == 1:
        raise ValueError("UPPE propagator cannot be used for monochromatic radiation.")
    L = (zf - zi) / subcycles
    dev.load_field(a_dev)
    iterations = 0
    for sub in range(subcycles):
        z0 = zi + sub * L
        z = 0.0
        mat.UpdateMaterial(z0 + 0.5 * L)
        while z < L and (z - L) ** 2 > (L / 1e6) ** 2:
            dz = dev.rk4_step(z0 - zi + z, L, z, dzmin)
            iterations += 1
            z += dz
    if outputs is None:
        outputs = tuple(dev.empty_field() for _ in range(4))
    A, J, chi, ne = outputs
    dev.finish(zf - zi, A, J, chi, ne)
    if dev.nonfinite():
        logging.warning("UPPE field holds NaN or Inf after propagating to z=%g", zf)
    return A, J, chi, ne, 4 * iterations


class TrackOutputs:
    """The four arrays that ``track`` returns (A, J, chiNL, ne: complex128 of shape (N0, N1, N2, N3),
    diagnostic planes last, as uppe_kernel.py:343-352 lays them out), assembled on the device plane
    by plane and copied to the host once at the end.  The complex64 -> complex128 widening and the
    strided plane writes run on the device; the host receives one contiguous copy per array.
    ``shift`` reorders the frequency axis of each stored plane (the paraxial solver's fftshift)."""

    def __init__(self, N, first_plane, shift=None):
        self.arrays = [torch.empty(tuple(N), dtype=torch.complex128, device="cuda") for _ in range(4)]
        self.arrays[0][..., 0] = torch.from_numpy(np.ascontiguousarray(first_plane, dtype=np.complex128)).to("cuda")
        for x in self.arrays[1:]:
            x[..., 0] = 0
        self.shift = shift

    def first_plane(self, order=None):
        """The incoming plane as a contiguous complex64 device field (optionally reordered)."""
        a = self.arrays[0][..., 0]
        if order is not None:
            a = order(a)
        return a.to(torch.complex64).contiguous()

    def store(self, k, A, J, chi, ne):
        for dst, src in zip(self.arrays, (A, J, chi, ne)):
            dst[..., k].copy_(self.shift(src) if self.shift is not None else src)

    def host(self):
        """NumPy views of pinned host copies.  A copy into freshly allocated pageable memory runs at
        the speed of its first-touch page faults (about 24 GB/s on GB300's host); the pinned blocks
        of torch's caching host allocator, reused once earlier results are released, take the copy
        faster, and the four arrays go on four streams so that their copies run side by side."""
        main = torch.cuda.current_stream()
        out, streams = [], []
        for x in self.arrays:
            h = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
            s = torch.cuda.Stream()
            s.wait_stream(main)
            with torch.cuda.stream(s):
                h.copy_(x, non_blocking=True)
            streams.append(s)
            out.append(h)
        for s in streams:
            s.synchronize()
        return tuple(h.numpy() for h in out)


def track(cl, xp, eikonal, vg, vol_dict):
    """Propagate the UPPE volume's wave through its diagnostic planes (uppe_kernel.py:333-424).

    :param cl: ignored (the reference's OpenCL bundle); the device is CUDA device 0 / current.
    :param numpy.array xp: ray phase space (bundles, rays, 8).  Without an ``incoming wave`` the
        primary rays give the field on the first plane; at the end the rays are relaunched from the
        last plane (modified in place).  May be None with an ``incoming wave`` (no relaunch).
    :param numpy.array eikonal: ray eikonal data (bundles, 4), modified in place.
    :param numpy.array vg: ray group velocity (bundles, rays, 4), modified in place.
    :param dict vol_dict: the volume's input dictionary.
    :returns: A, J, chiNL, ne (complex128, shape ``wave grid``) and dom4d (8,)."""
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
        logging.info("Start UPPE propagation using ray data.")
        logging.warning("Polarization information is lost upon entering UPPE region.")
        first = raywave.boundary_fields(field_grid, xp[:, 0, :], eikonal, 1)
    else:
        logging.info("Start UPPE propagation using wave data")
        first = vol_dict["incoming wave"](grid.w, grid.x1, grid.x2)

    chi = vol_dict["dispersion inside"].chi(grid.w).astype(np.cdouble)
    rates = None
    if vol_dict.get("ionizer", None) is not None:
        rates = RateCoefficients(vol_dict["ionizer"])

    dev = DeviceGrid(grid, vol_dict, rates, vol_dict.get("precision", "mixed"))
    try:
        dev.set_rotator(vol_dict.get("rotator", None))
        mat = Material(dev, grid, vol_dict["wave coordinates"], vol_dict.get("object", None), chi, chi3,
                       vol_dict["density reference"], window_speed, vol_dict.get("density lambda", None))
        dens_nodes = cell_centers(-size[3] / 2, size[3] / 2, steps)
        field_walls = cell_walls(dens_nodes[0], dens_nodes[-1], steps)
        diagnostic_walls = np.linspace(-size[3] / 2, size[3] / 2, N[3])
        dzmin = vol_dict["minimum step"]
        dom4d = np.concatenate((grid.plot_ext, [field_walls[0], field_walls[-1]]))

        res = TrackOutputs(N, first)
        a_dev = res.first_plane()
        outs = tuple(dev.empty_field() for _ in range(4))
        for k in range(diagnostic_steps):
            zi = diagnostic_walls[k]
            zf = diagnostic_walls[k + 1]
            logging.info("Advancing to diagnostic plane %d", k + 1)
            A0, J0, c0, n0, evals = propagator(dev, mat, a_dev, subcycles, zi, zf, dzmin, outs)
            logging.info("%d evaluations of j(w,kx,ky)", evals)
            res.store(k + 1, A0, J0, c0, n0)
            a_dev, outs = A0, (dev.empty_field(), J0, c0, n0)
        A, J, chiNL, ne = res.host()
    finally:
        dev.close()
    # relaunch the rays from the last plane (uppe_kernel.py:420-423)
    if xp is not None:
        relaunch = raywave.relaunch_rays_full if vol_dict.get("full relaunch", False) else raywave.relaunch_rays
        relaunch(field_grid, xp, eikonal, vg, A[..., -1], size[3], vol_dict["dispersion inside"])
    return A, J, chiNL, ne, dom4d
