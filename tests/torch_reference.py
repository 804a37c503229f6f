"""Test infrastructure: one UPPE RK4 z-step in plain PyTorch FP64 (complex128), differentiable by
torch.autograd.  It restates the oracle's step (oracle/uppe_oracle.py, itself pinned to SeaRay's
modules/uppe_kernel.py) with torch operations so that its autograd gradient can check the
hand-written CUDA adjoint."""
import numpy as np
import torch


class TorchStep:
    def __init__(self, orc):
        """orc: an oracle.uppe_oracle.Oracle whose medium has been updated (orc.mat.update(z))."""
        g, mat = orc.g, orc.mat
        self.g = g
        self.cart = g.cartesian
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a))
        self.kz = t(mat.kz)
        self.kg = t(mat.kg)
        self.ng = t(mat.ng)
        self.w = t(g.w)[:, None, None]
        self.nl = t(orc.nl_filter)[:, None, None]
        self.cond = t(orc.conditioner)[:, None, None]
        self.dt = g.dt
        self.Nt = g.Nt
        self.rates = orc.rates
        self.rotator = orc.rotator
        if not self.cart:
            self.H = t(g.H)
            self.lam = t(g.Lambda)
            self.Nk = g.Nk
        Ni = self.Nt
        i = np.arange(Ni)
        f = np.ones(Ni)
        f[(i < 4) | (i > Ni - 5)] = 0.0
        up = (i >= 4) & (i < 68)
        q = (i[up] - 4) / 64
        f[up] *= 10 * q ** 3 - 15 * q ** 4 + 6 * q ** 5
        dn = (i <= Ni - 5) & (i > Ni - 69)
        q = (Ni - 5 - i[dn]) / 64
        f[dn] *= 10 * q ** 3 - 15 * q ** 4 + 6 * q ** 5
        self.window = t(f)[:, None, None]

    def kspace(self, a):
        if self.cart:
            return torch.fft.fft(torch.fft.fft(a, dim=1), dim=2)
        b = torch.fft.fft(a, dim=2) * self.lam[None, :, None]
        out = torch.einsum("ijm,fjm->fim", self.H.to(b.dtype), b)
        pad = torch.zeros(b.shape[0], b.shape[1] - self.Nk, b.shape[2], dtype=b.dtype)
        return torch.cat([out, pad], dim=1) / self.lam[None, :, None]

    def rspace(self, a):
        if self.cart:
            return torch.fft.ifft(torch.fft.ifft(a, dim=2), dim=1)
        b = a * self.lam[None, :, None]
        out = torch.einsum("jim,fjm->fim", self.H.to(b.dtype), b[:, :self.Nk, :]) / self.lam[None, :, None]
        return torch.fft.ifft(out, dim=2)

    def phase(self, z):
        return torch.exp(-self.kz.imag * z) * torch.exp(1j * (self.kz.real + self.kg) * z)

    def rate(self, Et):
        r = self.rates
        if r.explicit:
            Em = r.field_conv * torch.abs(Et) + r.cutoff
            return r.rate_conv * r.C1 * Em ** r.C2 * torch.exp(r.C3 / Em)
        L = torch.log(r.field_conv * torch.abs(Et) + r.cutoff)
        c = r.clog
        return r.rate_conv * torch.exp(c[0] + c[1] * L + c[2] * L ** 2 + c[3] * L ** 3 + c[4] * L ** 4 + c[5] * L ** 5)

    def raman_chi(self, Et):
        """The oracle's raman_chi (AddChiUPPE, kernels/rotations.cl:85-129) with torch operations."""
        rot = self.rotator
        Nt = Et.shape[0]
        Er = torch.flip(Et, [0])
        F = 0.5 * (rot.dalpha / rot.hbar) * Er ** 2
        n = torch.arange(Nt, dtype=torch.float64)[:, None, None]
        chi = torch.zeros_like(Et)
        for j in range(2, rot.Wj.shape[0]):
            if rot.Tj[j] == 0.0:
                continue
            wdt = complex(rot.Wj[j]) * self.dt
            S = 2.0 * j * (j - 1) / (15 * (2 * j - 1))
            h2n = torch.exp(1j * wdt * n)
            a = F * h2n * np.exp(0.5j * wdt)
            rho = -1j * self.dt * (torch.cumsum(a, dim=0) - a)
            term = rot.Tj[j] * S * rho * torch.conj(h2n) * wdt
            chi = chi + torch.flip(torch.cumsum(2 * term.imag * self.ng[None] * rot.dalpha, dim=0), [0])
        return chi

    def rhs(self, q, z, redchi3):
        E = 1j * self.kz * self.phase(z) * q
        E = self.rspace(E)
        Et = torch.fft.irfft(E, n=self.Nt, dim=0)
        if self.rates is None:
            Jw = torch.zeros_like(E)
        else:
            r = self.rate(Et)
            r = torch.cat([r[:-1], torch.zeros_like(r[-1:])], dim=0)
            pair = 0.5 * (r[:-1] + r[1:]) * self.dt
            S = torch.flip(torch.cumsum(torch.flip(pair, [0]), dim=0), [0])
            S = torch.cat([S, torch.zeros_like(S[-1:])], dim=0)
            ne = self.ng[None] * (1.0 - torch.exp(-S)) * self.window
            Jw = torch.fft.rfft(ne * Et, dim=0) / (0.1 - 1j * self.w)
        chi = self.ng[None] * redchi3 * Et * Et
        if self.rotator is not None:  # before the Kerr term, as uppe_kernel.py:174-176
            chi = self.raman_chi(Et) + chi
        Jw = Jw + (-1j * self.w) * torch.fft.rfft(chi * Et, dim=0)
        Jw = Jw * self.nl
        Jw = self.kspace(Jw)
        return 0.5j * self.phase(-z) * Jw / self.kz.real

    def step(self, q0, z, dz, redchi3):
        C = self.cond
        k1 = self.rhs(q0, z, redchi3)
        qf = q0 + dz / 6 * k1
        q = (q0 + dz / 2 * k1) * C
        k2 = self.rhs(q, z + dz / 2, redchi3)
        qf = qf + dz / 3 * k2
        q = (q0 + dz / 2 * k2) * C
        k3 = self.rhs(q, z + dz / 2, redchi3)
        qf = qf + dz / 3 * k3
        q = (q0 + dz * k3) * C
        k4 = self.rhs(q, z + dz, redchi3)
        return (qf + dz / 6 * k4) * C

    def finish_field(self, q, z):
        return self.rspace(self.phase(z) * q)
