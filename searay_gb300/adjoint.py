"""Gradients of the UPPE propagation through torch.autograd, from the hand-written adjoint.

``propagate(dev, a0, chi3_over_nref, dz, nsteps)`` advances the real-space incoming field ``a0``
(complex64, [N0][N1][N2], on the device) through ``nsteps`` fixed RK4 steps of size ``dz`` on a
:class:`searay_gb300.uppe.DeviceGrid` whose material is already set, and returns the real-space
field at the end, ``A = T^-1 exp(i(kz+kg) z) q`` (the field output of ``uppe_kernel.finish``,
``modules/uppe_kernel.py:250-251``).  The result is differentiable with respect to ``a0`` and the
Kerr coefficient ``chi3_over_nref``.

The backward pass stores the spectral amplitude q every ``checkpoint_every`` steps during the
forward pass, recomputes the steps of one checkpoint interval, and applies the vector-Jacobian
products of the library (``uppe_adjoint_rk4_step``, ``uppe_adjoint_load``, ``uppe_adjoint_finish``)
in reverse order.  Gradients follow PyTorch's convention for complex tensors, dL/dRe + i dL/dIm.
"""
import torch


class _Propagate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a0, chi3_red, dev, dz, nsteps, checkpoint_every):
        dev.set_chi3(float(chi3_red))
        a = a0.detach().to(device="cuda", dtype=torch.complex64).contiguous()
        dev.load_field(a)
        ckpts = {}
        for n in range(nsteps):
            if n % checkpoint_every == 0:
                q = dev.empty_field()
                dev.get_field(q)
                ckpts[n] = q
            dev.rk4_step(n * dz, dz, 0.0, dz)
        A = dev.empty_field()
        dev.finish_field(nsteps * dz, A)
        ctx.dev, ctx.dz, ctx.nsteps, ctx.ck = dev, dz, nsteps, checkpoint_every
        ctx.ckpts = ckpts
        ctx.chi3_red = float(chi3_red)
        ctx.a_dtype, ctx.chi_like = a0.dtype, chi3_red
        return A

    @staticmethod
    def backward(ctx, gA):
        dev, dz, nsteps, ck = ctx.dev, ctx.dz, ctx.nsteps, ctx.ck
        dev.set_chi3(ctx.chi3_red)
        lam = dev.empty_field()
        dev.adjoint_finish(nsteps * dz, gA.to(torch.complex64).contiguous(), lam)
        dred = 0.0
        starts = sorted(ctx.ckpts.keys())
        for s0 in reversed(starts):
            s1 = min(s0 + ck, nsteps)
            # q at every step of the interval, recomputed from its checkpoint
            qs = [ctx.ckpts[s0]]
            dev.set_field(qs[0])
            for n in range(s0, s1 - 1):
                dev.rk4_step(n * dz, dz, 0.0, dz)
                q = dev.empty_field()
                dev.get_field(q)
                qs.append(q)
            for n in range(s1 - 1, s0 - 1, -1):
                lam_in = dev.empty_field()
                dred += dev.adjoint_step(qs[n - s0], lam, lam_in, n * dz, dz)
                lam = lam_in
        g_a = dev.empty_field()
        dev.adjoint_load(lam, g_a)
        g_chi = torch.as_tensor(dred, dtype=ctx.chi_like.dtype, device=ctx.chi_like.device) \
            if torch.is_tensor(ctx.chi_like) else None
        return g_a.to(ctx.a_dtype), g_chi, None, None, None, None


def propagate(dev, a0, chi3_over_nref, dz, nsteps, checkpoint_every=20):
    """Differentiable fixed-step propagation (see the module docstring)."""
    if not torch.is_tensor(chi3_over_nref):
        chi3_over_nref = torch.tensor(float(chi3_over_nref), dtype=torch.float64)
    return _Propagate.apply(a0, chi3_over_nref, dev, float(dz), int(nsteps), int(checkpoint_every))
