"""torch.autograd binding of the real-space data vector.

`real_data_vector(plan, omega_m, h0, chi, G, lnP, nu)` evaluates the masked
3x2pt data vector of a batch of points on the GPU (cl2pt_eval_real) and is
differentiable in lnP (the nonlinear P(k, z) table, [n][nk * nz]) and nu
(the nuisance parameters as float64 [n][13 * MAX_BINS], the flat
cl2pt_nuisance layout of abi.nuisance_to_array).  The backward pass calls
cl2pt_vjp_real, which recomputes the forward and runs the hand-written
adjoint kernels; nothing but the inputs is kept between the passes.

`value_and_vjp` is the fused form a sampler uses: one call returns the value
and the gradient of cot . dv.

`fourier_data_vector(plan, ..., ell)` is the same for the Fourier 3x2pt
vector at the multipoles ell (cl2pt_eval_fourier forward, cl2pt_vjp_fourier
backward).
"""
from __future__ import annotations

import torch

from . import abi
from .lib import Plan

NU_LEN = 13 * abi.MAX_BINS


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _check(t: torch.Tensor, name: str):
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError(f"{name}: expected a contiguous float64 CUDA tensor")


class RealDataVector(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan: Plan, omega_m, h0, chi, G, lnP, nu, mask=None, pm=None):
        for t, nm in ((omega_m, "omega_m"), (h0, "h0"), (chi, "chi"), (G, "G"), (lnP, "lnP"), (nu, "nu")):
            _check(t, nm)
        if nu.shape[-1] != NU_LEN:
            raise ValueError(f"nu: expected [n][{NU_LEN}]")
        n = omega_m.shape[0]
        out = torch.empty(n, plan.n_total, dtype=torch.float64, device=omega_m.device)
        plan.eval_real_device(omega_m, h0, chi, G, lnP, nu, out, mask=mask, pm=pm, stream=_stream())
        ctx.plan = plan
        ctx.mask, ctx.pm = mask, pm
        ctx.save_for_backward(omega_m, h0, chi, G, lnP, nu)
        return out

    @staticmethod
    def backward(ctx, g):
        omega_m, h0, chi, G, lnP, nu = ctx.saved_tensors
        g = g.contiguous()
        lbar = torch.empty_like(lnP)
        nbar = torch.empty_like(nu)
        ctx.plan.vjp_real_device(omega_m, h0, chi, G, lnP, nu, g, None, lbar, nbar,
                                 mask=ctx.mask, pm=ctx.pm, stream=_stream())
        return None, None, None, None, None, lbar, nbar, None, None


def real_data_vector(plan: Plan, omega_m, h0, chi, G, lnP, nu, mask=None, pm=None):
    """Differentiable data vector [n][n_total] (see the module docstring)."""
    return RealDataVector.apply(plan, omega_m, h0, chi, G, lnP, nu, mask, pm)


def value_and_vjp(plan: Plan, omega_m, h0, chi, G, lnP, nu, cot, mask=None, pm=None):
    """(dv, d(cot.dv)/dlnP, d(cot.dv)/dnu) in one pass."""
    n = omega_m.shape[0]
    dv = torch.empty(n, plan.n_total, dtype=torch.float64, device=omega_m.device)
    lbar = torch.empty_like(lnP)
    nbar = torch.empty_like(nu)
    plan.vjp_real_device(omega_m, h0, chi, G, lnP, nu, cot.contiguous(), dv, lbar, nbar,
                         mask=mask, pm=pm, stream=_stream())
    return dv, lbar, nbar


class FourierDataVector(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan: Plan, omega_m, h0, chi, G, lnP, nu, ell, lmax_shear=1e30, mask=None):
        for t, nm in ((omega_m, "omega_m"), (h0, "h0"), (chi, "chi"), (G, "G"), (lnP, "lnP"), (nu, "nu")):
            _check(t, nm)
        if nu.shape[-1] != NU_LEN:
            raise ValueError(f"nu: expected [n][{NU_LEN}]")
        n = omega_m.shape[0]
        out = torch.empty(n, plan.fourier_n_total(len(ell)), dtype=torch.float64, device=omega_m.device)
        plan.eval_fourier_device(omega_m, h0, chi, G, lnP, nu, ell, out, lmax_shear=lmax_shear, mask=mask,
                                 stream=_stream())
        ctx.plan, ctx.ell, ctx.lmax_shear, ctx.mask = plan, ell, lmax_shear, mask
        ctx.save_for_backward(omega_m, h0, chi, G, lnP, nu)
        return out

    @staticmethod
    def backward(ctx, g):
        omega_m, h0, chi, G, lnP, nu = ctx.saved_tensors
        g = g.contiguous()
        lbar = torch.empty_like(lnP)
        nbar = torch.empty_like(nu)
        ctx.plan.vjp_fourier_device(omega_m, h0, chi, G, lnP, nu, ctx.ell, g, None, lbar, nbar,
                                    lmax_shear=ctx.lmax_shear, mask=ctx.mask, stream=_stream())
        return None, None, None, None, None, lbar, nbar, None, None, None


def fourier_data_vector(plan: Plan, omega_m, h0, chi, G, lnP, nu, ell, lmax_shear=1e30, mask=None):
    """Differentiable Fourier vector [n][plan.fourier_n_total(len(ell))],
    differentiable in lnP and nu (see the module docstring)."""
    return FourierDataVector.apply(plan, omega_m, h0, chi, G, lnP, nu, ell, lmax_shear, mask)
