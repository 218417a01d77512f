"""The discrete adjoint of the Strang step as a differentiable function.

``overlap_loss(model, V, psi0, psi_target, nsteps, K)`` is the loss

    L(V, psi0) = 1 - |<psi_target, psi(T)>|^2,   psi(T) = [Strang step]^nsteps psi0

as a ``torch.autograd.Function``: the Python counterpart of the
``ChainRulesCore.rrule`` a Julia caller attaches to the same C entry point.
Its forward makes ONE ``gpss_adjoint`` call, which returns the loss and both
gradients (the forward sweep with checkpoints every K steps, then the reverse
sweep); its backward only scales the stored gradients by the incoming
cotangent, so a reverse pass costs no further device work.

Gradient conventions are PyTorch's: ``V.grad`` is dL/dV (real, field shape);
``psi0.grad`` is dL/dRe psi0 + i dL/dIm psi0 = 2 dL/d conj(psi0), the
Wirtinger gradient ``gpss_adjoint`` returns.

The forward sets the model's potential to ``V`` and its field to ``psi0``
(host copies, uploaded through the C ABI); the model's coeffD, beta and dt
stay as they are.  The adjoint is that of the unmerged FP64/FP32 Strang step
with Omega = 0 (the conditions ``gpss_adjoint`` checks).  PyTorch is used for
the autograd bookkeeping only: the gradients come from the CUDA kernels
behind ``gpss_adjoint``.
"""
import numpy as np
import torch

from . import GrossPitaevskiiParameters, PotentialArray


def _host(t, dtype):
    return np.asfortranarray(t.detach().to("cpu").numpy().astype(dtype, copy=False))


class _OverlapLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, V, psi0, model, psi_target, nsteps, K):
        f = model.f
        p = model.param
        model.set_params(GrossPitaevskiiParameters(PotentialArray(f, _host(V, np.float64)),
                                                   coeffD=p.coeffD, beta=p.beta, Omega=p.Omega))
        f.phi = _host(psi0, np.complex128)  # uploads: the model owns the field
        tgt = psi_target.detach().to("cpu").numpy() if torch.is_tensor(psi_target) else psi_target
        L, dV, g0 = model.adjoint(tgt, nsteps, K)
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(dV)).to(V.device),
                              torch.from_numpy(np.ascontiguousarray(g0)).to(psi0.device))
        return torch.tensor(L, dtype=torch.float64, device=V.device)

    @staticmethod
    def backward(ctx, gL):
        dV, g0 = ctx.saved_tensors
        gV = gL * dV if ctx.needs_input_grad[0] else None
        gpsi = gL.to(g0.dtype) * g0 if ctx.needs_input_grad[1] else None
        return gV, gpsi, None, None, None, None


def overlap_loss(model, V, psi0, psi_target, nsteps, K=50):
    """L = 1 - |<psi_target, psi(T)>|^2 after ``nsteps`` Strang steps of
    ``model`` from ``psi0`` under the potential ``V``, differentiable in ``V``
    (real tensor, field shape) and ``psi0`` (complex tensor, field shape).
    ``K`` is the checkpoint interval of the reverse sweep."""
    if tuple(V.shape) != tuple(model.f.g.n) or tuple(psi0.shape) != tuple(model.f.g.n):
        raise ValueError("V and psi0 must have the field's shape")
    if V.is_complex() or not psi0.is_complex():
        raise TypeError("V must be real and psi0 complex")
    return _OverlapLoss.apply(V, psi0, model, psi_target, int(nsteps), int(K))
