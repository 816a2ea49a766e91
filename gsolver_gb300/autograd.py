"""PyTorch autograd over the hand-written adjoint (no counterpart in the reference).

``objective(P, dz_rk, dz_lin, weights)`` returns a function J(FIELD_0) of a complex128 tensor
[n_r][n_t] (FIELD at the start, (r, omega)): the forward replays the propagator() calls with the
recorded step sizes through gs_forward_fixed and returns J = sum(weights * |FIELD_end|^2); the
backward is gs_gradient (forward + checkpointed adjoint, both on the GPU through the C ABI).
The gradient follows PyTorch's convention for a real function of a complex input,
dJ/dRe + i dJ/dIm.  PyTorch is needed only here; the library itself does not import it.
"""
import numpy as np


def objective(P, dz_rk, dz_lin, weights, checkpoint_stride=0):
    """J(field) for the Propagator P with the step sizes (dz_rk[k], dz_lin[k]) of k propagator()
    calls (RK4 stages, linear step) and objective weights [n_r][n_t]."""
    import torch

    dz_rk = np.ascontiguousarray(dz_rk, dtype=np.float64)
    dz_lin = np.ascontiguousarray(dz_lin, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)

    class _Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, field):
            ctx.save_for_backward(field)
            J, _ = P.forward_fixed(field.detach().cpu().numpy(), dz_rk, dz_lin, w)
            return field.new_tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            (field,) = ctx.saved_tensors
            _, g = P.gradient(field.detach().cpu().numpy(), dz_rk, dz_lin, w, checkpoint_stride)
            return gJ * torch.from_numpy(g).to(field.device)

    return _Objective.apply
