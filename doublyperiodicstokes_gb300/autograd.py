"""Differentiable Mdot: (V, W) = M(X) (F, T) as a torch.autograd.Function.

    op = DPStokes(StokesParams(...), N)
    V, W = mdot(op, X, F, T)          # X, F, T: [N, 3] cuda tensors
    loss = (g * V).sum(); loss.backward()   # X.grad, F.grad, T.grad

The backward is the library's dpst_mdot_backward: the transpose of the
operator applied to the incoming gradients (the adjoint of every stage:
interpolation, x-y FFT, z transform, per-wavenumber solve, wall correction,
spreading; in the triply periodic box the grid-to-grid map is self-adjoint)
for dl/dF and dl/dT, and the ES-kernel derivatives in the spreading and
interpolation weights for dl/dX.  The forward's velocity grid is taken from
the handle when it still holds it (no other Mdot or position update on the
handle since the forward), else recomputed.  Second derivatives and the
regular-kernel torque coupling are not provided."""
import torch
from torch.autograd.function import once_differentiable


class _Mdot(torch.autograd.Function):
    @staticmethod
    def forward(ctx, op, X, F, T):
        X = X.detach().contiguous()
        F = F.detach().contiguous()
        T = T.detach().contiguous() if T is not None else None
        op.set_positions(X)
        V, W = op.mdot(F, T)
        ctx.serial = op.forward_serial()
        ctx.op = op
        ctx.has_T = T is not None
        ctx.save_for_backward(X, F, T if T is not None else torch.empty(0, device=F.device))
        if W is None:
            return V, torch.zeros_like(V)
        return V, W

    @staticmethod
    @once_differentiable
    def backward(ctx, gV, gW):
        op = ctx.op
        X, F, T = ctx.saved_tensors
        T = T if ctx.has_T else None
        need_X, need_F, need_T = ctx.needs_input_grad[1], ctx.needs_input_grad[2], ctx.needs_input_grad[3]
        if gV is None:
            gV = torch.zeros_like(F)
        gV = gV.contiguous()
        if gW is not None and op.params.has_torque:
            gW = gW.contiguous()
        else:
            gW = None
        serial = ctx.serial if op.forward_serial() == ctx.serial else 0
        if serial == 0:
            op.set_positions(X)  # the handle has moved on since the forward
        gF, gT, gX = op.mdot_backward(F if need_X else None, T, gV, gW, need_F=need_F,
                                      need_T=need_T and T is not None, need_X=need_X, forward_serial=serial)
        return None, gX, gF, gT


def mdot(op, X, F, T=None):
    """Differentiable (V, W) = M(X) (F, T); W is zeros when the operator has
    no torques."""
    return _Mdot.apply(op, X, F, T)
