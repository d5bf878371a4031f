"""torch.autograd wrappers of the forward kernels, with the hand-written
adjoint kernels as their backward.  Used to gradcheck the adjoints; the
inversion itself calls the C ABI directly.

The reference has no gradients at all (finite-difference Jacobian,
TFM.cpp:124-135)."""
import torch


class PrismGravity(torch.autograd.Function):
    """gz = F(rho) on a regular prism mesh; d/drho by ztm_gfm_adjoint."""

    @staticmethod
    def forward(ctx_, rho, gctx, mesh, stations, precision="mixed"):
        ctx_.gctx = gctx
        ctx_.mesh = mesh
        ctx_.precision = precision
        ctx_.save_for_backward(stations)
        out = gctx.prism(mesh, rho.detach().contiguous(), stations, precision=precision)
        gctx.sync()
        return out

    @staticmethod
    def backward(ctx_, grad_out):
        (stations,) = ctx_.saved_tensors
        g = ctx_.gctx.adjoint(ctx_.mesh, stations, grad_out.contiguous(), precision=ctx_.precision)
        ctx_.gctx.sync()
        return g, None, None, None, None


class InterfaceGravity(torch.autograd.Function):
    """gz = F(depth, rho_col) on an interface mesh; gradients by
    ztm_gfm_interface_adjoint (top-face derivative for depth)."""

    @staticmethod
    def forward(ctx_, depth, rho_col, gctx, imesh, stations, precision="mixed"):
        ctx_.gctx = gctx
        ctx_.imesh = imesh
        ctx_.precision = precision
        d = depth.detach().contiguous()
        r = rho_col.detach().contiguous()
        ctx_.save_for_backward(d, r, stations)
        out = gctx.interface(imesh, d, r, stations, precision=precision)
        gctx.sync()
        return out

    @staticmethod
    def backward(ctx_, grad_out):
        d, r, stations = ctx_.saved_tensors
        g_rho, g_dep = ctx_.gctx.interface_adjoint(ctx_.imesh, d, r, stations,
                                                   grad_out.contiguous(),
                                                   precision=ctx_.precision)
        ctx_.gctx.sync()
        return g_dep, g_rho, None, None, None, None
