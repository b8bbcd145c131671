"""Differentiable Gaussian-atom projection for PyTorch.

``project(I, x, r, geom)`` returns the sinogram R (A, D0[, D1]) and carries
gradients to I, x and r.  The backward pass is the hand-written adjoint
kernel: for an upstream gradient G it computes, per atom, <dR_j/dtheta, G>
in one launch (the reference's derivs_RadProj, NewtonBases2D.py:415-515 /
NewtonBases.py:954-1069, which is exactly the vector-Jacobian product).
Forward in FP32, adjoint sums in compensated FP32 per angle chunk and FP64
across chunks; gradients are returned in the dtype of the inputs.
"""
import torch

from . import engine


class GaussRadonFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, I, x, r, geom):
        atoms = engine.DeviceAtoms(I.detach(), x.detach(), r.detach(), geom.device)
        R = engine.radproj(atoms, geom)
        ctx.geom = geom
        ctx.save_for_backward(I, x, r)
        return R

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, grad_R):
        I, x, r = ctx.saved_tensors
        geom = ctx.geom
        atoms = engine.DeviceAtoms(I.detach(), x.detach(), r.detach(), geom.device)
        _f, g, _H = engine.atom_derivs(atoms, geom, "inner",
                                       grad_R.float().contiguous(), order=1)
        d = atoms.dim
        gI = g[:, 0].to(I.dtype).reshape(I.shape)
        gx = g[:, 1:1 + d].to(x.dtype).reshape(x.shape)
        gr = g[:, 1 + d:].to(r.dtype).reshape(r.shape)
        return gI, gx, gr, None


def project(I, x, r, geom):
    """Differentiable forward projection of atoms (I, x, r) on ``geom``."""
    return GaussRadonFunction.apply(I, x, r, geom)


class GaussRadon(torch.nn.Module):
    """Module form: holds the geometry, maps (I, x, r) to the sinogram."""

    def __init__(self, geom):
        super().__init__()
        self.geom = geom

    def forward(self, I, x, r):
        return project(I, x, r, self.geom)
