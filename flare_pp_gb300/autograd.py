"""torch.autograd binding of the hand-written adjoint.

``FlareEnergy.apply(positions, gp, structure, precision)`` returns the energy
of a mapped SparseGP model for device positions (float64, n x 3).  Its
backward is the library's adjoint (forces are -dE/dx), so
``torch.autograd.grad(E, positions)`` gives -forces without any stored
descriptor derivatives.  The virial stress of the same evaluation is left on
the structure as ``structure.last_stress`` (flare order xx, xy, xz, yy, yz,
zz).
"""
import torch

from . import _lib
from ._lib import check, lib
from .api import PRECISIONS


class FlareEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, gp, structure, precision="mixed"):
        if positions.dtype != torch.float64 or not positions.is_cuda:
            raise TypeError("positions must be a CUDA float64 tensor")
        pos = positions.detach().contiguous()
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        check(lib().fpp_structure_set_positions(structure.handle, pos.data_ptr(), 1, stream))
        gp._ensure_mapped(stream)
        n = structure.noa
        e = torch.zeros(1, dtype=torch.float64, device=pos.device)
        f = torch.zeros((n, 3), dtype=torch.float64, device=pos.device)
        s = torch.zeros(6, dtype=torch.float64, device=pos.device)
        check(lib().fpp_predict_mapped(gp._model.handle, structure.handle,
                                       PRECISIONS[precision], e.data_ptr(), f.data_ptr(),
                                       s.data_ptr(), None, 1, stream))
        ctx.save_for_backward(f)
        structure.last_stress = s
        return e[0]

    @staticmethod
    def backward(ctx, grad_e):
        (f,) = ctx.saved_tensors
        return -grad_e * f, None, None, None


def energy_forces_stress(gp, structure, positions, precision="mixed"):
    """Energy (autograd-connected), forces and stress for device positions."""
    pos = positions.detach().requires_grad_(True)
    e = FlareEnergy.apply(pos, gp, structure, precision)
    (g,) = torch.autograd.grad(e, pos)
    return e.detach(), -g, structure.last_stress
