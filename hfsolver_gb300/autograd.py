"""RHF energy as a torch.autograd.Function of the nuclear coordinates.

The forward pass runs hfgpu_rhf_gradient (SCF, then the analytic gradient
kernels) and returns E_tot; the backward pass scales the saved gradient by the
incoming gradient.  PyTorch is only the tensor and autograd plumbing here: the
energy and its derivative come from libhfgpu.

    xyz = torch.tensor(coords_bohr, dtype=torch.float64, requires_grad=True)
    E = RHFEnergy.apply(xyz, atno)          # (natoms, 3) -> scalar
    E.backward()                             # xyz.grad = dE/dR, Ha/bohr
"""
import numpy as np
import torch

from . import api


class RHFEnergy(torch.autograd.Function):
    """E_tot(R) of a closed-shell molecule in 6-31G**; R is (natoms, 3) float64, bohr."""

    @staticmethod
    def forward(ctx, xyz, atno, options=None):
        if xyz.dtype != torch.float64 or xyz.dim() != 2 or xyz.shape[1] != 3:
            raise ValueError("xyz must be a (natoms, 3) float64 tensor")
        at = np.asarray(atno, dtype=np.int32)
        if at.shape != (xyz.shape[0],):
            raise ValueError("atno must hold one charge per row of xyz")
        opt = options if options is not None else api.RHFOptions(mp2="none", diis=True, tolP=1e-10, nscf=100)
        res, g = api.rhf_gradient(at, xyz.detach().cpu().numpy(), opt)
        ctx.save_for_backward(torch.from_numpy(g).to(xyz.device))
        return xyz.new_tensor(res["Etot"])

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None, None


def rhf_energy(xyz, atno, options=None):
    """Functional form of RHFEnergy.apply."""
    return RHFEnergy.apply(xyz, atno, options)
