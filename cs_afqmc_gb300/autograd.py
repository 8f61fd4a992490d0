"""The phaseless block as a differentiable torch function of h1: the reference takes the
block's derivatives with jax.jvp / jax.vjp of sampler.propagate_phaseless_ad*
(driver.py:207-235); here the same reverse-mode derivative is a torch.autograd.Function
whose backward is the library's adjoint sweep (afq_propagate_phaseless_vjp(_ex)).

The forward pass runs the recorded forward sweep and its adjoint together (the adjoint
needs the recorded walker snapshots, which the workspace holds only until the next call),
keeps d energy / d h1 and returns the energy; backward scales that gradient by the incoming
cotangent. FP64 (complex128) walkers only."""

from __future__ import annotations

from typing import Optional

import torch

from ._engine import _CACHE_KEY


class PhaselessBlock(torch.autograd.Function):
    """energy = block(h1); d energy / d h1 from the adjoint sweep."""

    @staticmethod
    def forward(ctx, h1, sampler, ham, ham_data, prop, prop_data, trial, wave_data, fields, zetas, do_sr,
                orbital_rotation):
        hd = {k: v for k, v in ham_data.items() if k not in (_CACHE_KEY, "rot_chol", "rot_h1", "exp_h1",
                                                            "mf_shifts", "h0_prop")}
        hd["h1"] = h1.detach()
        if orbital_rotation:
            energy, rdm1, _ = sampler.propagate_phaseless_ad_vjp(ham, hd, prop, prop_data, trial, wave_data,
                                                                 do_sr=do_sr, fields=fields, zetas=zetas)
        else:
            hd = ham.build_measurement_intermediates(hd, trial, wave_data)
            hd = ham.build_propagation_intermediates(hd, prop, trial, wave_data)
            energy, rdm1, _ = sampler.propagate_phaseless_ad_norot_vjp(ham, hd, prop, prop_data, trial, wave_data,
                                                                       do_sr=do_sr, fields=fields, zetas=zetas)
        ctx.save_for_backward(rdm1.to(h1.dtype))
        return energy.detach().clone()

    @staticmethod
    def backward(ctx, grad_energy):
        (rdm1,) = ctx.saved_tensors
        return (grad_energy * rdm1,) + (None,) * 11


def phaseless_energy(h1: torch.Tensor, sampler, ham, ham_data: dict, prop, prop_data, trial, wave_data: dict,
                     fields: Optional[torch.Tensor] = None, zetas: Optional[torch.Tensor] = None,
                     do_sr: bool = True, orbital_rotation: bool = False) -> torch.Tensor:
    """The blocked energy of one sampler block (sampler.propagate_phaseless_ad_norot, or
    propagate_phaseless_ad with orbital_rotation) as a differentiable function of h1
    ([2, norb, norb] float64 CUDA tensor): ham_data's intermediates are rebuilt from h1, and
    torch.autograd.grad(energy, h1) is the block's one-body density matrix. prop_data
    advances as the block does."""
    return PhaselessBlock.apply(h1, sampler, ham, ham_data, prop, prop_data, trial, wave_data, fields, zetas,
                                do_sr, orbital_rotation)
