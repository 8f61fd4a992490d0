"""Hamiltonian handler with the reference's API (ad_afqmc/hamiltonian.py:12-84)."""

from __future__ import annotations

from dataclasses import dataclass

import torch

from ._engine import as_dev


@dataclass
class hamiltonian:
    """ham_data holds h0, h1 [2, norb, norb], chol [nchol, norb*norb] (+ ene0); the
    build_* calls add the trial's half-rotated integrals and the propagator's
    intermediates, as device tensors."""

    norb: int

    def rotate_orbs(self, ham_data: dict, mo_coeff) -> dict:
        """h1 -> C^T h1 C, L_g -> C^T L_g C (hamiltonian.py:24-47)."""
        c = as_dev(mo_coeff)
        h1 = as_dev(ham_data["h1"])
        ham_data["h1"] = torch.stack([c.T @ h1[0] @ c, c.T @ h1[1] @ c])
        chol = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        ham_data["chol"] = torch.einsum("qi,gij,jp->gqp", c.T, chol, c).reshape(
            -1, self.norb * self.norb).contiguous()
        return ham_data

    def build_measurement_intermediates(self, ham_data: dict, trial, wave_data: dict) -> dict:
        """(hamiltonian.py:49-64)."""
        return trial._build_measurement_intermediates(ham_data, wave_data)

    def build_propagation_intermediates(self, ham_data: dict, prop, trial, wave_data: dict) -> dict:
        """(hamiltonian.py:66-81)."""
        return prop._build_propagation_intermediates(ham_data, trial, wave_data)

    def __hash__(self) -> int:
        return hash(self.norb)
