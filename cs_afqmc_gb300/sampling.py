"""Sampler (block loop) with the reference's API (ad_afqmc/sampling.py:15-404).

``propagate_phaseless`` runs n_sr_blocks x [n_ene_blocks x [n_prop_steps propagation steps,
QR, overlaps, clamped local energies, block energy, pop-control update], local SR]
entirely on the device through one C-ABI call (no host synchronisation), and returns the
weighted block energy as a 0-d CUDA tensor, as sampling.py:319-341 returns a JAX scalar.

Auxiliary fields and SR uniforms come from prop_data["key"] (a counter-based Philox stream)
unless passed explicitly, so a caller (or a test) can feed the exact draws given to the
oracle.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib
from ._engine import as_dev, device, stream_ptr
from .propagation import PropData, RngKey


@dataclass
class sampler:
    n_prop_steps: int = 50
    n_ene_blocks: int = 50
    n_sr_blocks: int = 1
    n_blocks: int = 50

    def draw_fields(self, prop, prop_data: PropData, nchol: int) -> torch.Tensor:
        """N(0,1) fields [n_sr, n_ene, n_prop, nw, nchol] from prop_data["key"]."""
        shape = (self.n_sr_blocks, self.n_ene_blocks, self.n_prop_steps, prop.n_walkers, nchol)
        n = 1
        for s in shape:
            n *= s
        out = torch.empty(shape, dtype=torch.float64, device=device())
        key: RngKey = prop_data["key"]
        _lib.call("afq_fill_normal", out.data_ptr(), n, key.seed, key.take(n), stream_ptr())
        return out

    def draw_zetas(self, prop_data: PropData, n: int) -> torch.Tensor:
        out = torch.empty(n, dtype=torch.float64, device=device())
        key: RngKey = prop_data["key"]
        _lib.call("afq_fill_uniform", out.data_ptr(), n, key.seed, key.take(n), stream_ptr())
        return out

    def propagate_phaseless(self, ham, ham_data: dict, prop, prop_data: PropData, trial,
                            wave_data: dict, fields: Optional[torch.Tensor] = None,
                            zetas: Optional[torch.Tensor] = None):
        """(energy, prop_data); energy = sum(E_b w_b)/sum(w_b) over the n_sr*n_ene blocks.
        Also stores prop_data["block_energies"] / ["block_weights"] (device)."""
        eng = prop._engine(trial, ham_data, wave_data, prop_data["walkers"])
        dict.__setitem__(prop_data, "_engine", eng)
        nblk = self.n_sr_blocks * self.n_ene_blocks
        f = self.draw_fields(prop, prop_data, eng.nchol) if fields is None else as_dev(fields)
        want = (self.n_sr_blocks, self.n_ene_blocks, self.n_prop_steps, eng.nw, eng.nchol)
        if f.numel() != nblk * self.n_prop_steps * eng.nw * eng.nchol:
            raise _lib.AfqError(f"fields must have shape {want}")
        z = self.draw_zetas(prop_data, self.n_sr_blocks) if zetas is None else as_dev(zetas)
        if z.numel() != self.n_sr_blocks:
            raise _lib.AfqError(f"zetas must have {self.n_sr_blocks} entries")
        be = torch.empty(nblk, dtype=torch.float64, device=device())
        bw = torch.empty(nblk, dtype=torch.float64, device=device())
        energy = torch.empty(1, dtype=torch.float64, device=device())
        st = prop_data.state(eng)
        _lib.call("afq_propagate_phaseless", eng.ctx, ctypes.byref(st), f.data_ptr(),
                  z.data_ptr(), self.n_prop_steps, self.n_ene_blocks, self.n_sr_blocks,
                  be.data_ptr(), bw.data_ptr(), energy.data_ptr(), stream_ptr())
        dict.__setitem__(prop_data, "block_energies", be)
        dict.__setitem__(prop_data, "block_weights", bw)
        return energy[0], prop_data

    def __hash__(self) -> int:
        return hash((self.n_prop_steps, self.n_ene_blocks, self.n_sr_blocks, self.n_blocks))
