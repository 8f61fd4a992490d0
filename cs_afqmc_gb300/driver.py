"""Single-rank AFQMC block driver (the non-AD branch of ad_afqmc/driver.py:16-492, without
MPI, file output or equilibration printing): repeated sampler.propagate_phaseless calls
with the per-block weight record, QR, global SR and e_estimate update kept on the device.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import torch

from . import _lib
from ._engine import device, stream_ptr
from .propagation import PropData


def run_blocks(sampler, ham, ham_data, prop, prop_data: PropData, trial, wave_data,
               n_blocks: int, fields=None, zetas=None):
    """Run n_blocks driver blocks. fields (optional): [n_blocks, n_sr, n_ene, n_prop, nw, G];
    zetas (optional): [n_blocks, n_sr + 1] (local SRs, then the driver's global SR).
    Returns device tensors (block_energy [n_blocks], block_weight [n_blocks]) and
    prop_data."""
    be = torch.empty(n_blocks, dtype=torch.float64, device=device())
    bw = torch.empty(n_blocks, dtype=torch.float64, device=device())
    for n in range(n_blocks):
        f = None if fields is None else fields[n]
        z_local = None if zetas is None else zetas[n][:-1]
        e, prop_data = sampler.propagate_phaseless(ham, ham_data, prop, prop_data, trial,
                                                   wave_data, fields=f, zetas=z_local)
        be[n].copy_(e)
        if zetas is None:
            zg = sampler.draw_zetas(prop_data, 1)
        else:
            zg = torch.as_tensor(zetas[n][-1:], dtype=torch.float64).to(device())
        eng = prop_data["_engine"]
        st = prop_data.state(eng)
        _lib.call("afq_block_end", eng.ctx, ctypes.byref(st), be[n:].data_ptr(), zg.data_ptr(),
                  bw[n:].data_ptr(), stream_ptr())
    return be, bw, prop_data
