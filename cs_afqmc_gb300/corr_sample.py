"""Correlated sampling of two systems on shared auxiliary fields, with the reference's API
(ad_afqmc/corr_sample/corr_sample.py:482-694), evaluated by GB300 kernels.

Two Hamiltonians (or two trials) propagate their own walkers with the SAME field draws, so
the difference of their energies has a much smaller variance than two independent runs:
the repository's namesake, and the finite-difference derivative of the differentiation
pattern (h1 +- lambda D on identical fields).

* :func:`field_block_scan` - one block of one system with given fields: n_prop_steps
  phaseless steps, QR, overlaps, block energy, pop-control update, no SR
  (corr_sample.py:514-555) -> ``afq_field_block``.
* :func:`corr_otler_rm` - zero the weights of walkers whose weight z-score exceeds
  z_thresh in either system (corr_sample.py:557-594) -> ``afq_cs_outlier_removal``.
* :func:`cs_block_scan` / :func:`cs_steps_scan` - fields drawn from system 1's key, one
  block of each system, outlier removal, then the per-step sums (sum E w, sum w) of both
  (corr_sample.py:596-694).

Everything stays on the device; the per-step sums come back as CUDA tensors.
"""

from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import torch

from . import _lib
from ._engine import as_dev, device, stream_ptr
from .propagation import PropData, RngKey


def _draw_fields(prop, prop_data: PropData, sampler, nchol: int) -> torch.Tensor:
    shape = (sampler.n_prop_steps, prop.n_walkers, nchol)
    n = shape[0] * shape[1] * shape[2]
    out = torch.empty(shape, dtype=torch.float64, device=device())
    key: RngKey = prop_data["key"]
    _lib.call("afq_fill_normal", out.data_ptr(), n, key.seed, key.take(n), stream_ptr())
    return out


def field_block_scan(prop_data: PropData, fields, ham_data: dict, prop, trial, wave_data: dict,
                     sampler) -> PropData:
    """One block with the given fields [n_prop_steps, nw, nchol]. Stores the block energy and
    weight (0-d CUDA tensors) and the clamped local energies [nw] in prop_data under
    "block_energy", "block_weight" and "local_energies"."""
    eng = prop._engine(trial, ham_data, wave_data, prop_data["walkers"])
    dict.__setitem__(prop_data, "_engine", eng)
    f = as_dev(fields)
    if f.numel() != sampler.n_prop_steps * eng.nw * eng.nchol:
        raise _lib.AfqError(f"fields must have shape {(sampler.n_prop_steps, eng.nw, eng.nchol)}")
    e_loc = torch.empty(eng.nw, dtype=torch.float64, device=device())
    be = torch.empty(1, dtype=torch.float64, device=device())
    bw = torch.empty(1, dtype=torch.float64, device=device())
    st = prop_data.state(eng)
    _lib.call("afq_field_block", eng.ctx, ctypes.byref(st), f.data_ptr(), sampler.n_prop_steps,
              e_loc.data_ptr(), be.data_ptr(), bw.data_ptr(), stream_ptr())
    dict.__setitem__(prop_data, "local_energies", e_loc)
    dict.__setitem__(prop_data, "block_energy", be[0])
    dict.__setitem__(prop_data, "block_weight", bw[0])
    return prop_data


def corr_otler_rm(prop_data1: PropData, prop_data2: PropData, z_thresh: float = 5.0,
                  sums: Optional[torch.Tensor] = None) -> Tuple[PropData, PropData]:
    """Zero both weights of every walker whose weight z-score exceeds z_thresh in either
    system. Needs "local_energies" from field_block_scan; writes the step sums
    (sum E1 w1, sum w1, sum E2 w2, sum w2) into `sums` (4 doubles) when given."""
    w1, w2 = prop_data1["weights"], prop_data2["weights"]
    if w1.numel() != w2.numel():
        raise _lib.AfqError("correlated systems must have the same number of walkers")
    out = sums if sums is not None else torch.empty(4, dtype=torch.float64, device=device())
    _lib.call("afq_cs_outlier_removal", w1.data_ptr(), w2.data_ptr(),
              prop_data1["local_energies"].data_ptr(), prop_data2["local_energies"].data_ptr(),
              w1.numel(), float(z_thresh), out.data_ptr(), stream_ptr())
    return prop_data1, prop_data2


def cs_block_scan(prop_data1, ham_data1, prop1, trial1, wave_data1,
                  prop_data2, ham_data2, prop2, trial2, wave_data2, sampler,
                  fields=None, sums: Optional[torch.Tensor] = None, z_thresh: float = 5.0):
    """One correlated block: fields from system 1's key (or given), a block of each system,
    outlier removal (corr_sample.py:596-629; z_thresh = inf keeps every walker)."""
    if prop1.n_walkers != prop2.n_walkers:
        raise _lib.AfqError("correlated systems must have the same number of walkers")
    eng1 = prop1._engine(trial1, ham_data1, wave_data1, prop_data1["walkers"])
    f = _draw_fields(prop1, prop_data1, sampler, eng1.nchol) if fields is None else as_dev(fields)
    prop_data1 = field_block_scan(prop_data1, f, ham_data1, prop1, trial1, wave_data1, sampler)
    prop_data2 = field_block_scan(prop_data2, f, ham_data2, prop2, trial2, wave_data2, sampler)
    return corr_otler_rm(prop_data1, prop_data2, z_thresh=z_thresh, sums=sums)


def cs_steps_scan(steps: int, prop_data1, ham_data1, prop1, trial1, wave_data1,
                  prop_data2, ham_data2, prop2, trial2, wave_data2, sampler, fields=None,
                  z_thresh: float = 5.0):
    """`steps` correlated blocks (corr_sample.py:667-694). fields (optional):
    [steps, n_prop_steps, nw, nchol]; z_thresh: the outlier cut (inf: none). Returns
    ((prop_data1, prop_data2),
    (loc_en1, loc_weight1, loc_en2, loc_weight2)): per-step sum E w and sum w of each
    system after outlier removal, CUDA tensors [steps]."""
    sums = torch.empty(steps, 4, dtype=torch.float64, device=device())
    for s in range(steps):
        f = None if fields is None else fields[s]
        prop_data1, prop_data2 = cs_block_scan(prop_data1, ham_data1, prop1, trial1, wave_data1,
                                               prop_data2, ham_data2, prop2, trial2, wave_data2,
                                               sampler, fields=f, sums=sums[s], z_thresh=z_thresh)
    return (prop_data1, prop_data2), (sums[:, 0], sums[:, 1], sums[:, 2], sums[:, 3])
