"""Single-rank AFQMC block driver (the non-AD branch of ad_afqmc/driver.py:16-492, without
MPI or file output): the equilibration sweeps (run_equilibration, driver.py:91-133) and
the sampling blocks (run_blocks, driver.py:245-308), each block a
sampler.propagate_phaseless call followed by the weight record, QR, global SR and
e_estimate update, all on the device.
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


def run_equilibration(ham, ham_data, prop, prop_data: PropData, trial, wave_data, n_eql: int,
                      fields=None, zetas=None, sampler=None):
    """The equilibration sweeps of driver.py:91-133: n_eql blocks of the equilibration
    sampler (sampling.sampler(n_prop_steps=50, n_ene_blocks=5, n_sr_blocks=10)), each
    followed by the block weight record, QR, global SR and e_estimate = 0.9 e_estimate +
    0.1 E_block (on one rank the population's block energy is the block's own). fields
    (optional): [n_eql, 10, 5, 50, nw, G]; zetas (optional): [n_eql, 11]. sampler: another
    equilibration sampler (tests use shorter blocks). Returns device tensors
    (block_energy [n_eql], block_weight [n_eql]) and prop_data."""
    from . import sampling
    samp = sampler if sampler is not None else sampling.sampler(n_prop_steps=50, n_ene_blocks=5, n_sr_blocks=10)
    return run_blocks(samp, ham, ham_data, prop, prop_data, trial, wave_data, n_eql, fields=fields, zetas=zetas)


def afqmc(ham, ham_data, prop, prop_data: PropData, trial, wave_data, sampler, n_eql: int, n_blocks: int):
    """driver.afqmc's energy path on one rank (driver.py:16-492 without MPI, observables or
    file output): n_eql equilibration sweeps, then n_blocks sampling blocks of `sampler`.
    Returns (weighted mean block energy, its standard error from the block values
    (None for fewer than two blocks), block energies, block weights, prop_data); the
    reference's blocking analysis and outlier rejection of the block record are host-side
    statistics left to the caller."""
    _, _, prop_data = run_equilibration(ham, ham_data, prop, prop_data, trial, wave_data, n_eql)
    be, bw, prop_data = run_blocks(sampler, ham, ham_data, prop, prop_data, trial, wave_data, n_blocks)
    e, w = be.double(), bw.double()
    mean = torch.sum(e * w) / torch.sum(w)
    err = None
    if n_blocks > 1:
        neff = torch.sum(w) ** 2 / torch.sum(w * w)
        var = torch.sum(w * (e - mean) ** 2) / torch.sum(w)
        err = float(torch.sqrt(var / (neff - 1)))
    return float(mean), err, be, bw, prop_data


def run_blocks_ad(sampler, ham, ham_data, prop, prop_data: PropData, trial, wave_data,
                  n_blocks: int, observable=None, do_sr: bool = True, fields=None, zetas=None,
                  ad_mode: str = "forward", orbital_rotation: bool = False):
    """AD branches of driver.py (driver.py:165-229, 245-308 on one
    rank). ad_mode "forward": per block the jvp of sampler.propagate_phaseless_ad_norot
    (do_sr=False: ..._nosr_norot) along the observable; "reverse": its vjp, the block's
    one-body density matrix rdm1 = d energy / d h1, and the observable sum(rdm1 * op). A
    non-finite result is replaced by the trial's value sum(rdm1_T * op) (and rdm1_T), then
    the block weight, QR, global SR and e_estimate update of the non-AD branch follow.
    observable: (op, constant) or None for (h1, 0) as driver.py:35-40. fields (optional):
    [n_blocks, n_sr, n_ene, n_prop, nw, G]; zetas (optional): [n_blocks, n_sr + 1].
    Returns device tensors (block_energy, block_observable, block_weight), each
    [n_blocks], and prop_data; in reverse mode prop_data["block_rdm1s"] holds the
    [n_blocks, 2, norb, norb] density matrices; ad_mode "2rdm" (the vjp of
    sampler.propagate_phaseless_ad_1 with respect to the electron-repulsion tensor, small
    systems) puts the [n_blocks, norb, norb, norb, norb] two-body density matrices into
    prop_data["block_rdm2s"] and reports the trial's observable, as driver.py:230-245 does. orbital_rotation (the reference's
    options["orbital_rotation"], default True there): the jvp / vjp of
    sampler.propagate_phaseless_ad (_nosr), the trial re-optimised for h1 + lambda D in every
    block; wave_data needs "rdm1", as the driver sets it."""
    if ad_mode not in ("forward", "reverse", "2rdm"):
        raise ValueError(f"ad_mode must be 'forward', 'reverse' or '2rdm', got {ad_mode!r}")
    if observable is None:
        op, const = torch.as_tensor(ham_data["h1"]), 0.0
    else:
        op, const = observable[0], float(observable[1])
    op = torch.as_tensor(op, dtype=torch.float64).to(device())
    rdm1 = trial.get_rdm1(wave_data)
    trial_observable = torch.sum(rdm1 * op)
    be = torch.empty(n_blocks, dtype=torch.float64, device=device())
    bo = torch.empty(n_blocks, dtype=torch.float64, device=device())
    bw = torch.empty(n_blocks, dtype=torch.float64, device=device())
    n_sr = sampler.n_sr_blocks if do_sr else 1
    rdm1s = rdm2s = rdm2_op = None
    if ad_mode == "reverse":
        rdm1s = torch.empty((n_blocks, 2, trial.norb, trial.norb), dtype=torch.float64, device=device())
    if ad_mode == "2rdm":  # the electron-repulsion tensor sum_g L_g (x) L_g (driver.py:44-52)
        n = trial.norb
        ch = torch.as_tensor(ham_data["chol"], dtype=torch.float64).to(device()).reshape(-1, n * n)
        rdm2_op = (ch.T @ ch).reshape(n, n, n, n)
        rdm2s = torch.empty((n_blocks, n, n, n, n), dtype=torch.float64, device=device())
    for n in range(n_blocks):
        f = None if fields is None else fields[n]
        z_local = None if (zetas is None or not do_sr) else zetas[n][:n_sr]
        if ad_mode == "forward":
            jvp = sampler.propagate_phaseless_ad_jvp if orbital_rotation else sampler.propagate_phaseless_ad_norot_jvp
            e, de, prop_data = jvp(ham, ham_data, op, prop, prop_data, trial, wave_data, do_sr=do_sr, fields=f,
                                   zetas=z_local)
        elif ad_mode == "2rdm":  # driver.py:230-245: the observable is the trial's value
            e, r2, prop_data = sampler.propagate_phaseless_ad_1_vjp(ham, ham_data, rdm2_op, prop, prop_data, trial,
                                                                    wave_data, fields=f, zetas=z_local)
            rdm2s[n].copy_(r2)
            de = trial_observable.clone()
        else:
            vjp = sampler.propagate_phaseless_ad_vjp if orbital_rotation else sampler.propagate_phaseless_ad_norot_vjp
            e, r, prop_data = vjp(ham, ham_data, prop, prop_data, trial, wave_data, do_sr=do_sr, fields=f,
                                  zetas=z_local)
            de = torch.sum(r * op)
            ok = torch.isfinite(de)
            rdm1s[n].copy_(torch.where(ok, r, rdm1.to(r.dtype)))
        be[n].copy_(e)
        bo[n].copy_(torch.where(torch.isfinite(de), de, trial_observable) + const)
        if zetas is None:
            zg = sampler.draw_zetas(prop_data, 1)
        else:
            zg = torch.as_tensor(zetas[n][-1:], dtype=torch.float64).to(device())
        eng = prop_data["_engine"]
        st = prop_data.state(eng)
        _lib.call("afq_block_end", eng.ctx, ctypes.byref(st), be[n:].data_ptr(), zg.data_ptr(),
                  bw[n:].data_ptr(), stream_ptr())
    if rdm1s is not None:
        dict.__setitem__(prop_data, "block_rdm1s", rdm1s)
    if rdm2s is not None:
        dict.__setitem__(prop_data, "block_rdm2s", rdm2s)
    return be, bo, bw, prop_data
