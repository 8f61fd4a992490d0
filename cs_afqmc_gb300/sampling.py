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
from ._engine import _CACHE_KEY, _scalar, as_dev, device, stream_ptr
from .propagation import PropData, RngKey
from .wavefunctions import _sym


def h1_direction(observable_op, norb: int) -> torch.Tensor:
    """observable_op as the [2, norb, norb] direction added to h1, symmetrised per spin as
    the measurement intermediates symmetrise h1. A [norb, norb] operator acts on both
    spins."""
    op = as_dev(observable_op)
    if op.dim() == 2:
        op = torch.stack([op, op])
    if tuple(op.shape) != (2, norb, norb):
        raise _lib.AfqError(f"observable_op must be [norb, norb] or [2, norb, norb], got {tuple(op.shape)}")
    return _sym(op)


def coupled_ham_data(ham, ham_data: dict, coupling: float, observable_op, prop, trial,
                     wave_data: dict) -> dict:
    """ham_data of h1 + coupling * observable_op with the measurement and propagation
    intermediates rebuilt, the trial held fixed (sampling.py:274-277)."""
    hd = {k: v for k, v in ham_data.items() if k != _CACHE_KEY}
    hd["h1"] = as_dev(ham_data["h1"]) + float(coupling) * h1_direction(observable_op, trial.norb)
    hd = ham.build_measurement_intermediates(hd, trial, wave_data)
    return ham.build_propagation_intermediates(hd, prop, trial, wave_data)


def rotated_ham_data(ham, ham_data: dict, coupling: float, observable_op, prop, trial, wave_data: dict):
    """(ham_data, wave_data) of h1 + coupling * observable_op with the trial re-optimised
    (trial.optimize) and the intermediates rebuilt (sampling.py:187-191). The mean-field
    shifts follow wave_data["rdm1"], which the driver holds fixed (driver.py:54-56); it is
    required here so that they do not silently follow the new trial."""
    if "rdm1" not in wave_data:
        raise _lib.AfqError("orbital rotation needs wave_data['rdm1'] (the driver sets it to the trial's rdm1)")
    hd = {k: v for k, v in ham_data.items() if k != _CACHE_KEY}
    hd["h1"] = as_dev(ham_data["h1"]) + float(coupling) * h1_direction(observable_op, trial.norb)
    wd = trial.optimize(hd, wave_data)
    hd = ham.build_measurement_intermediates(hd, trial, wd)
    return ham.build_propagation_intermediates(hd, prop, trial, wd), wd


def two_body_ham_data(ham, ham_data: dict, op4, prop, trial, wave_data: dict):
    """(ham_data, wave_data, parts) with the Cholesky vectors rebuilt from the two-body
    operator op4 [norb]*4, symmetrised over (ij|kl) = (kl|ij) = (ji|lk) = (lk|ji), by the
    modified Cholesky decomposition with as many vectors as ham_data["chol"], the trial
    re-optimised and the intermediates rebuilt (sampling.py:198-224). parts holds the
    tensors the block depends on (chol, exp_h1, mf, h0_prop), built with torch ops so that
    autograd reaches op4 through them."""
    from .linalg_utils import modified_cholesky
    if "rdm1" not in wave_data:
        raise _lib.AfqError("the two-body derivative needs wave_data['rdm1'] (the driver sets it to the trial's rdm1)")
    norb = trial.norb
    v = as_dev(op4).reshape(norb, norb, norb, norb)
    v = (v + v.permute(2, 3, 0, 1) + v.permute(1, 0, 3, 2) + v.permute(3, 2, 1, 0)) / 4.0
    nchol = int(as_dev(ham_data["chol"]).reshape(-1, norb * norb).shape[0])
    chol = modified_cholesky(v.reshape(norb * norb, norb * norb), norb, nchol)
    hd = {k: val for k, val in ham_data.items() if k not in (_CACHE_KEY, "rot_chol", "rot_h1", "exp_h1",
                                                             "mf_shifts", "h0_prop")}
    hd["chol"] = chol
    wd = trial.optimize(hd, wave_data)
    hd = ham.build_measurement_intermediates(hd, trial, wd)
    hd = ham.build_propagation_intermediates(hd, prop, trial, wd)
    mf, v0, v1 = prop._mf_v0_v1(hd, trial, wd)
    exp_h1 = prop._exp_h1(as_dev(hd["h1"]), v0, v1)
    h0 = float(_scalar(hd["h0"]))
    parts = {"chol": chol, "exp_h1": exp_h1, "mf": mf, "h0_prop": -h0 - torch.sum(mf * mf) / 2.0}
    return hd, wd, parts


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

    def propagate_free(self, ham, ham_data: dict, prop, prop_data: PropData, trial, wave_data: dict,
                       fields: Optional[torch.Tensor] = None):
        """n_blocks free-projection blocks of n_prop_steps steps (sampling.py:95-124, 344-360),
        unrestricted FP64 walkers. fields: [n_blocks, n_prop_steps, nw, nchol] or drawn from
        prop_data["key"]. Returns (prop_data, block_energy, block_weight, key) with complex128
        CUDA tensors [n_blocks]; prop_data is the final state (the reference returns the
        per-block trajectory)."""
        from .propagation import _free_state
        eng = prop._engine(trial, ham_data, wave_data, prop_data["walkers"])
        dict.__setitem__(prop_data, "_engine", eng)
        want = (self.n_blocks, self.n_prop_steps, eng.nw, eng.nchol)
        if fields is None:
            f = torch.empty(want, dtype=torch.float64, device=device())
            key: RngKey = prop_data["key"]
            _lib.call("afq_fill_normal", f.data_ptr(), f.numel(), key.seed, key.take(f.numel()), stream_ptr())
        else:
            f = as_dev(fields)
        if f.numel() != self.n_blocks * self.n_prop_steps * eng.nw * eng.nchol:
            raise _lib.AfqError(f"fields must have shape {want}")
        norms, normed = _free_state(prop_data, eng.nw)
        be = torch.empty(self.n_blocks, dtype=torch.complex128, device=device())
        bw = torch.empty(self.n_blocks, dtype=torch.complex128, device=device())
        st = prop_data.state(eng)
        ene0 = float(complex(_scalar(ham_data.get("ene0", 0.0))).real)
        _lib.call("afq_propagate_free_blocks", eng.ctx, ctypes.byref(st), f.data_ptr(), self.n_prop_steps,
                  self.n_blocks, ene0, norms.data_ptr(), normed.data_ptr(), be.data_ptr(), bw.data_ptr(),
                  stream_ptr())
        return prop_data, be, bw, prop_data.get("key")

    def propagate_phaseless_ad_norot(self, ham, ham_data: dict, coupling: float, observable_op,
                                     prop, prop_data: PropData, trial, wave_data: dict,
                                     fields: Optional[torch.Tensor] = None,
                                     zetas: Optional[torch.Tensor] = None):
        """(energy, prop_data) of the block with h1 + coupling * observable_op and the
        trial held fixed (sampling.py:266-285); the value whose derivative
        propagate_phaseless_ad_norot_jvp returns."""
        hd = ham_data if coupling == 0.0 else coupled_ham_data(ham, ham_data, coupling, observable_op,
                                                                prop, trial, wave_data)
        return self.propagate_phaseless(ham, hd, prop, prop_data, trial, wave_data, fields, zetas)

    def propagate_phaseless_ad_norot_jvp(self, ham, ham_data: dict, observable_op, prop,
                                         prop_data: PropData, trial, wave_data: dict,
                                         coupling: float = 0.0, do_sr: bool = True,
                                         fields: Optional[torch.Tensor] = None,
                                         zetas: Optional[torch.Tensor] = None):
        """Forward-mode derivative of propagate_phaseless_ad_norot (do_sr=False:
        propagate_phaseless_ad_nosr_norot, sampling.py:287-317) along observable_op at
        `coupling`, with a zero tangent on prop_data: what driver.py:207-215 computes with
        jax.jvp. Returns (energy, d energy / d coupling, prop_data), both 0-d CUDA tensors;
        prop_data also gets "block_energies", "block_weights", "dblock_energies",
        "dblock_weights". FP64 (complex128) walkers only."""
        hd = ham_data if coupling == 0.0 else coupled_ham_data(ham, ham_data, coupling, observable_op,
                                                                prop, trial, wave_data)
        eng = prop._engine(trial, hd, wave_data, prop_data["walkers"])
        if eng.precision != _lib.AFQ_PREC_FP64:
            raise _lib.AfqError("the derivative path needs FP64 (complex128) walkers")
        dict.__setitem__(prop_data, "_engine", eng)
        n_sr = self.n_sr_blocks if do_sr else 1
        nblk = n_sr * self.n_ene_blocks
        dh1 = h1_direction(observable_op, trial.norb)
        dexp = prop.exp_h1_tangent(hd, trial, wave_data, dh1)
        drot = trial.rot_h1_tangent(dh1, wave_data)
        if dexp.dim() == 3:
            dexp_up, dexp_dn = dexp[0].contiguous(), dexp[1].contiguous()
        else:
            dexp_up, dexp_dn = dexp, None
        if isinstance(drot, list):
            drot_up, drot_dn = drot
        else:
            drot_up, drot_dn = drot, None
        f, z = self._ad_draws(eng, prop_data, n_sr, do_sr, fields, zetas)
        return self._jvp_call(eng, prop_data, nblk, n_sr, do_sr, f, z, (dexp_up, dexp_dn), (drot_up, drot_dn))

    def propagate_phaseless_ad(self, ham, ham_data: dict, coupling: float, observable_op, prop,
                               prop_data: PropData, trial, wave_data: dict,
                               fields: Optional[torch.Tensor] = None, zetas: Optional[torch.Tensor] = None):
        """(energy, prop_data) of the block with h1 + coupling * observable_op and the trial
        re-optimised for it (sampling.py:173-196); the value whose derivative
        propagate_phaseless_ad_jvp returns."""
        hd, wd = rotated_ham_data(ham, ham_data, coupling, observable_op, prop, trial, wave_data)
        return self.propagate_phaseless(ham, hd, prop, prop_data, trial, wd, fields, zetas)

    def propagate_phaseless_ad_jvp(self, ham, ham_data: dict, observable_op, prop, prop_data: PropData, trial,
                                   wave_data: dict, coupling: float = 0.0, do_sr: bool = True,
                                   fields: Optional[torch.Tensor] = None, zetas: Optional[torch.Tensor] = None):
        """Forward-mode derivative of propagate_phaseless_ad (do_sr=False:
        propagate_phaseless_ad_nosr, sampling.py:221-254) along observable_op at `coupling`,
        with the trial's dependence on the coupling through trial.optimize: what
        driver.py:207-215 computes with jax.jvp when options["orbital_rotation"] is on (its
        default). Returns (energy, d energy / d coupling, prop_data) as
        propagate_phaseless_ad_norot_jvp does. FP64 (complex128) walkers only."""
        if "rdm1" not in wave_data:
            raise _lib.AfqError("orbital rotation needs wave_data['rdm1'] (the driver sets it to the trial's rdm1)")
        dh1 = h1_direction(observable_op, trial.norb)
        h0 = {k: v for k, v in ham_data.items() if k != _CACHE_KEY}
        h0["h1"] = as_dev(ham_data["h1"]) + float(coupling) * dh1
        wd, dmo = trial.optimize_tangent(h0, wave_data, dh1)
        hd = ham.build_measurement_intermediates(h0, trial, wd)
        hd = ham.build_propagation_intermediates(hd, prop, trial, wd)
        eng = prop._engine(trial, hd, wd, prop_data["walkers"])
        if eng.precision != _lib.AFQ_PREC_FP64:
            raise _lib.AfqError("the derivative path needs FP64 (complex128) walkers")
        dict.__setitem__(prop_data, "_engine", eng)
        n_sr = self.n_sr_blocks if do_sr else 1
        nblk = n_sr * self.n_ene_blocks
        dexp = prop.exp_h1_tangent(hd, trial, wd, dh1)
        dexp_up, dexp_dn = (dexp[0].contiguous(), dexp[1].contiguous()) if dexp.dim() == 3 else (dexp, None)
        drot, drc = trial.rotation_tangents(hd, wd, dmo, dh1)
        uhf_trial = isinstance(drot, list)
        dtr = (dmo[0], dmo[1]) if uhf_trial else (dmo, None)
        drot_p = (drot[0], drot[1]) if uhf_trial else (drot, None)
        drc_p = (drc[0], drc[1]) if uhf_trial else (drc, None)
        f, z = self._ad_draws(eng, prop_data, n_sr, do_sr, fields, zetas)
        return self._jvp_call(eng, prop_data, nblk, n_sr, do_sr, f, z, (dexp_up, dexp_dn), drot_p, dtr, drc_p)

    def _jvp_call(self, eng, prop_data: PropData, nblk: int, n_sr: int, do_sr: bool, f, z, dexp, drot,
                  dtrial=(None, None), drc=(None, None)):
        """afq_propagate_phaseless_jvp_ex with the tangent inputs; returns (energy, d energy,
        prop_data) and records the per-block values and derivatives in prop_data."""
        def ptr(x):
            return None if x is None else x.data_ptr()

        tin = _lib.JvpInputs(ptr(dexp[0]), ptr(dexp[1]), ptr(drot[0]), ptr(drot[1]), ptr(dtrial[0]),
                             ptr(dtrial[1]), ptr(drc[0]), ptr(drc[1]))
        tws = getattr(eng, "tangent_workspace", None)
        nbytes = eng.lib.afq_tangent_workspace_size(ctypes.byref(eng.dims))
        if nbytes == 0:
            raise _lib.AfqError("afq_tangent_workspace_size: " + eng.lib.afq_last_error().decode())
        if tws is None or tws.numel() < nbytes + 256:
            tws = torch.empty(nbytes + 256, dtype=torch.uint8, device=device())
            eng.tangent_workspace = tws
        tptr = tws.data_ptr() + (-tws.data_ptr()) % 256
        out = torch.empty(4 * nblk + 2, dtype=torch.float64, device=device())
        be, bw, dbe, dbw = (out[i * nblk:(i + 1) * nblk] for i in range(4))
        energy, denergy = out[4 * nblk:4 * nblk + 1], out[4 * nblk + 1:]
        st = prop_data.state(eng)
        _lib.call("afq_propagate_phaseless_jvp_ex", eng.ctx, ctypes.byref(st), ctypes.byref(tin), tptr, nbytes,
                  f.data_ptr(), None if z is None else z.data_ptr(), self.n_prop_steps, self.n_ene_blocks, n_sr,
                  0 if do_sr else _lib.AFQ_JVP_NO_SR, be.data_ptr(), bw.data_ptr(), dbe.data_ptr(),
                  dbw.data_ptr(), energy.data_ptr(), denergy.data_ptr(), stream_ptr())
        dict.__setitem__(prop_data, "block_energies", be)
        dict.__setitem__(prop_data, "block_weights", bw)
        dict.__setitem__(prop_data, "dblock_energies", dbe)
        dict.__setitem__(prop_data, "dblock_weights", dbw)
        return energy[0], denergy[0], prop_data

    def _ad_draws(self, eng, prop_data: PropData, n_sr: int, do_sr: bool, fields, zetas):
        """Fields [n_sr, n_ene, n_prop, nw, nchol] and SR uniforms [n_sr] of one AD block,
        drawn from prop_data["key"] where not given."""
        nblk = n_sr * self.n_ene_blocks
        want = (n_sr, self.n_ene_blocks, self.n_prop_steps, eng.nw, eng.nchol)
        if fields is None:
            f = torch.empty(want, dtype=torch.float64, device=device())
            key: RngKey = prop_data["key"]
            _lib.call("afq_fill_normal", f.data_ptr(), f.numel(), key.seed, key.take(f.numel()),
                      stream_ptr())
        else:
            f = as_dev(fields)
        if f.numel() != nblk * self.n_prop_steps * eng.nw * eng.nchol:
            raise _lib.AfqError(f"fields must have shape {want}")
        if do_sr:
            z = self.draw_zetas(prop_data, n_sr) if zetas is None else as_dev(zetas)
            if z.numel() != n_sr:
                raise _lib.AfqError(f"zetas must have {n_sr} entries")
        else:
            z = None
        return f, z

    def propagate_phaseless_ad_norot_vjp(self, ham, ham_data: dict, prop, prop_data: PropData, trial,
                                         wave_data: dict, do_sr: bool = True,
                                         fields: Optional[torch.Tensor] = None,
                                         zetas: Optional[torch.Tensor] = None):
        """Reverse-mode derivative of propagate_phaseless_ad_norot (do_sr=False:
        propagate_phaseless_ad_nosr_norot): what driver.py:217-224 computes with jax.vjp at
        coupling 1 and a zero rdm_op, i.e. the gradient of the block energy with respect to
        h1, the block's one-body density matrix estimate. Returns (energy 0-d, rdm1
        [2, norb, norb], prop_data), CUDA tensors; prop_data also gets "block_energies" and
        "block_weights". FP64 (complex128) walkers only."""
        energy, g, prop_data = self._vjp_call(prop, prop_data, trial, ham_data, wave_data, do_sr, fields, zetas,
                                              rotation=False)
        gexp, grot = g[0], g[1]
        uhf_trial = isinstance(wave_data["mo_coeff"], (list, tuple))
        g_exp = prop.exp_h1_cotangent(ham_data, trial, wave_data, gexp if not prop.restricted else gexp[0])
        g_rot = trial.rot_h1_cotangent(grot if uhf_trial else grot[0], wave_data)
        rdm1 = _sym(g_exp + g_rot)  # the transpose of the per-spin symmetrisation is itself
        return energy, rdm1, prop_data

    def propagate_phaseless_ad_vjp(self, ham, ham_data: dict, prop, prop_data: PropData, trial, wave_data: dict,
                                   do_sr: bool = True, fields: Optional[torch.Tensor] = None,
                                   zetas: Optional[torch.Tensor] = None):
        """Reverse-mode derivative of propagate_phaseless_ad (do_sr=False:
        propagate_phaseless_ad_nosr): the block's one-body density matrix d energy / d h1 with
        the trial's dependence on h1 through trial.optimize, what driver.py:217-224 computes
        with jax.vjp under the default options["orbital_rotation"]. The device sweep returns
        the gradients with respect to exp_h1, rot_h1, the trial and rot_chol; the map from h1
        to those (the SCF tangent of trial.optimize, the trial rotation, the Frechet
        derivative of expm) is linear in the direction, so its transpose is taken with torch
        autograd through the same tangent code the forward mode uses. Returns (energy, rdm1
        [2, norb, norb], prop_data)."""
        if "rdm1" not in wave_data:
            raise _lib.AfqError("orbital rotation needs wave_data['rdm1'] (the driver sets it to the trial's rdm1)")
        h0 = {k: v for k, v in ham_data.items() if k != _CACHE_KEY}
        wd = trial.optimize(h0, wave_data)
        hd = ham.build_measurement_intermediates(h0, trial, wd)
        hd = ham.build_propagation_intermediates(hd, prop, trial, wd)
        energy, g, prop_data = self._vjp_call(prop, prop_data, trial, hd, wd, do_sr, fields, zetas, rotation=True)
        gexp, grot, gtrial, grc = g
        uhf_trial = isinstance(wd["mo_coeff"], (list, tuple))
        norb = trial.norb
        nchol = int(hd["chol"].shape[0])
        D = torch.zeros((2, norb, norb), dtype=torch.float64, device=device(), requires_grad=True)
        with torch.enable_grad():
            dh1 = _sym(D)
            _, dmo = trial.optimize_tangent(h0, wave_data, dh1)
            dexp = prop.exp_h1_tangent(hd, trial, wd, dh1)
            drot, drc = trial.rotation_tangents(hd, wd, dmo, dh1)
            ge = gexp if not prop.restricted else gexp[0]
            lin = torch.sum(ge * dexp)
            if uhf_trial:
                n_up, n_dn = trial.nelec
                rc = grc.reshape(nchol, -1)
                lin = lin + torch.sum(grot[0] * drot[0]) + torch.sum(grot[1] * drot[1])
                lin = lin + torch.sum(gtrial[0] * dmo[0]) + torch.sum(gtrial[1] * dmo[1])
                lin = lin + torch.sum(rc[:, :n_up * norb].reshape(drc[0].shape) * drc[0])
                lin = lin + torch.sum(rc[:, n_up * norb:].reshape(drc[1].shape) * drc[1])
            else:
                lin = lin + torch.sum(grot[0] * drot) + torch.sum(gtrial[0] * dmo)
                lin = lin + torch.sum(grc.reshape(drc.shape) * drc)
            (rdm1,) = torch.autograd.grad(lin, D)
        return energy, rdm1.detach(), prop_data

    def propagate_phaseless_ad_1(self, ham, ham_data: dict, coupling: float, observable_op, prop,
                                 prop_data: PropData, trial, wave_data: dict,
                                 fields: Optional[torch.Tensor] = None, zetas: Optional[torch.Tensor] = None):
        """(energy, prop_data) of the block whose Cholesky vectors are rebuilt from the
        two-body operator observable_op [norb]*4 (symmetrised over its four index
        permutations, modified Cholesky with as many vectors as ham_data["chol"]), the
        trial re-optimised (sampling.py:198-229). `coupling` is unused, as in the
        reference."""
        with torch.no_grad():
            hd, wd, _ = two_body_ham_data(ham, ham_data, observable_op, prop, trial, wave_data)
        return self.propagate_phaseless(ham, hd, prop, prop_data, trial, wd, fields, zetas)

    def propagate_phaseless_ad_1_vjp(self, ham, ham_data: dict, observable_op, prop, prop_data: PropData, trial,
                                     wave_data: dict, fields: Optional[torch.Tensor] = None,
                                     zetas: Optional[torch.Tensor] = None):
        """Reverse-mode derivative of propagate_phaseless_ad_1 with respect to the two-body
        operator: what driver.py:230-234 takes with jax.vjp in ad_mode "2rdm" (the block's
        two-body density matrix estimate when observable_op is the electron-repulsion
        tensor). The device sweep returns the gradients with respect to exp_h1, rot_h1, the
        trial, rot_chol, chol, the mean-field shifts and h0_prop; torch autograd carries them
        back through the intermediates, trial.optimize and the modified Cholesky
        decomposition. Returns (energy, rdm2 [norb]*4, prop_data). FP64 walkers only; the
        host part holds norb^4-sized tensors and a graph of the decomposition (small
        systems)."""
        op = as_dev(observable_op).detach().clone().requires_grad_(True)
        with torch.enable_grad():
            hd, wd, parts = two_body_ham_data(ham, ham_data, op, prop, trial, wave_data)
            plain = {k: (v.detach() if isinstance(v, torch.Tensor) else v) for k, v in hd.items()}
            plain["rot_chol"] = [x.detach() for x in hd["rot_chol"]] if isinstance(hd["rot_chol"], list) \
                else hd["rot_chol"].detach()
            plain["rot_h1"] = [x.detach() for x in hd["rot_h1"]] if isinstance(hd["rot_h1"], list) \
                else hd["rot_h1"].detach()
            wplain = dict(wd)
            wplain["mo_coeff"] = [x.detach() for x in wd["mo_coeff"]] if isinstance(wd["mo_coeff"], list) \
                else wd["mo_coeff"].detach()
            energy, g, prop_data = self._vjp_call(prop, prop_data, trial, plain, wplain, True, fields, zetas,
                                                  rotation=True, chol_grads=True)
            gexp, grot, gtrial, grc, gchol, gmf, gh0p = g
            uhf_trial = isinstance(wd["mo_coeff"], (list, tuple))
            norb = trial.norb
            nchol = int(parts["chol"].shape[0])
            exp_h1 = parts["exp_h1"]
            lin = torch.sum((gexp if exp_h1.dim() == 3 else gexp[0]) * exp_h1)
            lin = lin + torch.sum(gchol * parts["chol"])
            mf, h0p = parts["mf"], parts["h0_prop"]
            lin = lin + torch.sum(gmf.real * mf.real + gmf.imag * mf.imag)
            lin = lin + gh0p.real * h0p.real + gh0p.imag * h0p.imag
            if uhf_trial:
                n_up = trial.nelec[0]
                rc = grc.reshape(nchol, -1)
                for s_, (o0, o1) in enumerate(((0, n_up * norb), (n_up * norb, rc.shape[1]))):
                    lin = lin + torch.sum(rc[:, o0:o1].reshape(hd["rot_chol"][s_].shape) * hd["rot_chol"][s_])
                    lin = lin + torch.sum(grot[s_] * hd["rot_h1"][s_]) + torch.sum(gtrial[s_] * wd["mo_coeff"][s_])
            else:
                lin = lin + torch.sum(grc.reshape(hd["rot_chol"].shape) * hd["rot_chol"])
                lin = lin + torch.sum(grot[0] * hd["rot_h1"]) + torch.sum(gtrial[0] * wd["mo_coeff"])
            (rdm2,) = torch.autograd.grad(lin, op)
        return energy, rdm2.detach(), prop_data

    def propagate_phaseless_chol_vjp(self, ham, ham_data: dict, prop, prop_data: PropData, trial, wave_data: dict,
                                     do_sr: bool = True, fields: Optional[torch.Tensor] = None,
                                     zetas: Optional[torch.Tensor] = None):
        """Reverse-mode derivative of the block energy of propagate_phaseless with respect to
        the Cholesky vectors, the trial held fixed: every quantity that depends on them -
        the vhs operator, the mean-field shifts, h0_prop, exp_h1 (through v0 and the
        mean-field part of h1_mod) and rot_chol (propagation.py:292-325,
        wavefunctions.py:602-619) - is rebuilt with torch ops, the device sweep returns the
        cotangents of each (afq_propagate_phaseless_vjp_ex), and torch autograd carries them
        back to chol. This is the chain the reference differentiates with jax.vjp when its
        two-body mode varies the Cholesky vectors (sampling.py:198-229, driver.py:230-245),
        here without re-optimising the trial. Returns (energy, d energy / d chol
        [nchol, norb * norb], prop_data). FP64 walkers only."""
        if "rdm1" not in wave_data:
            raise _lib.AfqError("the Cholesky derivative needs wave_data['rdm1'] (the driver sets it to the trial's rdm1)")
        norb = trial.norb
        chol = as_dev(ham_data["chol"]).reshape(-1, norb * norb).detach().clone().requires_grad_(True)
        nchol = int(chol.shape[0])
        with torch.enable_grad():
            hd = {k: v for k, v in ham_data.items() if k not in (_CACHE_KEY, "rot_chol", "rot_h1", "exp_h1",
                                                                 "mf_shifts", "h0_prop")}
            hd["chol"] = chol
            hd = ham.build_measurement_intermediates(hd, trial, wave_data)
            hd = ham.build_propagation_intermediates(hd, prop, trial, wave_data)
            mf, v0, v1 = prop._mf_v0_v1(hd, trial, wave_data)
            exp_h1 = prop._exp_h1(as_dev(hd["h1"]), v0, v1)
            h0p = -float(_scalar(hd["h0"])) - torch.sum(mf * mf) / 2.0
            plain = {k: (v.detach() if isinstance(v, torch.Tensor) else v) for k, v in hd.items()}
            for key in ("rot_chol", "rot_h1"):
                plain[key] = [x.detach() for x in hd[key]] if isinstance(hd[key], list) else hd[key].detach()
            energy, g, prop_data = self._vjp_call(prop, prop_data, trial, plain, wave_data, do_sr, fields, zetas,
                                                  rotation=True, chol_grads=True)
            gexp, _, _, grc, gchol, gmf, gh0p = g
            lin = torch.sum((gexp if exp_h1.dim() == 3 else gexp[0]) * exp_h1)
            lin = lin + torch.sum(gchol * chol)
            lin = lin + torch.sum(gmf.real * mf.real + gmf.imag * mf.imag)
            lin = lin + gh0p.real * h0p.real + gh0p.imag * h0p.imag
            if isinstance(hd["rot_chol"], list):
                n_up = trial.nelec[0]
                rc = grc.reshape(nchol, -1)
                for s_, (o0, o1) in enumerate(((0, n_up * norb), (n_up * norb, rc.shape[1]))):
                    lin = lin + torch.sum(rc[:, o0:o1].reshape(hd["rot_chol"][s_].shape) * hd["rot_chol"][s_])
            else:
                lin = lin + torch.sum(grc.reshape(hd["rot_chol"].shape) * hd["rot_chol"])
            (gc,) = torch.autograd.grad(lin, chol)
        return energy, gc.detach(), prop_data

    def propagate_phaseless_u_vjp(self, ham, ham_data: dict, u: float, prop, prop_data: PropData, trial,
                                  wave_data: dict, do_sr: bool = True, fields: Optional[torch.Tensor] = None,
                                  zetas: Optional[torch.Tensor] = None):
        """d (block energy) / dU for Cholesky vectors proportional to sqrt(U), as in the
        Hubbard model's L_i = sqrt(U) n_i: dL/dU = L / (2U), so dE/dU = <dE/dL, L> / (2U).
        Returns (energy, dE/dU, prop_data)."""
        if not u > 0:
            raise _lib.AfqError("U must be positive")
        energy, gc, prop_data = self.propagate_phaseless_chol_vjp(ham, ham_data, prop, prop_data, trial, wave_data,
                                                                   do_sr, fields, zetas)
        chol = as_dev(ham_data["chol"]).reshape(gc.shape)
        return energy, torch.sum(gc * chol) / (2.0 * float(u)), prop_data

    def _vjp_call(self, prop, prop_data: PropData, trial, ham_data: dict, wave_data: dict, do_sr: bool, fields,
                  zetas, rotation: bool, chol_grads: bool = False):
        """afq_propagate_phaseless_vjp_ex on the engine of (trial, ham_data, wave_data).
        Returns (energy 0-d, (gexp [2, norb, norb], grot [up, dn or None], gtrial, grot_chol),
        prop_data); gtrial / grot_chol only with rotation."""
        eng = prop._engine(trial, ham_data, wave_data, prop_data["walkers"])
        if eng.precision != _lib.AFQ_PREC_FP64:
            raise _lib.AfqError("the derivative path needs FP64 (complex128) walkers")
        dict.__setitem__(prop_data, "_engine", eng)
        n_sr = self.n_sr_blocks if do_sr else 1
        nblk = n_sr * self.n_ene_blocks
        f, z = self._ad_draws(eng, prop_data, n_sr, do_sr, fields, zetas)
        nbytes = eng.lib.afq_vjp_workspace_size(ctypes.byref(eng.dims), self.n_prop_steps,
                                                self.n_ene_blocks, n_sr)
        if nbytes == 0:
            raise _lib.AfqError("afq_vjp_workspace_size: " + eng.lib.afq_last_error().decode())
        vws = getattr(eng, "vjp_workspace", None)
        if vws is None or vws.numel() < nbytes + 256:
            vws = torch.empty(nbytes + 256, dtype=torch.uint8, device=device())
            eng.vjp_workspace = vws
        vptr = vws.data_ptr() + (-vws.data_ptr()) % 256
        norb = trial.norb
        dev = device()
        out = torch.empty(2 * nblk + 1, dtype=torch.float64, device=dev)
        be, bw, energy = out[:nblk], out[nblk:2 * nblk], out[2 * nblk:]
        gexp = torch.empty((2, norb, norb), dtype=torch.float64, device=dev)
        n_up, n_dn = trial.nelec
        uhf_trial = isinstance(wave_data["mo_coeff"], (list, tuple))
        occ = (n_up, n_dn) if uhf_trial else (n_up,)
        grot = [torch.empty((o, norb), dtype=torch.float64, device=dev) for o in occ] + ([] if uhf_trial else [None])
        gtrial, grc = [None, None], None
        gchol = gmf = gh0p = None
        if chol_grads:
            nch = int(ham_data["chol"].shape[0])
            gchol = torch.empty((nch, norb * norb), dtype=torch.float64, device=dev)
            gmf = torch.empty(nch, dtype=torch.complex128, device=dev)
            gh0p = torch.empty(1, dtype=torch.complex128, device=dev)
        if rotation:
            gtrial = [torch.empty((norb, o), dtype=torch.float64, device=dev) for o in occ] + \
                ([] if uhf_trial else [None])
            grc = torch.empty((int(ham_data["chol"].shape[0]), sum(occ) * norb), dtype=torch.float64, device=dev)

        def ptr(x):
            return None if x is None else x.data_ptr()

        outs = _lib.VjpOutputs(gexp[0].data_ptr(), None if prop.restricted else gexp[1].data_ptr(), ptr(grot[0]),
                               ptr(grot[1]), ptr(gtrial[0]), ptr(gtrial[1]), ptr(grc), ptr(gchol), ptr(gmf),
                               ptr(gh0p))
        st = prop_data.state(eng)
        _lib.call("afq_propagate_phaseless_vjp_ex", eng.ctx, ctypes.byref(st), vptr, nbytes, f.data_ptr(),
                  None if z is None else z.data_ptr(), self.n_prop_steps, self.n_ene_blocks, n_sr,
                  0 if do_sr else _lib.AFQ_JVP_NO_SR, be.data_ptr(), bw.data_ptr(), energy.data_ptr(),
                  ctypes.byref(outs), stream_ptr())
        dict.__setitem__(prop_data, "block_energies", be)
        dict.__setitem__(prop_data, "block_weights", bw)
        if chol_grads:
            return energy[0], (gexp, grot, gtrial, grc, gchol, gmf, gh0p[0]), prop_data
        return energy[0], (gexp, grot, gtrial, grc), prop_data

    def __hash__(self) -> int:
        return hash((self.n_prop_steps, self.n_ene_blocks, self.n_sr_blocks, self.n_blocks))
