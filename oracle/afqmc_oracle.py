"""FP64 NumPy oracle for the phaseless-AFQMC walker-propagation and local-energy path.

This module is TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and only as the
checker or as the timed CPU restatement of the reference. The product path
(``cs_afqmc_gb300``) never calls it.

It restates, in plain NumPy at float64/complex128, the reference package ``ad_afqmc``
(zh-yichi/cs_afqmc, pure Python on JAX), line by line, for:

* RHF / UHF trial measurements: overlap, half Green's function, force bias, mixed local
  energy, half-rotated intermediates (ad_afqmc/wavefunctions.py)
* propagation intermediates and the phaseless propagation step
  (ad_afqmc/propagation.py)
* QR orthonormalisation (ad_afqmc/linalg_utils.py) and comb stochastic reconfiguration
  (ad_afqmc/sr.py)
* the sampler's block loop and the driver's per-block bookkeeping
  (ad_afqmc/sampling.py, ad_afqmc/driver.py)

Parity pin: the RHF/UHF known-answer values of tests/test_wavefunctions.py:127-183 in the
reference (overlap, Green's-function sum, force-bias sum, energy at the seed-102 fixture)
are reproduced by this module; ``tests/test_oracle_golden.py`` checks them. The functions
beyond those (propagate, QR, SR, block loop) are pinned by restatement only: the
reference's own tests check them by output shape (tests/test_propagation.py:88-127).

Random inputs are never drawn here: auxiliary fields and the SR uniforms are arguments, so
the oracle and the GPU path consume identical draws. JAX's PRNG streams are not reproduced.

Walker containers follow the reference: restricted walkers are one array
``[nw, norb, max(n_up, n_dn)]``; unrestricted walkers are a 2-list ``[up, dn]`` with shapes
``[nw, norb, n_up]`` and ``[nw, norb, n_dn]``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np
import scipy.linalg

# ----------------------------------------------------------------------------------------
# small batched helpers
# ----------------------------------------------------------------------------------------


def _h(a: np.ndarray) -> np.ndarray:
    """Conjugate transpose of the last two axes."""
    return np.conj(np.swapaxes(a, -1, -2))


def _t(a: np.ndarray) -> np.ndarray:
    return np.swapaxes(a, -1, -2)


# ----------------------------------------------------------------------------------------
# RHF trial  (wavefunctions.py:453-635)
# ----------------------------------------------------------------------------------------


def rhf_overlap_restricted(walkers: np.ndarray, mo: np.ndarray) -> np.ndarray:
    """det(C^H W)^2 per walker (wavefunctions.py:478-480). walkers [nw,norb,nocc]."""
    return np.linalg.det(_h(mo) @ walkers) ** 2


def rhf_overlap(walkers_up, walkers_dn, mo) -> np.ndarray:
    """det(C^H W_up) det(C^H W_dn) (wavefunctions.py:482-488)."""
    return np.linalg.det(_h(mo) @ walkers_up) * np.linalg.det(_h(mo) @ walkers_dn)


def rhf_green(walkers: np.ndarray, mo: np.ndarray) -> np.ndarray:
    """Half Green's function (W (C^H W)^-1)^T, shape [nw, nocc, norb]
    (wavefunctions.py:490-501)."""
    return _t(walkers @ np.linalg.inv(_h(mo) @ walkers))


def rhf_force_bias_restricted(walkers, rot_chol, mo) -> np.ndarray:
    """2 sum_ij rot_chol[g,i,j] G[i,j] (wavefunctions.py:503-511)."""
    g = rhf_green(walkers, mo)
    return 2.0 * np.einsum("gij,wij->wg", rot_chol, g, optimize=True)


def rhf_force_bias(walkers_up, walkers_dn, rot_chol, mo) -> np.ndarray:
    """Two-slab walkers, G_up + G_dn contracted once (wavefunctions.py:513-527)."""
    g = rhf_green(walkers_up, mo) + rhf_green(walkers_dn, mo)
    return np.einsum("gij,wij->wg", rot_chol, g, optimize=True)


def _exchange_coulomb(rot_chol: np.ndarray, green: np.ndarray):
    """f_g = rot_chol_g G^T per walker; returns (c [nw,G], exc [nw]) with c_g = tr f_g and
    exc = sum_g sum_ik f_g[i,k] f_g[k,i] (wavefunctions.py:537-539)."""
    f = np.einsum("gij,wkj->wgik", rot_chol, green, optimize=True)
    c = np.einsum("wgii->wg", f, optimize=True)
    exc = np.einsum("wgik,wgki->w", f, f, optimize=True)
    return c, exc


def rhf_energy_restricted(walkers, h0, rot_h1, rot_chol, mo) -> np.ndarray:
    """Mixed local energy, RHF restricted walkers (wavefunctions.py:529-541):
    h0 + 2 sum G*rot_h1 + 2 sum_g c_g^2 - exc."""
    g = rhf_green(walkers, mo)
    ene1 = 2.0 * np.einsum("wij,ij->w", g, rot_h1, optimize=True)
    c, exc = _exchange_coulomb(rot_chol, g)
    ene2 = 2.0 * np.sum(c * c, axis=1) - exc
    return ene2 + ene1 + h0


def rhf_energy(walkers_up, walkers_dn, h0, rot_h1, rot_chol, mo) -> np.ndarray:
    """Two-slab walkers with the RHF trial (wavefunctions.py:543-561)."""
    g = rhf_green(walkers_up, mo) + rhf_green(walkers_dn, mo)
    ene1 = np.einsum("wij,ij->w", g, rot_h1, optimize=True)
    c, exc = _exchange_coulomb(rot_chol, g)
    return np.sum(c * c, axis=1) - exc + ene1 + h0


def rhf_build_measurement_intermediates(ham_data: dict, mo: np.ndarray, norb: int) -> dict:
    """Symmetrise h1 per spin with (h + h^T)/2 (not Hermitian), rot_h1 = C^H (h1_a+h1_b)/2,
    rot_chol_g = C^H L_g (wavefunctions.py:602-619)."""
    h1 = np.array(ham_data["h1"])
    h1 = np.stack([(h1[0] + h1[0].T) / 2.0, (h1[1] + h1[1].T) / 2.0])
    ham_data["h1"] = h1
    ham_data["rot_h1"] = _h(mo) @ ((h1[0] + h1[1]) / 2.0)
    ham_data["rot_chol"] = np.einsum(
        "pi,gij->gpj", _h(mo), np.asarray(ham_data["chol"]).reshape(-1, norb, norb)
    )
    return ham_data


# ----------------------------------------------------------------------------------------
# UHF trial  (wavefunctions.py:638-844)
# ----------------------------------------------------------------------------------------


def uhf_overlap(walkers_up, walkers_dn, mo: Sequence[np.ndarray]) -> np.ndarray:
    """det(C_a^H W_up) det(C_b^H W_dn) (wavefunctions.py:658-667)."""
    return np.linalg.det(_h(mo[0]) @ walkers_up) * np.linalg.det(_h(mo[1]) @ walkers_dn)


def uhf_green(walkers_up, walkers_dn, mo) -> List[np.ndarray]:
    """[G_up [nw,n_up,norb], G_dn [nw,n_dn,norb]] (wavefunctions.py:669-692)."""
    return [rhf_green(walkers_up, mo[0]), rhf_green(walkers_dn, mo[1])]


def uhf_force_bias(walkers_up, walkers_dn, rot_chol, mo) -> np.ndarray:
    """sum over spins of rot_chol[s]:G[s] (wavefunctions.py:694-709)."""
    g = uhf_green(walkers_up, walkers_dn, mo)
    return np.einsum("gij,wij->wg", rot_chol[0], g[0]) + np.einsum(
        "gij,wij->wg", rot_chol[1], g[1]
    )


def uhf_energy(walkers_up, walkers_dn, h0, rot_h1, rot_chol, mo) -> np.ndarray:
    """(sum c_up^2 + sum c_dn^2 + 2 sum c_up c_dn - exc_up - exc_dn)/2 + ene1 + h0
    (wavefunctions.py:711-743)."""
    g = uhf_green(walkers_up, walkers_dn, mo)
    ene1 = (np.einsum("wij,ij->w", g[0], rot_h1[0], optimize=True)
            + np.einsum("wij,ij->w", g[1], rot_h1[1], optimize=True))
    c_up, exc_up = _exchange_coulomb(rot_chol[0], g[0])
    c_dn, exc_dn = _exchange_coulomb(rot_chol[1], g[1])
    ene2 = (
        np.sum(c_up * c_up, 1) + np.sum(c_dn * c_dn, 1) + 2.0 * np.sum(c_up * c_dn, 1)
        - exc_up - exc_dn
    ) / 2.0
    return ene2 + ene1 + h0


def uhf_build_measurement_intermediates(ham_data: dict, mo, norb: int) -> dict:
    """(wavefunctions.py:817-841)."""
    h1 = np.array(ham_data["h1"])
    h1 = np.stack([(h1[0] + h1[0].T) / 2.0, (h1[1] + h1[1].T) / 2.0])
    ham_data["h1"] = h1
    ham_data["rot_h1"] = [_h(mo[0]) @ h1[0], _h(mo[1]) @ h1[1]]
    chol = np.asarray(ham_data["chol"]).reshape(-1, norb, norb)
    ham_data["rot_chol"] = [
        np.einsum("pi,gij->gpj", _h(mo[0]), chol),
        np.einsum("pi,gij->gpj", _h(mo[1]), chol),
    ]
    return ham_data


# ----------------------------------------------------------------------------------------
# Trial dispatch (the singledispatch of wavefunctions.py:45-241)
# ----------------------------------------------------------------------------------------


@dataclass
class Trial:
    """kind 'rhf' (wave_data mo [norb,nocc]) or 'uhf' (mo = [C_a, C_b])."""

    kind: str
    norb: int
    nelec: Tuple[int, int]

    def overlap(self, walkers, mo):
        if isinstance(walkers, list):
            if self.kind == "rhf":
                return rhf_overlap(walkers[0], walkers[1], mo)
            return uhf_overlap(walkers[0], walkers[1], mo)
        if self.kind == "rhf":
            return rhf_overlap_restricted(walkers, mo)
        # base-class restricted dispatch: slice the single slab (wavefunctions.py:98-104)
        return uhf_overlap(walkers[:, :, : self.nelec[0]], walkers[:, :, : self.nelec[1]], mo)

    def force_bias(self, walkers, ham_data, mo):
        rc = ham_data["rot_chol"]
        if isinstance(walkers, list):
            if self.kind == "rhf":
                return rhf_force_bias(walkers[0], walkers[1], rc, mo)
            return uhf_force_bias(walkers[0], walkers[1], rc, mo)
        if self.kind == "rhf":
            return rhf_force_bias_restricted(walkers, rc, mo)
        return uhf_force_bias(walkers[:, :, : self.nelec[0]], walkers[:, :, : self.nelec[1]], rc, mo)

    def energy(self, walkers, ham_data, mo):
        h0, rh1, rc = ham_data["h0"], ham_data["rot_h1"], ham_data["rot_chol"]
        if isinstance(walkers, list):
            if self.kind == "rhf":
                return rhf_energy(walkers[0], walkers[1], h0, rh1, rc, mo)
            return uhf_energy(walkers[0], walkers[1], h0, rh1, rc, mo)
        if self.kind == "rhf":
            return rhf_energy_restricted(walkers, h0, rh1, rc, mo)
        return uhf_energy(
            walkers[:, :, : self.nelec[0]], walkers[:, :, : self.nelec[1]], h0, rh1, rc, mo
        )

    def build_measurement_intermediates(self, ham_data, mo):
        if self.kind == "rhf":
            return rhf_build_measurement_intermediates(ham_data, mo, self.norb)
        return uhf_build_measurement_intermediates(ham_data, mo, self.norb)


# ----------------------------------------------------------------------------------------
# Propagation intermediates  (propagation.py:292-325 restricted, 464-509 unrestricted)
# ----------------------------------------------------------------------------------------


def build_propagation_intermediates(
    ham_data: dict, rdm1: np.ndarray, norb: int, nelec, dt: float, restricted: bool
) -> dict:
    """mf_shifts_g = i sum L_g*(rho_a+rho_b); h0_prop = -h0 - sum mf^2/2;
    v0 = 1/2 sum_g L_g L_g^T; h1_mod = h1 - v0 - Re(i sum_g mf_g L_g); exp_h1 = expm(-dt h1_mod/2).

    The restricted propagator averages the two spin blocks of h1 (propagation.py:315); the
    unrestricted one keeps one exp_h1 per spin (propagation.py:497-508).
    """
    chol = np.asarray(ham_data["chol"]).reshape(-1, norb, norb)
    rho = rdm1[0] + rdm1[1]
    mf = 1.0j * np.einsum("gij,ij->g", chol, rho, optimize=True)
    ham_data["mf_shifts"] = mf
    ham_data["h0_prop"] = -ham_data["h0"] - np.sum(mf**2) / 2.0
    v0 = 0.5 * np.einsum("gik,gjk->ij", chol, chol, optimize=True)
    v1 = np.real(1.0j * np.einsum("g,gik->ik", mf, chol, optimize=True))
    h1 = np.asarray(ham_data["h1"])
    if restricted:
        h1_mod = (h1[0] + h1[1]) / 2.0 - v0 - v1
        ham_data["exp_h1"] = scipy.linalg.expm(-dt * h1_mod / 2.0)
    else:
        ham_data["exp_h1"] = np.stack(
            [
                scipy.linalg.expm(-dt * (h1[0] - v0 - v1) / 2.0),
                scipy.linalg.expm(-dt * (h1[1] - v0 - v1) / 2.0),
            ]
        )
    return ham_data


# ----------------------------------------------------------------------------------------
# Propagator  (propagation.py:67-165, 201-290, 331-400)
# ----------------------------------------------------------------------------------------


def apply_trotprop_det(exp_h1: np.ndarray, vhs: np.ndarray, walkers: np.ndarray, n_exp_terms: int):
    """Batched W <- e^{h1/2} (W + sum_{m=1}^{n_exp_terms-1} V^m W / m!) with W = e^{h1/2} W
    first (propagation.py:67-92). vhs [nw,norb,norb], walkers [nw,norb,k]."""
    w = exp_h1 @ walkers
    carry = w
    terms = []
    for _ in range(1, n_exp_terms):
        carry = vhs @ carry
        terms.append(carry)
    acc = np.zeros_like(w)
    for m, t in enumerate(terms):
        acc = acc + t / math.factorial(m + 1)
    w = w + acc
    return exp_h1 @ w


def make_vhs(shifted_fields: np.ndarray, chol: np.ndarray, dt: float, norb: int) -> np.ndarray:
    """vhs = i sqrt(dt) fields . chol, reshaped [nw, norb, norb] (propagation.py:265-271)."""
    return (1.0j * math.sqrt(dt) * (shifted_fields @ chol.reshape(chol.shape[0], -1))).reshape(
        -1, norb, norb
    )


def apply_trotprop(ham_data, walkers, shifted_fields, dt, norb, n_exp_terms):
    vhs = make_vhs(shifted_fields, np.asarray(ham_data["chol"]), dt, norb)
    if isinstance(walkers, list):
        e = ham_data["exp_h1"]
        return [
            apply_trotprop_det(e[0], vhs, walkers[0], n_exp_terms),
            apply_trotprop_det(e[1], vhs, walkers[1], n_exp_terms),
        ]
    return apply_trotprop_det(ham_data["exp_h1"], vhs, walkers, n_exp_terms)


@dataclass
class Propagator:
    dt: float = 0.01
    n_walkers: int = 50
    n_exp_terms: int = 6

    def propagate(self, trial: Trial, ham_data: dict, prop_data: dict, fields: np.ndarray, mo):
        """One phaseless step (propagation.py:100-165). Mutates and returns prop_data."""
        dt = self.dt
        sdt = math.sqrt(dt)
        mf = ham_data["mf_shifts"]
        force_bias = trial.force_bias(prop_data["walkers"], ham_data, mo)
        field_shifts = -sdt * (1.0j * force_bias - mf)
        shifted_fields = fields - field_shifts
        shift_term = np.sum(shifted_fields * mf, axis=1)
        fb_term = np.sum(fields * field_shifts - field_shifts * field_shifts / 2.0, axis=1)
        prop_data["walkers"] = apply_trotprop(
            ham_data, prop_data["walkers"], shifted_fields, dt, trial.norb, self.n_exp_terms
        )
        overlaps_new = trial.overlap(prop_data["walkers"], mo)
        ratio = overlaps_new / prop_data["overlaps"]
        with np.errstate(all="ignore"):
            imp_fun = (
                np.exp(
                    -sdt * shift_term
                    + fb_term
                    + dt * (prop_data["pop_control_ene_shift"] + ham_data["h0_prop"])
                )
                * ratio
            )
            theta = np.angle(np.exp(-sdt * shift_term) * ratio)
            imp = np.abs(imp_fun) * np.cos(theta)
        imp = np.where(np.isnan(imp), 0.0, imp)
        imp = np.where(imp < 1.0e-3, 0.0, imp)
        imp = np.where(imp > 100.0, 0.0, imp)
        w = imp * prop_data["weights"]
        w = np.where(w > 100, 0.0, w)
        prop_data["weights"] = w
        prop_data["pop_control_ene_shift"] = prop_data["e_estimate"] - 0.1 * np.log(
            np.sum(w) / self.n_walkers
        ) / dt
        prop_data["overlaps"] = overlaps_new
        return prop_data

    def propagate_free(self, trial: Trial, ham_data: dict, prop_data: dict, fields: np.ndarray, mo,
                       ene0: float = 0.0):
        """One free-projection step, unrestricted walkers (propagation.py:436-462, intermediates
        464-490): no force bias; shift_term_s = sum_g x_g mf_g / (2 n_s); each slab times
        exp(-sqrt(dt) shift_term_s) exp(dt (h0_prop + ene0) / (2 n_s)); QR of both slabs with
        norms *= prod(diag R_up) prod(diag R_dn); overlaps = overlap(walkers) * norms;
        normed_overlaps = overlap of the walkers QR-ed once more."""
        dt, sdt = self.dt, math.sqrt(self.dt)
        nel = trial.nelec
        mf = ham_data["mf_shifts"]
        s = fields @ mf  # [nw]
        h0p = ham_data["h0_prop"] + ene0
        consts = [np.exp(-sdt * s / (2.0 * nel[i])) * np.exp(dt * h0p / (2.0 * nel[i])) for i in range(2)]
        w = apply_trotprop(ham_data, prop_data["walkers"], fields.astype(np.complex128), dt, trial.norb,
                           self.n_exp_terms)
        w = [consts[0][:, None, None] * w[0], consts[1][:, None, None] * w[1]]
        qs, norms = [], np.ones(fields.shape[0], dtype=np.complex128)
        for x in w:
            q, r = np.linalg.qr(x)
            qs.append(q)
            norms = norms * np.prod(np.diagonal(r, axis1=1, axis2=2), axis=1)
        prop_data["walkers"] = qs
        prop_data["norms"] = prop_data["norms"] * norms
        prop_data["overlaps"] = trial.overlap(qs, mo) * prop_data["norms"]
        prop_data["normed_overlaps"] = trial.overlap([np.linalg.qr(x)[0] for x in qs], mo)
        return prop_data

    def orthonormalize_walkers(self, prop_data: dict) -> dict:
        """Q of the reduced QR of each walker (propagation.py:251-253, 422-424 ->
        linalg_utils.py:51-65). LAPACK Householder convention, as jnp.linalg.qr."""
        w = prop_data["walkers"]
        if isinstance(w, list):
            prop_data["walkers"] = [np.linalg.qr(w[0])[0], np.linalg.qr(w[1])[0]]
        else:
            prop_data["walkers"] = np.linalg.qr(w)[0]
        return prop_data

    def stochastic_reconfiguration(self, prop_data: dict, zeta: float) -> dict:
        """Comb resampling (sr.py:24-47): z = W (i + zeta)/nw, idx = searchsorted(cumsum|w|, z)
        (left side), walkers gathered, weights set to the mean."""
        weights = prop_data["weights"]
        nw = weights.shape[0]
        cw = np.cumsum(np.abs(weights))
        tw = cw[-1]
        z = tw * (np.arange(nw) + zeta) / nw
        idx = np.searchsorted(cw, z)
        idx = np.minimum(idx, nw - 1)  # JAX clamps out-of-range gathers
        w = prop_data["walkers"]
        if isinstance(w, list):
            prop_data["walkers"] = [w[0][idx], w[1][idx]]
        else:
            prop_data["walkers"] = w[idx]
        prop_data["weights"] = np.ones(nw) * (tw / nw)
        prop_data["sr_indices"] = idx
        return prop_data


# ----------------------------------------------------------------------------------------
# CPMC for the Hubbard model with on-site U (propagation.py:515-657, slow form 660-773;
# uhf_cpmc trial wavefunctions.py:848-955)
# ----------------------------------------------------------------------------------------


def cpmc_full_green(walkers, mo):
    """[nw, 2, norb, norb]: G_s = (W_s (C_s^T W_s)^-1 C_s^T)^T (wavefunctions.py:894-914)."""
    out = []
    for w, c in zip(walkers, mo):
        a = w @ np.linalg.inv(np.einsum("pi,wpk->wik", c, w))
        out.append(np.transpose(a @ c.T, (0, 2, 1)))
    return np.stack(out, axis=1)


def cpmc_overlap(walkers, mo):
    return np.linalg.det(np.einsum("pi,wpk->wik", mo[0], walkers[0])) * \
        np.linalg.det(np.einsum("pi,wpk->wik", mo[1], walkers[1]))


def cpmc_hs_constant(dt: float, u: float) -> np.ndarray:
    """[[up, dn] for field 0, [up, dn] for field 1] (propagation.py:532-536)."""
    gamma = np.arccosh(np.exp(dt * u / 2))
    const = np.exp(-dt * u / 2)
    return const * np.array([[np.exp(gamma), np.exp(-gamma)], [np.exp(-gamma), np.exp(gamma)]])


def cpmc_init(walkers, mo, weights=None):
    """Real walkers and overlaps, full Green's functions (propagation.py:518-537)."""
    w = [np.real(walkers[0]).copy(), np.real(walkers[1]).copy()]
    nw = w[0].shape[0]
    return {"walkers": w, "overlaps": np.real(cpmc_overlap(w, mo)),
            "weights": np.ones(nw) if weights is None else weights.copy(),
            "greens": cpmc_full_green(w, mo)}


def _cpmc_one_body(exp_h1, pd, mo):
    """propagation.py:539-563."""
    pd["walkers"] = [np.einsum("ij,wjk->wik", exp_h1[0], pd["walkers"][0]),
                     np.einsum("ij,wjk->wik", exp_h1[1], pd["walkers"][1])]
    ov = cpmc_overlap(pd["walkers"], mo)
    pd["weights"] = pd["weights"] * np.real(ov / pd["overlaps"])
    pd["weights"] = np.where(pd["weights"] < 1.0e-8, 0.0, pd["weights"])
    pd["overlaps"] = ov
    pd["greens"] = cpmc_full_green(pd["walkers"], mo)
    return pd


def cpmc_propagate(exp_h1, dt: float, u: float, pd: dict, gaussian, mo, e_estimate: float,
                   pop_control_ene_shift: float, n_walkers: int, slow: bool = False):
    """One CPMC step (propagation.py:565-657): one-body half step, for every site x a discrete
    Hubbard-Stratonovich field chosen with probabilities from the overlap ratios (uniforms
    (erf(g / sqrt 2) + 1) / 2 of the given Gaussians [nw, norb]), the rank-one updates of the
    Green's functions, one-body half step, weights * exp(dt E_pc), the > 100 clamp and the new
    pop-control shift. slow: the ratios from determinants (propagation.py:660-773) instead of
    the Green's function. Returns (pd, new pop_control_ene_shift)."""
    import scipy.special
    hs = cpmc_hs_constant(dt, u)
    norb = pd["walkers"][0].shape[1]
    pd = _cpmc_one_body(exp_h1, pd, mo)
    uni = (scipy.special.erf(gaussian / 2 ** 0.5) + 1) / 2
    for x in range(norb):
        if slow:
            rat = []
            cand = []
            for f in range(2):
                wu = pd["walkers"][0].copy()
                wd = pd["walkers"][1].copy()
                wu[:, x, :] *= hs[f, 0]
                wd[:, x, :] *= hs[f, 1]
                ov = cpmc_overlap([wu, wd], mo)
                r = np.real(ov / pd["overlaps"]) / 2.0
                rat.append(np.where(r < 1.0e-8, 0.0, r))
                cand.append((wu, wd, ov))
            norm = rat[0] + rat[1]
            p0 = rat[0] / norm
            m = uni[:, x] < p0
            pd["walkers"] = [np.where(m[:, None, None], cand[0][0], cand[1][0]),
                             np.where(m[:, None, None], cand[0][1], cand[1][1])]
            pd["overlaps"] = np.where(m, cand[0][2], cand[1][2])
            pd["weights"] = pd["weights"] * norm
            continue
        g = pd["greens"]
        rats = []
        for f in range(2):
            c = hs[f] - 1
            r = (1 + c[0] * g[:, 0, x, x]) * (1 + c[1] * g[:, 1, x, x])
            rats.append(np.where(r < 1.0e-8, 0.0, r))
        p0, p1 = rats[0] / 2.0, rats[1] / 2.0
        norm = p0 + p1
        p0 = p0 / norm
        m = uni[:, x] < p0
        consts = np.where(m[:, None], hs[0][None, :], hs[1][None, :])  # [nw, 2]
        pd["walkers"][0] = pd["walkers"][0].copy()
        pd["walkers"][1] = pd["walkers"][1].copy()
        pd["walkers"][0][:, x, :] *= consts[:, 0:1]
        pd["walkers"][1][:, x, :] *= consts[:, 1:2]
        ratios = np.where(m, rats[0], rats[1])
        uc = consts - 1
        # wavefunctions.py:916-945 with update indices (0, x), (1, x): different spins, so
        # g_ij = g_ji = 0 and the second update sees the first spin block unchanged
        gn = g.copy()
        sg_i = g[:, 0, x, :].copy()
        sg_i[:, x] -= 1
        sg_j = g[:, 1, x, :].copy()
        sg_j[:, x] -= 1
        g_ii, g_jj = g[:, 0, x, x], g[:, 1, x, x]
        fac_i = uc[:, 0] / ratios
        gn[:, 0] += fac_i[:, None, None] * np.einsum(
            "wi,wj->wij", g[:, 0, :, x], uc[:, 1:2] * (-g_jj[:, None] * sg_i) - sg_i)
        fac_j = uc[:, 1] / ratios
        gn[:, 1] += fac_j[:, None, None] * np.einsum(
            "wi,wj->wij", g[:, 1, :, x], uc[:, 0:1] * (-g_ii[:, None] * sg_j) - sg_j)
        pd["greens"] = gn
        pd["overlaps"] = ratios * pd["overlaps"]
        pd["weights"] = pd["weights"] * norm
    pd = _cpmc_one_body(exp_h1, pd, mo)
    pd["weights"] = pd["weights"] * np.exp(dt * pop_control_ene_shift)
    pd["weights"] = np.where(pd["weights"] > 100.0, 0.0, pd["weights"])
    pcs = e_estimate - 0.1 * np.log(np.sum(pd["weights"]) / n_walkers) / dt
    return pd, pcs


def _cpmc_pair_update(pd: dict, hs_pair, si: int, i: int, sj: int, j: int, uni, mo, slow: bool,
                      literal: bool = False):
    """One two-entry discrete-field update at (spin si, site i), (spin sj, site j) with the
    constants hs_pair [field][entry] (propagation.py:949-1220). Fast: the ratio and the
    two-step Green's-function update of uhf_cpmc (wavefunctions.py:873-945) with both steps
    built from the Green's function before the update. (The reference's code reads column j
    of the once-updated array in its second step; for two entries of one spin that is not
    the exact rank-two update, and its own test asserts agreement with the slow form, which
    the exact update gives.) literal=True restates that code as written instead
    (wavefunctions.py:916-945: the second add's outer-product column green[spin_j, :, j]
    taken after the first add), to measure how far it is from the slow form. Slow:
    determinant ratios (propagation.py:1263-1591)."""
    w = pd["walkers"]
    if slow:
        cand, rat = [], []
        for f in range(2):
            wn = [w[0].copy(), w[1].copy()]
            wn[si][:, i, :] *= hs_pair[f, 0]
            wn[sj][:, j, :] *= hs_pair[f, 1]
            ov = cpmc_overlap(wn, mo)
            r = np.real(ov / pd["overlaps"]) / 2.0
            rat.append(np.where(r < 1.0e-8, 0.0, r))
            cand.append((wn, ov))
        norm = rat[0] + rat[1]
        m = uni < rat[0] / norm
        pd["walkers"] = [np.where(m[:, None, None], cand[0][0][s], cand[1][0][s]) for s in range(2)]
        pd["overlaps"] = np.where(m, cand[0][1], cand[1][1])
        pd["weights"] = pd["weights"] * norm
        return pd
    g = pd["greens"]
    same = 1.0 if si == sj else 0.0
    rats = []
    for f in range(2):
        c = hs_pair[f] - 1
        r = (1 + c[0] * g[:, si, i, i]) * (1 + c[1] * g[:, sj, j, j]) \
            - same * c[0] * c[1] * g[:, si, i, j] * g[:, sj, j, i]
        rats.append(np.where(r < 1.0e-8, 0.0, r))
    p0, p1 = rats[0] / 2.0, rats[1] / 2.0
    norm = p0 + p1
    m = uni < p0 / norm
    consts = np.where(m[:, None], hs_pair[0][None, :], hs_pair[1][None, :])
    wn = [w[0].copy(), w[1].copy()]
    wn[si][:, i, :] *= consts[:, 0:1]
    wn[sj][:, j, :] *= consts[:, 1:2]
    ratios = np.where(m, rats[0], rats[1])
    uc = consts - 1
    sg_i = g[:, si, i, :].copy()
    sg_i[:, i] -= 1
    sg_j = g[:, sj, j, :].copy()
    sg_j[:, j] -= 1
    g_ii, g_jj = g[:, si, i, i], g[:, sj, j, j]
    g_ij, g_ji = same * g[:, si, i, j], same * g[:, sj, j, i]
    gn = g.copy()
    gn[:, si] += (uc[:, 0] / ratios)[:, None, None] * np.einsum(
        "wa,wb->wab", g[:, si, :, i], uc[:, 1:2] * (g_ij[:, None] * sg_j - g_jj[:, None] * sg_i) - sg_i)
    col_j = gn[:, sj, :, j].copy() if literal else g[:, sj, :, j]
    gn[:, sj] += (uc[:, 1] / ratios)[:, None, None] * np.einsum(
        "wa,wb->wab", col_j, uc[:, 0:1] * (g_ji[:, None] * sg_i - g_ii[:, None] * sg_j) - sg_j)
    pd["walkers"] = wn
    pd["greens"] = gn
    pd["overlaps"] = ratios * pd["overlaps"]
    pd["weights"] = pd["weights"] * norm
    return pd


def cpmc_nn_propagate(exp_h1, dt: float, u: float, u1: float, neighbors, pd: dict, uniforms, mo,
                      e_estimate: float, pop_control_ene_shift: float, n_walkers: int, slow: bool = False,
                      literal: bool = False):
    """One step of CPMC with on-site U and nearest-neighbour V = u1 (propagator_cpmc_nn,
    propagation.py:889-1230; slow: propagator_cpmc_nn_slow, 1232-1591): one-body half step,
    the on-site sweep (fields from hs(u) on (up, x), (dn, x)), then for every neighbour pair
    (i, j) four two-entry updates with hs(u1) on (up i, up j), (up i, dn j), (dn i, up j),
    (dn i, dn j), one-body half step, weights * exp(dt E_pc), the > 100 clamp and the new
    shift. uniforms [nw, norb + 4 npairs]: column x for site x, then norb + k npairs + p for
    update k of pair p (the reference draws both sets from its key). literal: the fast form's
    Green's-function update as the reference's code writes it (see _cpmc_pair_update).
    Returns (pd, shift)."""
    hs0 = cpmc_hs_constant(dt, u)
    hs1 = cpmc_hs_constant(dt, u1)
    norb = pd["walkers"][0].shape[1]
    npairs = len(neighbors)
    pd = _cpmc_one_body(exp_h1, pd, mo)
    for x in range(norb):
        pd = _cpmc_pair_update(pd, hs0, 0, x, 1, x, uniforms[:, x], mo, slow, literal)
    for p, (i, j) in enumerate(neighbors):
        for k, (si, sj) in enumerate(((0, 0), (0, 1), (1, 0), (1, 1))):
            pd = _cpmc_pair_update(pd, hs1, si, i, sj, j, uniforms[:, norb + k * npairs + p], mo, slow, literal)
    pd = _cpmc_one_body(exp_h1, pd, mo)
    pd["weights"] = pd["weights"] * np.exp(dt * pop_control_ene_shift)
    pd["weights"] = np.where(pd["weights"] > 100.0, 0.0, pd["weights"])
    pcs = e_estimate - 0.1 * np.log(np.sum(pd["weights"]) / n_walkers) / dt
    return pd, pcs


def cpmc_continuous_propagate(exp_h1, dt: float, hs: float, pd: dict, gaussian, mo, e_estimate: float,
                              pop_control_ene_shift: float, n_walkers: int):
    """One step of the continuous-field CPMC variant (propagation.py:1595-1675; the force bias
    and fb_term there are multiplied by zero). Returns (pd, new pop_control_ene_shift)."""
    w = [np.einsum("ij,wjk->wik", exp_h1[0], pd["walkers"][0]),
         np.einsum("ij,wjk->wik", exp_h1[1], pd["walkers"][1])]
    w = [np.exp(gaussian * hs)[:, :, None] * w[0], np.exp(-gaussian * hs)[:, :, None] * w[1]]
    w = [np.einsum("ij,wjk->wik", exp_h1[0], w[0]), np.einsum("ij,wjk->wik", exp_h1[1], w[1])]
    ov = cpmc_overlap(w, mo)
    imp = np.exp(dt * pop_control_ene_shift) * ov / pd["overlaps"]
    wt = pd["weights"] * np.real(imp)
    wt = np.where(wt < 1.0e-8, 0.0, wt)
    wt = np.where(wt > 100.0, 0.0, wt)
    pd = {"walkers": w, "overlaps": ov, "weights": wt, "greens": pd.get("greens")}
    return pd, e_estimate - 0.1 * np.log(np.sum(wt) / n_walkers) / dt


def init_prop_data(prop: Propagator, trial: Trial, ham_data: dict, mo, walkers) -> dict:
    """weights 1, e_estimate = mean real energy, overlaps (propagation.py:210-232, 333-357)."""
    pd = {"weights": np.ones(prop.n_walkers), "walkers": walkers}
    e = np.real(trial.energy(walkers, ham_data, mo))
    pd["e_estimate"] = np.sum(e) / prop.n_walkers
    pd["pop_control_ene_shift"] = pd["e_estimate"]
    pd["overlaps"] = trial.overlap(walkers, mo)
    return pd


# ----------------------------------------------------------------------------------------
# Sampler  (sampling.py:22-144, 319-341) and driver bookkeeping (driver.py:207-308)
# ----------------------------------------------------------------------------------------


@dataclass
class Sampler:
    n_prop_steps: int = 50
    n_ene_blocks: int = 50
    n_sr_blocks: int = 1
    n_blocks: int = 50

    def block_scan(self, prop, trial, ham_data, prop_data, mo, fields):
        """fields [n_prop_steps, nw, G] (sampling.py:50-92)."""
        for s in range(self.n_prop_steps):
            prop_data = prop.propagate(trial, ham_data, prop_data, fields[s], mo)
        prop_data["n_killed_walkers"] += prop_data["weights"].size - np.count_nonzero(
            prop_data["weights"]
        )
        prop_data = prop.orthonormalize_walkers(prop_data)
        prop_data["overlaps"] = trial.overlap(prop_data["walkers"], mo)
        e = np.real(trial.energy(prop_data["walkers"], ham_data, mo))
        e = np.where(np.abs(e - prop_data["e_estimate"]) > np.sqrt(2.0 / prop.dt), prop_data["e_estimate"], e)
        bw = np.sum(prop_data["weights"])
        be = np.sum(e * prop_data["weights"]) / bw
        prop_data["pop_control_ene_shift"] = 0.9 * prop_data["pop_control_ene_shift"] + 0.1 * be
        return prop_data, be, bw

    def block_scan_free(self, prop, trial, ham_data, prop_data, mo, fields, ene0=0.0):
        """fields [n_prop_steps, nw, G] (sampling.py:95-124): free steps, then the complex
        local energies and block_energy = sum E O / sum O, block_weight = sum O."""
        for st in range(self.n_prop_steps):
            prop_data = prop.propagate_free(trial, ham_data, prop_data, fields[st], mo, ene0)
        e = trial.energy(prop_data["walkers"], ham_data, mo)
        o = prop_data["overlaps"]
        return prop_data, np.sum(e * o) / np.sum(o), np.sum(o)

    def propagate_free(self, prop, trial, ham_data, prop_data, mo, fields, ene0=0.0):
        """n_blocks free-projection blocks (sampling.py:344-360); fields
        [n_blocks, n_prop_steps, nw, G]. Returns (prop_data, block_energy, block_weight)."""
        prop_data["overlaps"] = trial.overlap(prop_data["walkers"], mo)
        be, bw = [], []
        for b in range(fields.shape[0]):
            prop_data, e, wt = self.block_scan_free(prop, trial, ham_data, prop_data, mo, fields[b], ene0)
            be.append(e)
            bw.append(wt)
        return prop_data, np.array(be), np.array(bw)

    def propagate_phaseless(self, prop, trial, ham_data, prop_data, mo, fields, zetas, do_sr=True):
        """fields [n_sr_blocks, n_ene_blocks, n_prop_steps, nw, G]; zetas [n_sr_blocks]
        (sampling.py:126-144, 319-341). do_sr=False: the no-SR block of
        propagate_phaseless_ad_nosr (sampling.py:287-317; n_sr_blocks 1). Returns (energy,
        prop_data, block_e, block_w)."""
        prop_data["overlaps"] = trial.overlap(prop_data["walkers"], mo)
        prop_data["n_killed_walkers"] = 0
        prop_data["pop_control_ene_shift"] = prop_data["e_estimate"]
        be_all, bw_all = [], []
        for s in range(self.n_sr_blocks):
            for b in range(self.n_ene_blocks):
                prop_data, be, bw = self.block_scan(prop, trial, ham_data, prop_data, mo, fields[s, b])
                be_all.append(be)
                bw_all.append(bw)
            if not do_sr:
                continue
            prop_data = prop.stochastic_reconfiguration(prop_data, zetas[s])
            prop_data["overlaps"] = trial.overlap(prop_data["walkers"], mo)
        prop_data["n_killed_walkers"] /= self.n_sr_blocks * self.n_ene_blocks * prop.n_walkers
        be_all, bw_all = np.array(be_all), np.array(bw_all)
        return np.sum(be_all * bw_all) / np.sum(bw_all), prop_data, be_all, bw_all


def run_blocks(
    sampler: Sampler,
    prop: Propagator,
    trial: Trial,
    ham_data: dict,
    prop_data: dict,
    mo,
    draw_fields: Callable[[int], np.ndarray],
    draw_zetas: Callable[[int], np.ndarray],
    n_blocks: int,
):
    """Single-rank driver loop without AD (driver.py:207-308): per block
    propagate_phaseless, record (energy, sum of weights), QR, global SR (one rank: the same
    comb), e_estimate <- 0.9 e_estimate + 0.1 E_block.

    draw_fields(n) -> fields for block n, shape [n_sr, n_ene, n_prop, nw, G];
    draw_zetas(n) -> [n_sr + 1] uniforms (n_sr local SRs, then the driver's global SR).
    """
    energies, weights = [], []
    for n in range(n_blocks):
        f = draw_fields(n)
        z = draw_zetas(n)
        e, prop_data, _, _ = sampler.propagate_phaseless(prop, trial, ham_data, prop_data, mo, f, z[:-1])
        energies.append(e)
        weights.append(np.sum(prop_data["weights"]))
        prop_data = prop.orthonormalize_walkers(prop_data)
        prop_data = prop.stochastic_reconfiguration(prop_data, z[-1])
        prop_data["e_estimate"] = 0.9 * prop_data["e_estimate"] + 0.1 * e
    return np.array(energies), np.array(weights), prop_data


# ---------------------------------------------------------------------------------------
# correlated sampling (ad_afqmc/corr_sample/corr_sample.py)
# ---------------------------------------------------------------------------------------

def en_samples(prop, trial, ham_data, prop_data, mo) -> np.ndarray:
    """Real local energies clamped to e_estimate beyond sqrt(2/dt) (corr_sample.py:482-491)."""
    e = np.real(trial.energy(prop_data["walkers"], ham_data, mo))
    return np.where(np.abs(e - prop_data["e_estimate"]) > np.sqrt(2.0 / prop.dt), prop_data["e_estimate"], e)


def corr_otler_rm(w1: np.ndarray, w2: np.ndarray, z_thresh: float = 5.0):
    """Weight-outlier removal of a correlated pair (corr_sample.py:557-594): population-std
    z-scores of each system, the larger of the two per walker (jnp.where semantics), weights
    of walkers above z_thresh set to 0 in both systems."""
    with np.errstate(divide="ignore", invalid="ignore"):
        z1 = np.abs(w1 - np.mean(w1)) / np.std(w1)
        z2 = np.abs(w2 - np.mean(w2)) / np.std(w2)
    z = np.where(z1 > z2, z1, z2)
    return np.where(z > z_thresh, 0.0, w1), np.where(z > z_thresh, 0.0, w2)


def cs_steps_scan(sampler: "Sampler", sys1: tuple, sys2: tuple, fields: np.ndarray):
    """Correlated blocks of two systems on shared fields (corr_sample.py:596-694).
    sys = (prop, trial, ham_data, prop_data, mo); fields [steps, n_prop_steps, nw, G].
    Each step: field_block_scan of both systems (Sampler.block_scan: n_prop_steps steps, QR,
    overlaps, block energy, pop-control update, no SR), outlier removal, then the sums
    (sum E w, sum w) of both. Returns (prop_data1, prop_data2, loc_en1, loc_w1, loc_en2, loc_w2)."""
    p1, t1, h1, pd1, mo1 = sys1
    p2, t2, h2, pd2, mo2 = sys2
    for pd in (pd1, pd2):  # corr_sample.init_prop sets it (corr_sample.py:472)
        pd.setdefault("n_killed_walkers", 0)
    out = []
    for f in fields:
        pd1, _, _ = sampler.block_scan(p1, t1, h1, pd1, mo1, f)
        pd2, _, _ = sampler.block_scan(p2, t2, h2, pd2, mo2, f)
        pd1["weights"], pd2["weights"] = corr_otler_rm(pd1["weights"], pd2["weights"])
        e1 = en_samples(p1, t1, h1, pd1, mo1)
        e2 = en_samples(p2, t2, h2, pd2, mo2)
        out.append((np.sum(e1 * pd1["weights"]), np.sum(pd1["weights"]),
                    np.sum(e2 * pd2["weights"]), np.sum(pd2["weights"])))
    out = np.array(out)
    return pd1, pd2, out[:, 0], out[:, 1], out[:, 2], out[:, 3]


def _eigh_fixed_sign(fock: np.ndarray):
    """eigh with each eigenvector's largest-magnitude component made non-negative
    (wavefunctions.py:582-586, 788-792): the first index of the largest |component| decides."""
    e, v = np.linalg.eigh(fock)
    idx = np.argmax(np.abs(v), axis=0)
    sign = np.where(v[idx, np.arange(v.shape[1])] < 0, -1.0, 1.0)
    return e, v * sign[None, :]


def rhf_optimize(h1, chol, mo, nelec: int, n_iter: int = 30) -> np.ndarray:
    """RHF self-consistent-field iterations of rhf.optimize (wavefunctions.py:566-600):
    from dm = 2 C C^T, n_iter times fock = h1 + J - K/2, eigh, occupy the lowest nelec; the
    trial becomes the lowest nelec eigenvectors of the last Fock matrix. h1 [2, n, n] (the
    spin average is used, symmetrised), chol [G, n, n]."""
    h = (np.asarray(h1)[0] + np.asarray(h1)[1]) / 2.0
    h = (h + h.T) / 2.0
    dm = 2.0 * mo @ mo.T
    v = None
    for _ in range(n_iter):
        f = np.einsum("gij,ik->gjk", chol, dm)
        c = np.einsum("gii->g", f)
        vj = np.einsum("g,gij->ij", c, chol)
        vk = np.einsum("glj,gjk->lk", f, chol)
        e, v = _eigh_fixed_sign(h + vj - 0.5 * vk)
        occ = v[:, np.argsort(e)[:nelec]]
        dm = 2.0 * occ @ occ.T
    return v[:, :nelec]


def uhf_optimize(h1, chol, mo, nelec, n_iter: int = 30):
    """UHF iterations of uhf.optimize (wavefunctions.py:750-813): fock_s = h1_s + J_up +
    J_dn - K_s from dm0 = C_s C_s^T (the trial's own rdm1)."""
    h = [(np.asarray(h1)[s] + np.asarray(h1)[s].T) / 2.0 for s in range(2)]
    dm = [mo[0] @ mo[0].T, mo[1] @ mo[1].T]
    vs = [None, None]
    for _ in range(n_iter):
        f = [np.einsum("gij,ik->gjk", chol, dm[s]) for s in range(2)]
        vj = sum(np.einsum("g,gij->ij", np.einsum("gii->g", f[s]), chol) for s in range(2))
        new = []
        for s in range(2):
            vk = np.einsum("glj,gjk->lk", f[s], chol)
            e, v = _eigh_fixed_sign(h[s] + vj - vk)
            occ = v[:, np.argsort(e)[:nelec[s]]]
            new.append(occ @ occ.T)
            vs[s] = v
        dm = new
    return [vs[0][:, :nelec[0]], vs[1][:, :nelec[1]]]


def phaseless_derivative_fd(sampler: "Sampler", prop: "Propagator", trial: "Trial", ham_data: dict,
                            direction: np.ndarray, rdm1: np.ndarray, mo, prop_data: dict,
                            fields: np.ndarray, zetas, restricted: bool, h: float = 1e-3,
                            do_sr: bool = True, orbital_rotation: bool = False, n_opt_iter: int = 30):
    """d/d lambda of the blocked energy and of each block's (energy, weight) for
    h1 + lambda * direction (direction [2, norb, norb]) with prop_data, fields and SR
    uniforms held fixed: the quantity that driver.py:207-215 takes with jax.jvp of
    sampling.py:266-285 (norot) or 287-317 (nosr_norot); orbital_rotation: of
    sampling.py:173-196 / 221-254, the trial re-optimised at every lambda (rdm1, and so the
    mean-field shifts, stay those given, as the driver fixes wave_data["rdm1"]). ham_data is
    the raw {h0, h1, chol}; intermediates are rebuilt at each lambda. Central differences at
    h and h/2, Richardson-extrapolated (error O(h^4)). Returns (energy, d energy, block_e,
    d block_e, block_w, d block_w) at lambda = 0."""
    import copy

    def run(lam):
        hd = {"h0": ham_data["h0"], "h1": np.asarray(ham_data["h1"]) + lam * direction,
              "chol": ham_data["chol"]}
        m = mo
        if orbital_rotation:
            chol3 = np.asarray(ham_data["chol"]).reshape(-1, trial.norb, trial.norb)
            m = rhf_optimize(hd["h1"], chol3, mo, trial.nelec[0], n_opt_iter) if trial.kind == "rhf" else \
                uhf_optimize(hd["h1"], chol3, mo, trial.nelec, n_opt_iter)
        hd = trial.build_measurement_intermediates(hd, m)
        hd = build_propagation_intermediates(hd, rdm1, trial.norb, trial.nelec, prop.dt, restricted)
        pd = copy.deepcopy(prop_data)
        if orbital_rotation:  # _ad_block recomputes the overlaps with the new trial
            pd["overlaps"] = trial.overlap(pd["walkers"], m)
        e, _, be, bw = sampler.propagate_phaseless(prop, trial, hd, pd, m, fields, zetas, do_sr=do_sr)
        return np.concatenate([[e], be, bw])

    v0 = run(0.0)
    d1 = (run(h) - run(-h)) / (2 * h)
    d2 = (run(h / 2) - run(-h / 2)) / h
    d = (4 * d2 - d1) / 3
    nb = (len(v0) - 1) // 2
    return v0[0], d[0], v0[1:1 + nb], d[1:1 + nb], v0[1 + nb:], d[1 + nb:]


def phaseless_chol_derivative_fd(sampler: "Sampler", prop: "Propagator", trial: "Trial", ham_data: dict,
                                 chol_of: Callable[[float], np.ndarray], theta: float, rdm1: np.ndarray, mo,
                                 prop_data: dict, fields: np.ndarray, zetas, restricted: bool, h: float = 1e-3,
                                 do_sr: bool = True):
    """d/d theta of the blocked energy for Cholesky vectors chol_of(theta) [nchol, norb*norb]
    (the Hubbard model's sqrt(U) n_i with theta = U), the trial, prop_data, fields and SR
    uniforms held fixed and every intermediate rebuilt at each theta (the quantity the GPU's
    Cholesky vjp maps to d/d theta). Central differences at h and h/2, Richardson-extrapolated.
    Returns (energy, d energy)."""
    import copy

    def run(t):
        hd = {"h0": ham_data["h0"], "h1": ham_data["h1"], "chol": chol_of(t)}
        hd = trial.build_measurement_intermediates(hd, mo)
        hd = build_propagation_intermediates(hd, rdm1, trial.norb, trial.nelec, prop.dt, restricted)
        e, _, _, _ = sampler.propagate_phaseless(prop, trial, hd, copy.deepcopy(prop_data), mo, fields, zetas,
                                                 do_sr=do_sr)
        return e

    e0 = run(theta)
    d1 = (run(theta + h) - run(theta - h)) / (2 * h)
    d2 = (run(theta + h / 2) - run(theta - h / 2)) / h
    return e0, (4 * d2 - d1) / 3


def blocking_analysis(weights: np.ndarray, energies: np.ndarray, neql: int = 0):
    """Weighted mean and plateau error of blocked samples (stat_utils.py:8-52), computed in
    float64 throughout (the reference's blocked arrays are float32)."""
    weights = np.asarray(weights, dtype=np.float64)[neql:]
    energies = np.asarray(energies, dtype=np.float64)[neql:]
    n = weights.shape[0]
    we = weights * energies
    mean = we.sum() / weights.sum()
    prev, plateau = 0.0, None
    for i in range(1, n + 1):
        if not i < n / 2.0:
            break
        nb = n // i
        bw = np.array([weights[j * i:(j + 1) * i].sum() for j in range(nb)])
        be = np.array([we[j * i:(j + 1) * i].sum() for j in range(nb)]) / bw
        v1, v2 = bw.sum(), (bw**2).sum()
        m = (bw * be).sum() / v1
        err = ((bw * (be - m) ** 2).sum() / (v1 - v2 / v1) / (nb - 1)) ** 0.5
        if err <= 1.05 * prev and plateau is None:
            plateau = max(err, prev)
        prev = err
    return mean, plateau
