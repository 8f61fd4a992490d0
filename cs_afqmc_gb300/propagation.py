"""Phaseless-AFQMC propagators with the reference's API, evaluated by GB300 kernels.

Mirrors ad_afqmc/propagation.py: ``propagator_restricted`` (201-328) and
``propagator_unrestricted`` (331-512) with ``init_prop_data``, ``propagate``,
``orthonormalize_walkers``, ``stochastic_reconfiguration_local`` /
``stochastic_reconfiguration_global`` and ``_build_propagation_intermediates``.

``prop_data`` is a :class:`PropData` dict. Walkers, weights and overlaps are CUDA tensors;
the scalars ``e_estimate``, ``pop_control_ene_shift`` and ``n_killed_walkers`` live in a
device array and read back as 0-d CUDA tensors, so nothing synchronises with the host.
``prop_data["key"]`` is an :class:`RngKey` (seed and Philox offsets), standing in for the
JAX PRNG key.

``precision`` selects the walker dtype: "fp64" -> complex128 walkers and FP64 kernels;
"mixed" -> complex64 walkers and FP16 tensor-core contractions with hi/lo split operands
(FP32 accumulation; FP64 log-determinants, weights and sums).
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Any, List, Optional, Sequence

import numpy as np
import torch

from . import _engine, _lib
from ._engine import as_dev, device, stream_ptr

_SCALAR_KEYS = {"e_estimate": _lib.AFQ_S_E_ESTIMATE,
                "pop_control_ene_shift": _lib.AFQ_S_POP_CONTROL_SHIFT,
                "n_killed_walkers": _lib.AFQ_S_N_KILLED}


class RngKey:
    """Counter-based key: draws are a pure function of (seed, offset)."""

    def __init__(self, seed: int, offset: int = 0):
        self.seed = int(seed) & ((1 << 64) - 1)
        self.offset = int(offset)

    def take(self, n: int) -> int:
        """Reserve n draws and return their starting offset (kept even)."""
        o = self.offset
        self.offset += n + (n & 1)
        return o

    def __repr__(self):
        return f"RngKey(seed={self.seed}, offset={self.offset})"


class PropData(dict):
    """prop_data dict whose scalar entries are views of a device array."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        if "_scalars" not in self:
            dict.__setitem__(self, "_scalars",
                             torch.zeros(_lib.AFQ_NSCALARS, dtype=torch.float64, device=device()))

    def __getitem__(self, k):
        if k in _SCALAR_KEYS:
            return dict.__getitem__(self, "_scalars")[_SCALAR_KEYS[k]]
        return dict.__getitem__(self, k)

    def __setitem__(self, k, v):
        if k in _SCALAR_KEYS:
            s = dict.__getitem__(self, "_scalars")
            if isinstance(v, torch.Tensor):
                s[_SCALAR_KEYS[k]].copy_(v.reshape(()).to(torch.float64).real
                                         if v.is_complex() else v.reshape(()))
            else:
                s[_SCALAR_KEYS[k]] = float(np.real(v))
            return
        dict.__setitem__(self, k, v)

    def __contains__(self, k):
        return k in _SCALAR_KEYS or dict.__contains__(self, k)

    def state(self, eng: _engine.Engine) -> _lib.WalkerState:
        wu, wd = eng.walkers(self["walkers"])
        w, o = self["weights"], self["overlaps"]
        if w.dtype != torch.float64 or not w.is_contiguous() or w.numel() != eng.nw:
            raise _lib.AfqError("weights must be contiguous float64 [nw]")
        if o.dtype != torch.complex128 or not o.is_contiguous() or o.numel() != eng.nw:
            raise _lib.AfqError("overlaps must be contiguous complex128 [nw]")
        return _lib.WalkerState(walkers_up=wu, walkers_dn=wd, weights=w.data_ptr(),
                                overlaps=o.data_ptr(), scalars=self["_scalars"].data_ptr())


@dataclass
class propagator_restricted:
    """Propagator for walkers with the same alpha and beta dets (propagation.py:201-328)."""

    dt: float = 0.01
    n_walkers: int = 50
    n_exp_terms: int = 6
    n_batch: int = 1
    precision: str = "fp64"
    mixed_config: int = 0  # accuracy options of the mixed path (0 = library default)

    restricted = True

    @property
    def walker_dtype(self) -> torch.dtype:
        return torch.complex128 if self.precision == "fp64" else torch.complex64

    def _engine(self, trial, ham_data, wave_data, walkers) -> _engine.Engine:
        return _engine.engine_for(trial, ham_data, wave_data, walkers, dt=self.dt,
                                  n_exp_terms=self.n_exp_terms, n_batch=self.n_batch,
                                  need_propagation=True, mixed_config=self.mixed_config)

    def _cast_walkers(self, walkers):
        if isinstance(walkers, (list, tuple)):
            return [as_dev(w, self.walker_dtype) for w in walkers]
        return as_dev(walkers, self.walker_dtype)

    # ---- state ----------------------------------------------------------------------
    def init_prop_data(self, trial, wave_data: dict, ham_data: dict,
                       init_walkers=None) -> PropData:
        """weights 1, walkers, e_estimate = mean real energy, overlaps
        (propagation.py:210-232, 333-357)."""
        pd = PropData()
        pd["weights"] = torch.ones(self.n_walkers, dtype=torch.float64, device=device())
        if init_walkers is not None:
            pd["walkers"] = self._cast_walkers(init_walkers)
        else:
            pd["walkers"] = trial.get_init_walkers(wave_data, self.n_walkers,
                                                   restricted=self.restricted,
                                                   dtype=self.walker_dtype)
        e = trial.calc_energy(pd["walkers"], ham_data, wave_data).real
        pd["e_estimate"] = e.sum() / self.n_walkers
        pd["pop_control_ene_shift"] = pd["e_estimate"]
        pd["overlaps"] = trial.calc_overlap(pd["walkers"], wave_data)
        if not self.restricted:
            pd["normed_overlaps"] = pd["overlaps"]
            pd["norms"] = torch.ones(self.n_walkers, dtype=torch.complex128, device=device())
        pd["n_killed_walkers"] = 0.0
        if "exp_h1" in ham_data:
            bind(self, trial, ham_data, wave_data, pd)
        return pd

    # ---- propagation ----------------------------------------------------------------
    def propagate(self, trial, ham_data: dict, prop_data: PropData, fields,
                  wave_data: dict) -> PropData:
        """One phaseless step with auxiliary fields [nw, nchol] (propagation.py:100-165)."""
        eng = self._engine(trial, ham_data, wave_data, prop_data["walkers"])
        f = as_dev(fields)
        if tuple(f.shape) != (eng.nw, eng.nchol):
            raise _lib.AfqError(f"fields must be [{eng.nw}, {eng.nchol}], got {tuple(f.shape)}")
        dict.__setitem__(prop_data, "_engine", eng)
        st = prop_data.state(eng)
        _lib.call("afq_propagate", eng.ctx, ctypes.byref(st), f.data_ptr(), stream_ptr())
        return prop_data

    def propagate_free(self, trial, ham_data: dict, prop_data: PropData, fields,
                       wave_data: dict) -> PropData:
        """Free projection is defined for unrestricted walkers only (propagation.py:166-188)."""
        raise NotImplementedError("Free projection not implemented for this propagator.")

    def orthonormalize_walkers(self, prop_data: PropData, trial=None, ham_data=None,
                               wave_data=None) -> PropData:
        """Q of the reduced QR of every walker (propagation.py:251-253, 422-424)."""
        eng = _any_engine(prop_data, trial, ham_data, wave_data, self)
        st = prop_data.state(eng)
        _lib.call("afq_orthonormalize_walkers", eng.ctx, ctypes.byref(st), stream_ptr())
        return prop_data

    def stochastic_reconfiguration_local(self, prop_data: PropData, trial=None, ham_data=None,
                                         wave_data=None, zeta=None) -> PropData:
        """Comb resampling with a uniform zeta drawn from prop_data["key"] (or given)
        (propagation.py:234-240 -> sr.py:24-47)."""
        eng = _any_engine(prop_data, trial, ham_data, wave_data, self)
        if zeta is None:
            z = torch.empty(1, dtype=torch.float64, device=device())
            key: RngKey = prop_data["key"]
            _lib.call("afq_fill_uniform", z.data_ptr(), 1, key.seed, key.take(1), stream_ptr())
        else:
            z = as_dev(zeta).reshape(1)
        st = prop_data.state(eng)
        idx = torch.empty(eng.nw, dtype=torch.int32, device=device())
        _lib.call("afq_stochastic_reconfiguration", eng.ctx, ctypes.byref(st), z.data_ptr(),
                  idx.data_ptr(), stream_ptr())
        dict.__setitem__(prop_data, "sr_indices", idx)
        return prop_data

    def stochastic_reconfiguration_global(self, prop_data: PropData, comm: Any = None,
                                          **kw) -> PropData:
        """One GPU, one rank: the global comb equals the local one (sr.py:66-106 with a
        single rank)."""
        if comm is not None and getattr(comm, "Get_size", lambda: 1)() != 1:
            raise NotImplementedError("multi-rank SR: run independent replicas per GPU")
        return self.stochastic_reconfiguration_local(prop_data, **kw)

    # ---- intermediates --------------------------------------------------------------
    def _mf_v0_v1(self, ham_data: dict, trial, wave_data: dict):
        norb = trial.norb
        rdm1 = trial.get_rdm1(wave_data)
        rho = rdm1[0] + rdm1[1]
        chol = as_dev(ham_data["chol"]).reshape(-1, norb, norb)
        mf = 1.0j * torch.einsum("gij,ij->g", chol, rho).to(torch.complex128)
        v0 = 0.5 * torch.einsum("gik,gjk->ij", chol, chol)
        v1 = torch.real(1.0j * torch.einsum("g,gik->ik", mf, chol.to(torch.complex128)))
        return mf, v0, v1

    def _build_propagation_intermediates(self, ham_data: dict, trial, wave_data: dict) -> dict:
        """mf_shifts, h0_prop, exp_h1 = expm(-dt h1_mod/2) (propagation.py:292-325)."""
        mf, v0, v1 = self._mf_v0_v1(ham_data, trial, wave_data)
        ham_data["mf_shifts"] = mf
        h0 = float(np.real(_engine._scalar(ham_data["h0"])))
        ham_data["h0_prop"] = -h0 - torch.sum(mf * mf).item() / 2.0
        h1 = as_dev(ham_data["h1"])
        ham_data["exp_h1"] = self._exp_h1(h1, v0, v1)
        return ham_data

    def exp_h1_tangent(self, ham_data: dict, trial, wave_data: dict, dh1) -> torch.Tensor:
        """d exp_h1 / d lambda for h1 -> h1 + lambda dh1 (dh1 [2, norb, norb], symmetrised
        per spin as the measurement intermediates symmetrise h1): the Frechet derivative
        of expm at -dt h1_mod/2 in the direction -dt dh1_mod/2. mf_shifts and v0, v1 do
        not depend on h1."""
        _, v0, v1 = self._mf_v0_v1(ham_data, trial, wave_data)
        return self._exp_h1_tangent(as_dev(ham_data["h1"]), v0, v1, as_dev(dh1))

    def exp_h1_cotangent(self, ham_data: dict, trial, wave_data: dict, gexp) -> torch.Tensor:
        """Transpose of exp_h1_tangent: d energy / d h1 per spin [2, norb, norb] (before the
        symmetrisation) from d energy / d exp_h1. The transpose of the Frechet derivative
        L(A, .) of expm is L(A^T, .)."""
        _, v0, v1 = self._mf_v0_v1(ham_data, trial, wave_data)
        return self._exp_h1_cotangent(as_dev(ham_data["h1"]), v0, v1, gexp)

    def _exp_h1(self, h1, v0, v1):
        h1_mod = (h1[0] + h1[1]) / 2.0 - v0 - v1
        return torch.linalg.matrix_exp(-self.dt * h1_mod / 2.0).contiguous()

    def _exp_h1_cotangent(self, h1, v0, v1, gexp):
        h1_mod = (h1[0] + h1[1]) / 2.0 - v0 - v1
        g = -self.dt / 4.0 * expm_frechet((-self.dt * h1_mod / 2.0).T.contiguous(), as_dev(gexp))
        return torch.stack([g, g])

    def _exp_h1_tangent(self, h1, v0, v1, dh1):
        h1_mod = (h1[0] + h1[1]) / 2.0 - v0 - v1
        return expm_frechet(-self.dt * h1_mod / 2.0, -self.dt * (dh1[0] + dh1[1]) / 4.0)

    def __hash__(self) -> int:
        return hash((type(self).__name__, self.dt, self.n_walkers, self.n_exp_terms,
                     self.n_batch, self.precision, self.mixed_config))


@dataclass
class propagator_unrestricted(propagator_restricted):
    """Two-slab walkers, one exp_h1 per spin (propagation.py:331-512)."""

    restricted = False

    def _exp_h1(self, h1, v0, v1):
        return torch.stack([torch.linalg.matrix_exp(-self.dt * (h1[0] - v0 - v1) / 2.0),
                            torch.linalg.matrix_exp(-self.dt * (h1[1] - v0 - v1) / 2.0)]).contiguous()

    def _build_propagation_intermediates(self, ham_data: dict, trial, wave_data: dict) -> dict:
        """Also the free-projection intermediates mf_shifts_fp and h0_prop_fp
        (propagation.py:473-486)."""
        ham_data = super()._build_propagation_intermediates(ham_data, trial, wave_data)
        mf = ham_data["mf_shifts"]
        n_up, n_dn = trial.nelec
        ham_data["mf_shifts_fp"] = torch.stack([mf / n_up / 2.0, mf / n_dn / 2.0])
        h0p = ham_data["h0_prop"] + float(np.real(_engine._scalar(ham_data.get("ene0", 0.0))))
        ham_data["h0_prop_fp"] = [h0p / n_up / 2.0, h0p / n_dn / 2.0]
        return ham_data

    def propagate_free(self, trial, ham_data: dict, prop_data: PropData, fields,
                       wave_data: dict) -> PropData:
        """One free-projection step with unshifted fields [nw, nchol] (propagation.py:436-462):
        updates walkers, prop_data["norms"], ["overlaps"] (overlap * norms) and
        ["normed_overlaps"]. FP64 (complex128) walkers."""
        eng = self._engine(trial, ham_data, wave_data, prop_data["walkers"])
        f = as_dev(fields)
        if tuple(f.shape) != (eng.nw, eng.nchol):
            raise _lib.AfqError(f"fields must be [{eng.nw}, {eng.nchol}], got {tuple(f.shape)}")
        dict.__setitem__(prop_data, "_engine", eng)
        norms, normed = _free_state(prop_data, eng.nw)
        st = prop_data.state(eng)
        ene0 = float(np.real(_engine._scalar(ham_data.get("ene0", 0.0))))
        _lib.call("afq_propagate_free", eng.ctx, ctypes.byref(st), f.data_ptr(), ene0, norms.data_ptr(),
                  normed.data_ptr(), stream_ptr())
        return prop_data

    def _exp_h1_tangent(self, h1, v0, v1, dh1):
        return torch.stack([expm_frechet(-self.dt * (h1[s] - v0 - v1) / 2.0, -self.dt * dh1[s] / 2.0)
                            for s in range(2)]).contiguous()

    def _exp_h1_cotangent(self, h1, v0, v1, gexp):
        return torch.stack([-self.dt / 2.0 * expm_frechet((-self.dt * (h1[s] - v0 - v1) / 2.0).T.contiguous(),
                                                          as_dev(gexp[s])) for s in range(2)])

    def __hash__(self) -> int:
        return super().__hash__()


def _free_state(prop_data: PropData, nw: int):
    """prop_data["norms"] and ["normed_overlaps"] as complex128 device tensors of their own
    (init_prop_data starts normed_overlaps as the overlaps themselves)."""
    out = []
    for key in ("norms", "normed_overlaps"):
        t = prop_data.get(key)
        t = torch.ones(nw, dtype=torch.complex128, device=device()) if t is None else as_dev(t, torch.complex128)
        if key == "normed_overlaps" and t.data_ptr() == prop_data["overlaps"].data_ptr():
            t = t.clone()
        t = t.contiguous()
        dict.__setitem__(prop_data, key, t)
        out.append(t)
    return out


def expm_frechet(a: torch.Tensor, da: torch.Tensor) -> torch.Tensor:
    """Frechet derivative L(a, da) = d/dt expm(a + t da) at t = 0, the upper-right block
    of expm([[a, da], [0, a]]) (Higham, Functions of Matrices, 2008, thm. 3.6)."""
    n = a.shape[0]
    m = torch.zeros(2 * n, 2 * n, dtype=a.dtype, device=a.device)
    m[:n, :n] = a
    m[n:, n:] = a
    m[:n, n:] = da
    return torch.linalg.matrix_exp(m)[:n, n:].contiguous()


@dataclass
class propagator_cpmc(propagator_unrestricted):
    """CPMC for the Hubbard model with on-site U (propagation.py:515-657), FP64 with real
    walkers. ham_data needs "u" and the unrestricted propagation intermediates (exp_h1);
    the trial is wavefunctions.uhf_cpmc."""

    def init_prop_data(self, trial, wave_data: dict, ham_data: dict, init_walkers=None) -> PropData:
        """The unrestricted initial state, then real walkers and overlaps, the full Green's
        functions and hs_constant (propagation.py:518-537)."""
        from .wavefunctions import cpmc_overlap_green
        pd = super().init_prop_data(trial, wave_data, ham_data, init_walkers)
        w = [pd["walkers"][0].real.contiguous(), pd["walkers"][1].real.contiguous()]
        dict.__setitem__(pd, "walkers", w)
        ovl, greens = cpmc_overlap_green(trial, w, wave_data)
        dict.__setitem__(pd, "overlaps", ovl)
        dict.__setitem__(pd, "greens", greens)
        u = float(np.real(_engine._scalar(ham_data["u"])))
        gamma = math.acosh(math.exp(self.dt * u / 2))
        c = math.exp(-self.dt * u / 2)
        dict.__setitem__(pd, "hs_constant", torch.tensor(
            [[c * math.exp(gamma), c * math.exp(-gamma)], [c * math.exp(-gamma), c * math.exp(gamma)]],
            dtype=torch.float64, device=device()))
        return pd

    def propagate(self, trial, ham_data: dict, prop_data: PropData, gaussian_rns,
                  wave_data: dict) -> PropData:
        """One CPMC step with Gaussians [nw, norb] turned into uniforms (propagation.py:565-657)."""
        norb, (n_up, n_dn) = trial.norb, trial.nelec
        w = prop_data["walkers"]
        g = as_dev(gaussian_rns).contiguous()
        if tuple(g.shape) != (self.n_walkers, norb):
            raise _lib.AfqError(f"gaussian_rns must be [{self.n_walkers}, {norb}], got {tuple(g.shape)}")
        e = ham_data["exp_h1"]
        e = e if isinstance(e, torch.Tensor) else torch.as_tensor(np.asarray(e))
        eu, ed = as_dev(e[0]).contiguous(), as_dev(e[1]).contiguous()
        mo = wave_data["mo_coeff"]
        cu, cd = as_dev(mo[0]).contiguous(), as_dev(mo[1]).contiguous()
        for t in (w[0], w[1], prop_data["weights"], prop_data["overlaps"], prop_data["greens"]):
            if t.dtype != torch.float64 or not t.is_contiguous():
                raise _lib.AfqError("CPMC state must be contiguous float64 (init_prop_data of this class)")
        u = float(np.real(_engine._scalar(ham_data["u"])))
        _lib.call("afq_cpmc_propagate", norb, n_up, n_dn, self.n_walkers, float(self.dt), u, eu.data_ptr(),
                  ed.data_ptr(), cu.data_ptr(), cd.data_ptr(), w[0].data_ptr(), w[1].data_ptr(),
                  prop_data["weights"].data_ptr(), prop_data["overlaps"].data_ptr(),
                  prop_data["greens"].data_ptr(), prop_data["_scalars"].data_ptr(), g.data_ptr(), stream_ptr())
        return prop_data

    def __hash__(self) -> int:
        return super().__hash__()


@dataclass
class propagator_cpmc_nn(propagator_cpmc):
    """CPMC with on-site U and a nearest-neighbour interaction ham_data["u_1"]
    (propagator_cpmc_nn, propagation.py:889-1230), FP64 with real walkers. neighbors: a
    tuple of site pairs (i, j), i != j. The two-entry updates within one spin use the exact
    rank-two Green's-function update (the reference's fast form reads a column after its
    first step; its test checks that form against the determinant form, which this one
    matches)."""

    neighbors: Optional[tuple] = None

    def init_prop_data(self, trial, wave_data: dict, ham_data: dict, init_walkers=None) -> PropData:
        """propagator_cpmc's state plus hs_constant_onsite and hs_constant_nn
        (propagation.py:893-918)."""
        pd = super().init_prop_data(trial, wave_data, ham_data, init_walkers)
        dict.__setitem__(pd, "hs_constant_onsite", pd["hs_constant"])
        u1 = float(np.real(_engine._scalar(ham_data["u_1"])))
        gamma = math.acosh(math.exp(self.dt * u1 / 2))
        c = math.exp(-self.dt * u1 / 2)
        dict.__setitem__(pd, "hs_constant_nn", torch.tensor(
            [[c * math.exp(gamma), c * math.exp(-gamma)], [c * math.exp(-gamma), c * math.exp(gamma)]],
            dtype=torch.float64, device=device()))
        return pd

    def _neighbor_array(self, norb: int) -> torch.Tensor:
        nb = getattr(self, "_nbr_dev", None)
        if nb is None or nb[0] != (norb, self.neighbors):
            pairs = np.asarray(self.neighbors if self.neighbors is not None else (), dtype=np.int64).reshape(-1, 2)
            if pairs.size and (pairs.min() < 0 or pairs.max() >= norb or np.any(pairs[:, 0] == pairs[:, 1])):
                raise _lib.AfqError(f"neighbors must be pairs of distinct sites in [0, {norb})")
            t = torch.as_tensor(pairs.astype(np.int32)).contiguous().to(device())
            object.__setattr__(self, "_nbr_dev", ((norb, self.neighbors), t))
            return t
        return nb[1]

    def propagate(self, trial, ham_data: dict, prop_data: PropData, _gaussian_rns, wave_data: dict,
                  uniforms: Optional[torch.Tensor] = None) -> PropData:
        """One step (propagation.py:920-1226). The reference ignores the Gaussians and draws
        its uniforms from prop_data["key"]; here too, unless `uniforms`
        [nw, norb + 4 npairs] is given (column x for site x, then norb + k npairs + p for
        update k of pair p)."""
        norb, (n_up, n_dn) = trial.norb, trial.nelec
        nbr = self._neighbor_array(norb)
        npairs = int(nbr.shape[0])
        ncol = norb + 4 * npairs
        if uniforms is None:
            uni = torch.empty((self.n_walkers, ncol), dtype=torch.float64, device=device())
            key: RngKey = prop_data["key"]
            _lib.call("afq_fill_uniform", uni.data_ptr(), uni.numel(), key.seed, key.take(uni.numel()),
                      stream_ptr())
        else:
            uni = as_dev(uniforms).contiguous()
        if tuple(uni.shape) != (self.n_walkers, ncol):
            raise _lib.AfqError(f"uniforms must be [{self.n_walkers}, {ncol}], got {tuple(uni.shape)}")
        w = prop_data["walkers"]
        e = ham_data["exp_h1"]
        e = e if isinstance(e, torch.Tensor) else torch.as_tensor(np.asarray(e))
        eu, ed = as_dev(e[0]).contiguous(), as_dev(e[1]).contiguous()
        mo = wave_data["mo_coeff"]
        cu, cd = as_dev(mo[0]).contiguous(), as_dev(mo[1]).contiguous()
        for t in (w[0], w[1], prop_data["weights"], prop_data["overlaps"], prop_data["greens"]):
            if t.dtype != torch.float64 or not t.is_contiguous():
                raise _lib.AfqError("CPMC state must be contiguous float64 (init_prop_data of this class)")
        u = float(np.real(_engine._scalar(ham_data["u"])))
        u1 = float(np.real(_engine._scalar(ham_data["u_1"])))
        _lib.call("afq_cpmc_nn_propagate", norb, n_up, n_dn, self.n_walkers, float(self.dt), u, u1,
                  nbr.data_ptr() if npairs else None, npairs, eu.data_ptr(), ed.data_ptr(), cu.data_ptr(),
                  cd.data_ptr(), w[0].data_ptr(), w[1].data_ptr(), prop_data["weights"].data_ptr(),
                  prop_data["overlaps"].data_ptr(), prop_data["greens"].data_ptr(), prop_data["_scalars"].data_ptr(),
                  uni.data_ptr(), stream_ptr())
        return prop_data

    def __hash__(self) -> int:
        return hash((self.dt, self.n_walkers, self.neighbors))


@dataclass
class propagator_cpmc_continuous(propagator_cpmc):
    """Continuous-field CPMC (propagation.py:1595-1675): ham_data["hs_constant"] scales the
    Gaussian fields; no discrete sweep and no Green's functions. Real walkers, as
    propagator_cpmc keeps them (the reference's unrestricted state is complex with zero
    imaginary parts for real inputs)."""

    def propagate(self, trial, ham_data: dict, prop_data: PropData, gaussian_rns,
                  wave_data: dict) -> PropData:
        norb, (n_up, n_dn) = trial.norb, trial.nelec
        w = prop_data["walkers"]
        g = as_dev(gaussian_rns).contiguous()
        if tuple(g.shape) != (self.n_walkers, norb):
            raise _lib.AfqError(f"gaussian_rns must be [{self.n_walkers}, {norb}], got {tuple(g.shape)}")
        e = ham_data["exp_h1"]
        e = e if isinstance(e, torch.Tensor) else torch.as_tensor(np.asarray(e))
        eu, ed = as_dev(e[0]).contiguous(), as_dev(e[1]).contiguous()
        mo = wave_data["mo_coeff"]
        cu, cd = as_dev(mo[0]).contiguous(), as_dev(mo[1]).contiguous()
        hs = float(np.real(_engine._scalar(ham_data["hs_constant"])))
        _lib.call("afq_cpmc_continuous_propagate", norb, n_up, n_dn, self.n_walkers, float(self.dt), hs,
                  eu.data_ptr(), ed.data_ptr(), cu.data_ptr(), cd.data_ptr(), w[0].data_ptr(), w[1].data_ptr(),
                  prop_data["weights"].data_ptr(), prop_data["overlaps"].data_ptr(),
                  prop_data["_scalars"].data_ptr(), g.data_ptr(), stream_ptr())
        return prop_data

    def __hash__(self) -> int:
        return super().__hash__()


def _any_engine(prop_data, trial, ham_data, wave_data, prop):
    """QR and SR need only sizes: reuse the engine that last propagated these walkers."""
    eng = prop_data.get("_engine") if isinstance(prop_data, dict) else None
    if trial is not None and ham_data is not None:
        eng = prop._engine(trial, ham_data, wave_data, prop_data["walkers"])
    if eng is None:
        raise _lib.AfqError("no engine bound to prop_data: call bind(trial, ham_data, wave_data) "
                            "through init_prop_data first")
    return eng


def bind(prop, trial, ham_data, wave_data, prop_data: PropData) -> PropData:
    """Remember the engine of (prop, trial, ham_data) in prop_data so that QR and SR can be
    called with the reference's one-argument signatures."""
    dict.__setitem__(prop_data, "_engine", prop._engine(trial, ham_data, wave_data,
                                                        prop_data["walkers"]))
    return prop_data
