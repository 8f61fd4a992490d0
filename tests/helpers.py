"""Builds the same small system twice: in the FP64 oracle (numpy) and in the GPU framework,
with identical inputs, walkers, fields and SR uniforms."""

from __future__ import annotations

import numpy as np

from cs_afqmc_gb300 import synthetic
from oracle import afqmc_oracle as O


class Case:
    def __init__(self, kind="rhf", norb=12, nelec=(3, 3), nchol=30, nw=8, dt=0.005,
                 restricted=True, precision="fp64", seed=5, perturb=0.2, n_batch=1,
                 orthonormal=False, h1_shift=None, hubbard=None, mixed_config=0):
        import torch
        from cs_afqmc_gb300 import hamiltonian, propagation, wavefunctions

        self.kind, self.norb, self.nelec, self.nchol, self.nw = kind, norb, nelec, nchol, nw
        self.dt, self.restricted = dt, restricted
        if hubbard is not None:  # (lx, ly, u): periodic lattice, diagonal Cholesky vectors
            lx, ly, u = hubbard
            s = synthetic.hubbard_2d(lx=lx, ly=ly, u=u, nelec=nelec, real_trial=True)
            assert kind == "rhf" and s.norb == norb and s.chol.shape[0] == nchol
        else:
            s = synthetic.molecular(norb, nelec, nchol, seed=seed, kind=kind)
        if h1_shift is not None:  # a second Hamiltonian on the same trial (correlated sampling)
            s.h1 = s.h1 + h1_shift
        self.sys = s
        rng = np.random.default_rng(seed + 100)
        mo = s.mo_coeff
        # walkers: trial + complex perturbation
        if restricted:
            w = np.repeat(mo[None].astype(np.complex128), nw, 0)
            w = w + perturb * (rng.standard_normal(w.shape) + 1j * rng.standard_normal(w.shape))
            self.walkers0 = w
        else:
            if kind == "rhf":
                mos = [mo[:, : nelec[0]], mo[:, : nelec[1]]]
            else:
                mos = mo
            ws = []
            for m in mos:
                w = np.repeat(m[None].astype(np.complex128), nw, 0)
                ws.append(w + perturb * (rng.standard_normal(w.shape) + 1j * rng.standard_normal(w.shape)))
            self.walkers0 = ws
        if orthonormal:  # walkers as they are at a measurement: right after the QR
            if isinstance(self.walkers0, list):
                self.walkers0 = [np.linalg.qr(x)[0] for x in self.walkers0]
            else:
                self.walkers0 = np.linalg.qr(self.walkers0)[0]
        # ---- oracle
        self.o_trial = O.Trial(kind, norb, nelec)
        ho = {"h0": s.h0, "h1": s.h1.copy(), "chol": s.chol.copy()}
        ho = self.o_trial.build_measurement_intermediates(ho, mo)
        ho = O.build_propagation_intermediates(ho, s.rdm1, norb, nelec, dt, restricted)
        self.o_ham = ho
        self.o_prop = O.Propagator(dt=dt, n_walkers=nw, n_exp_terms=6)
        # ---- GPU framework
        self.ham = hamiltonian.hamiltonian(norb)
        self.trial = wavefunctions.rhf(norb, nelec) if kind == "rhf" else wavefunctions.uhf(norb, nelec)
        self.wave_data = {"mo_coeff": mo, "rdm1": s.rdm1}
        hd = {"h0": s.h0, "h1": s.h1.copy(), "chol": s.chol.copy(), "ene0": 0.0}
        hd = self.ham.build_measurement_intermediates(hd, self.trial, self.wave_data)
        P = propagation.propagator_restricted if restricted else propagation.propagator_unrestricted
        self.prop = P(dt=dt, n_walkers=nw, n_exp_terms=6, n_batch=n_batch, precision=precision,
                      mixed_config=mixed_config)
        hd = self.ham.build_propagation_intermediates(hd, self.prop, self.trial, self.wave_data)
        self.ham_data = hd
        self.torch = torch

    def gpu_walkers(self, walkers=None, dtype=None):
        import torch
        w = self.walkers0 if walkers is None else walkers
        dtype = dtype or self.prop.walker_dtype
        if isinstance(w, list):
            return [torch.as_tensor(x, dtype=dtype, device="cuda").contiguous() for x in w]
        return torch.as_tensor(w, dtype=dtype, device="cuda").contiguous()

    def oracle_prop_data(self, walkers=None):
        w = self.walkers0 if walkers is None else walkers
        w = [x.copy() for x in w] if isinstance(w, list) else w.copy()
        return O.init_prop_data(self.o_prop, self.o_trial, self.o_ham, self.sys.mo_coeff, w)

    def gpu_prop_data(self, seed=11):
        from cs_afqmc_gb300.propagation import RngKey
        pd = self.prop.init_prop_data(self.trial, self.wave_data, self.ham_data,
                                      init_walkers=self.gpu_walkers())
        pd["key"] = RngKey(seed)
        return pd


def to_np(x):
    if isinstance(x, list):
        return [to_np(y) for y in x]
    return x.detach().cpu().numpy()


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
