"""Properties of the FP64 oracle's propagation pieces that the reference's own tests leave
unchecked (they test shapes only, with JAX-drawn fields): the Taylor series of the
propagator against the matrix exponential, the comb resampling on a hand-worked weight
vector, the QR convention, and the weight rules of the phaseless step (propagation.py:
133-164). No GPU."""

import math

import numpy as np
import pytest
import scipy.linalg

from cs_afqmc_gb300 import synthetic
from oracle import afqmc_oracle as O


def _system(norb=8, nelec=(3, 3), nchol=20, nw=6, dt=0.005, seed=3):
    s = synthetic.molecular(norb, nelec, nchol, seed=seed, kind="rhf")
    trial = O.Trial("rhf", norb, nelec)
    ham = {"h0": s.h0, "h1": s.h1.copy(), "chol": s.chol.copy()}
    ham = trial.build_measurement_intermediates(ham, s.mo_coeff)
    ham = O.build_propagation_intermediates(ham, s.rdm1, norb, nelec, dt, True)
    prop = O.Propagator(dt=dt, n_walkers=nw, n_exp_terms=6)
    rng = np.random.default_rng(seed + 1)
    w = np.repeat(s.mo_coeff[None].astype(np.complex128), nw, 0)
    w = w + 0.05 * (rng.standard_normal(w.shape) + 1j * rng.standard_normal(w.shape))
    pd = O.init_prop_data(prop, trial, ham, s.mo_coeff, w)
    return s, trial, ham, prop, pd


def test_taylor_series_is_the_exponential_to_sixth_order():
    """W -> E (sum_{m<6} V^m / m!) E W: with E = I it is expm(V) W up to the V^6 / 720 term,
    and with V = 0 it is E E W (propagation.py:67-92)."""
    rng = np.random.default_rng(1)
    n, k, nw = 10, 4, 3
    w = rng.standard_normal((nw, n, k)) + 1j * rng.standard_normal((nw, n, k))
    v = 0.05 * (rng.standard_normal((nw, n, n)) + 1j * rng.standard_normal((nw, n, n)))
    got = O.apply_trotprop_det(np.eye(n), v, w, 6)
    for i in range(nw):
        ref = scipy.linalg.expm(v[i]) @ w[i]
        nv = np.linalg.norm(v[i], 2)
        bound = nv ** 6 / math.factorial(6) * np.exp(nv) * np.linalg.norm(w[i], 2)
        assert np.linalg.norm(got[i] - ref, 2) <= 1.01 * bound
        assert np.linalg.norm(got[i] - ref, 2) > 0.0  # the series is truncated, not exact
    e = scipy.linalg.expm(-0.01 * (rng.standard_normal((n, n)) + rng.standard_normal((n, n)).T))
    assert np.allclose(O.apply_trotprop_det(e, np.zeros_like(v), w, 6), e @ e @ w, atol=1e-14)


def test_comb_resampling_known_indices():
    """sr.py:24-47 on w = [0, 1, 2, 0, 1], zeta = 0.5: cumsum [0, 1, 3, 3, 4], total 4,
    z = 4 (i + 0.5) / 5 = [0.4, 1.2, 2.0, 2.8, 3.6], left-side search -> [1, 2, 2, 2, 4]."""
    prop = O.Propagator(dt=0.01, n_walkers=5)
    walkers = np.arange(5, dtype=np.complex128)[:, None, None] * np.ones((5, 2, 1))
    pd = {"weights": np.array([0.0, 1.0, 2.0, 0.0, 1.0]), "walkers": walkers.copy()}
    pd = prop.stochastic_reconfiguration(pd, 0.5)
    assert list(pd["sr_indices"]) == [1, 2, 2, 2, 4]
    assert np.allclose(pd["walkers"][:, 0, 0].real, [1, 2, 2, 2, 4])
    assert np.allclose(pd["weights"], 0.8) and math.isclose(pd["weights"].sum(), 4.0)


@pytest.mark.parametrize("zeta", [0.0, 0.3, 0.999999])
def test_comb_never_picks_a_dead_walker(zeta):
    rng = np.random.default_rng(7)
    nw = 40
    wts = rng.uniform(0.5, 1.5, nw)
    wts[rng.choice(nw, 10, replace=False)] = 0.0
    prop = O.Propagator(dt=0.01, n_walkers=nw)
    pd = prop.stochastic_reconfiguration({"weights": wts.copy(), "walkers": np.zeros((nw, 2, 1))}, zeta)
    assert np.all(wts[pd["sr_indices"]] > 0.0)
    assert np.all(np.diff(pd["sr_indices"]) >= 0)
    assert math.isclose(pd["weights"].sum(), wts.sum())


def test_qr_keeps_the_span_lapack_convention():
    """orthonormalize_walkers: Q^H Q = I and Q (Q^H W) = W with Q^H W upper triangular and a
    real diagonal (the Householder convention of jnp.linalg.qr, linalg_utils.py:51-65)."""
    _, _, _, prop, pd = _system()
    w0 = pd["walkers"].copy()
    pd = prop.orthonormalize_walkers(pd)
    q = pd["walkers"]
    for i in range(q.shape[0]):
        assert np.allclose(q[i].conj().T @ q[i], np.eye(q.shape[2]), atol=1e-13)
        r = q[i].conj().T @ w0[i]
        assert np.allclose(q[i] @ r, w0[i], atol=1e-13)
        assert np.allclose(np.tril(r, -1), 0.0, atol=1e-13)
        assert np.allclose(np.diagonal(r).imag, 0.0, atol=1e-13)


@pytest.mark.filterwarnings("ignore:divide by zero:RuntimeWarning")
def test_phaseless_weight_rules():
    """propagation.py:133-164: an importance factor below 1e-3 or above 100, or NaN, kills the
    walker; the population-control shift is e_estimate - 0.1 ln(sum w / nw) / dt."""
    s, trial, ham, prop, pd = _system()
    rng = np.random.default_rng(4)
    fields = rng.standard_normal((prop.n_walkers, s.nchol))
    ref = prop.propagate(trial, ham, {k: (v.copy() if hasattr(v, "copy") else v) for k, v in pd.items()},
                         fields, s.mo_coeff)
    w = ref["weights"]
    assert np.all((w == 0.0) | ((w >= 1e-3) & (w <= 100.0)))
    assert math.isclose(ref["pop_control_ene_shift"],
                        ref["e_estimate"] - 0.1 * math.log(w.sum() / prop.n_walkers) / prop.dt, rel_tol=1e-14)
    # lowering the population-control shift by 1/dt scales every importance factor by e^-1;
    # lowering it by 7/dt pushes all of them (here near 1) below 1e-3
    for shift, alive in ((-1.0, True), (-7.0, False)):
        p2 = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in pd.items()}
        p2["pop_control_ene_shift"] = pd["pop_control_ene_shift"] + shift / prop.dt
        p2 = prop.propagate(trial, ham, p2, fields, s.mo_coeff)
        if alive:
            live = (w > 0) & (w * math.exp(-1.0) >= 1e-3)
            assert np.allclose(p2["weights"][live], w[live] * math.exp(-1.0), rtol=1e-12)
        else:
            assert np.all(p2["weights"] == 0.0)
    # a shift of +6/dt pushes them above 100
    p3 = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in pd.items()}
    p3["pop_control_ene_shift"] = pd["pop_control_ene_shift"] + 6.0 / prop.dt
    p3 = prop.propagate(trial, ham, p3, fields, s.mo_coeff)
    assert np.all(p3["weights"] == 0.0)
    # a zero overlap makes the ratio infinite / NaN: weight 0, not an error
    p4 = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in pd.items()}
    p4["overlaps"] = p4["overlaps"].copy()
    p4["overlaps"][0] = 0.0
    p4 = prop.propagate(trial, ham, p4, fields, s.mo_coeff)
    assert p4["weights"][0] == 0.0 and np.all(np.isfinite(p4["weights"]))
