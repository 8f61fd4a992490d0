"""Correlated sampling (ad_afqmc/corr_sample/corr_sample.py:514-694) on the GPU against the
FP64 oracle: two Hamiltonians h1 and h1 + lambda D on the same trial and the same field
draws, cs_steps_scan with field blocks, weight-outlier removal and per-step sums.

Tolerance: FP64 kernels reorder sums relative to NumPy, so the per-step sums agree to
1e-9 relative and the walkers to 1e-8 after several blocks (as in test_gpu_fp64_parity).
The mixed path is checked to 5e-5 relative on the same quantities.
"""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu


def _pair(precision, kind="rhf", restricted=True, norb=12, nelec=(3, 3), nchol=30, nw=16):
    rng = np.random.default_rng(17)
    d = rng.normal(0.0, 0.05, (norb, norb))
    d = np.triu(d) + np.triu(d, 1).T
    lam = 1e-2
    kw = dict(kind=kind, restricted=restricted, norb=norb, nelec=nelec, nchol=nchol, nw=nw,
              precision=precision, orthonormal=True, perturb=0.05)
    return Case(**kw, h1_shift=lam * d), Case(**kw, h1_shift=-lam * d)


def _flat(w):
    return np.concatenate([x.ravel() for x in w]) if isinstance(w, list) else w.ravel()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 5e-5)])
@pytest.mark.parametrize("kind,restricted,nelec", [("rhf", True, (3, 3)), ("uhf", False, (4, 2))])
def test_cs_steps_scan_matches_oracle(precision, tol, kind, restricted, nelec):
    from cs_afqmc_gb300 import corr_sample, sampling
    a, b = _pair(precision, kind, restricted, nelec=nelec)
    steps, n_prop = 3, 4
    fields = np.random.default_rng(5).standard_normal((steps, n_prop, a.nw, a.nchol))
    samp_o = O.Sampler(n_prop_steps=n_prop, n_ene_blocks=1, n_sr_blocks=1)
    pa_o, pb_o = a.oracle_prop_data(), b.oracle_prop_data()
    pa_o, pb_o, e1, w1, e2, w2 = O.cs_steps_scan(
        samp_o, (a.o_prop, a.o_trial, a.o_ham, pa_o, a.sys.mo_coeff),
        (b.o_prop, b.o_trial, b.o_ham, pb_o, b.sys.mo_coeff), fields)
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=1, n_sr_blocks=1)
    pa, pb = a.gpu_prop_data(), b.gpu_prop_data()
    (pa, pb), (ge1, gw1, ge2, gw2) = corr_sample.cs_steps_scan(
        steps, pa, a.ham_data, a.prop, a.trial, a.wave_data,
        pb, b.ham_data, b.prop, b.trial, b.wave_data, samp, fields=fields)
    for g, o in ((ge1, e1), (gw1, w1), (ge2, e2), (gw2, w2)):
        assert rel_err(to_np(g), o) < tol
    assert rel_err(_flat(to_np(pa["walkers"])), _flat(pa_o["walkers"])) < 10 * tol
    assert rel_err(to_np(pb["weights"]), pb_o["weights"]) < tol
    # the correlated energy difference
    d_gpu = to_np(ge1).sum() / to_np(gw1).sum() - to_np(ge2).sum() / to_np(gw2).sum()
    d_o = e1.sum() / w1.sum() - e2.sum() / w2.sum()
    assert abs(d_gpu - d_o) < tol * max(1.0, abs(e1.sum() / w1.sum()))


def test_outlier_removal_matches_oracle():
    import torch
    from cs_afqmc_gb300 import _lib
    from cs_afqmc_gb300._engine import stream_ptr
    rng = np.random.default_rng(3)
    nw = 1000
    w1 = rng.uniform(0.5, 1.5, nw)
    w2 = w1 * rng.uniform(0.9, 1.1, nw)
    w1[[7, 300]] = 40.0    # outliers in system 1
    w2[[55]] = 60.0        # and in system 2
    e1, e2 = rng.normal(-5, 1, nw), rng.normal(-5, 1, nw)
    r1, r2 = O.corr_otler_rm(w1.copy(), w2.copy())
    dw1 = torch.as_tensor(w1, device="cuda")
    dw2 = torch.as_tensor(w2, device="cuda")
    de1, de2 = torch.as_tensor(e1, device="cuda"), torch.as_tensor(e2, device="cuda")
    sums = torch.empty(4, dtype=torch.float64, device="cuda")
    _lib.call("afq_cs_outlier_removal", dw1.data_ptr(), dw2.data_ptr(), de1.data_ptr(), de2.data_ptr(),
              nw, 5.0, sums.data_ptr(), stream_ptr())
    assert np.array_equal(to_np(dw1), r1) and np.array_equal(to_np(dw2), r2)
    assert r1[7] == 0 and r2[300] == 0 and r1[55] == 0
    ref = [np.sum(e1 * r1), np.sum(r1), np.sum(e2 * r2), np.sum(r2)]
    assert rel_err(to_np(sums), ref) < 1e-13


@pytest.mark.parametrize("kind,restricted,nelec", [("rhf", True, (3, 3)), ("uhf", False, (4, 2))])
def test_cs_derivative_equals_forward_mode_on_the_same_trajectory(kind, restricted, nelec):
    """Correlated sampling and the forward-mode derivative estimate the same quantity when
    they follow the same trajectory: K field blocks without SR and without outlier
    removal (z_thresh = inf) from the same walkers and the same (lambda = 0) starting
    e_estimate, blocked energy sum_k E_k W_k / sum_k W_k. The central difference of the
    correlated pair at lambda = +-1e-4 then equals the jvp of
    propagate_phaseless_ad_nosr_norot with K energy blocks (relative 1e-6: the difference's
    own O(lambda^2) error). The driver's per-block forward mode differs from both by design:
    each block's walkers enter with a zero tangent and SR follows every block."""
    import torch
    from cs_afqmc_gb300 import corr_sample, sampling
    norb, nchol, nw = 12, 30, 16
    rng = np.random.default_rng(17)
    d = rng.normal(0.0, 0.05, (norb, norb))
    d = np.triu(d) + np.triu(d, 1).T
    lam = 1e-4
    kw = dict(kind=kind, restricted=restricted, norb=norb, nelec=nelec, nchol=nchol, nw=nw, orthonormal=True,
              perturb=0.05)
    a, b, c = Case(**kw, h1_shift=lam * d), Case(**kw, h1_shift=-lam * d), Case(**kw)
    K, n_prop = 3, 4
    fields = np.random.default_rng(5).standard_normal((K, n_prop, nw, nchol))
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=1, n_sr_blocks=1)
    pc = c.gpu_prop_data()
    pa, pb = a.gpu_prop_data(), b.gpu_prop_data()
    for p_ in (pa, pb):  # the starting state does not depend on lambda (the jvp's zero tangent)
        p_["e_estimate"] = pc["e_estimate"]
        p_["pop_control_ene_shift"] = pc["pop_control_ene_shift"]
    (_, _), (e1, w1, e2, w2) = corr_sample.cs_steps_scan(
        K, pa, a.ham_data, a.prop, a.trial, a.wave_data,
        pb, b.ham_data, b.prop, b.trial, b.wave_data, samp, fields=fields, z_thresh=float("inf"))
    e1, w1, e2, w2 = (to_np(x) for x in (e1, w1, e2, w2))
    fd = (e1.sum() / w1.sum() - e2.sum() / w2.sum()) / (2 * lam)
    samp_k = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=K, n_sr_blocks=1)
    e, de, _ = samp_k.propagate_phaseless_ad_norot_jvp(c.ham, c.ham_data, d, c.prop, pc, c.trial, c.wave_data,
                                                       do_sr=False, fields=torch.as_tensor(fields[None]).cuda())
    assert abs(e.item() - (e1.sum() / w1.sum() + e2.sum() / w2.sum()) / 2) < 1e-7 * abs(e.item())
    assert abs(de.item() - fd) < 1e-6 * max(abs(fd), 1e-3), (de.item(), fd)
