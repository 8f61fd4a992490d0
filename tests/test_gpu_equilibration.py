"""The equilibration sweeps of the reference's driver (driver.py:91-133): blocks of the
equilibration sampler (n_prop_steps = 50, n_ene_blocks = 5, n_sr_blocks = 10), each followed
by the weight record, QR, global SR and e_estimate = 0.9 e_estimate + 0.1 E_block, on the GPU
through driver.run_equilibration against the oracle's run_blocks with the same sampler,
identical fields and SR uniforms. Tolerances: FP64 1e-9 relative (energies, weights,
walkers), mixed 5e-5 on the block energies of the first sweep."""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

N_PROP, N_ENE, N_SR = 50, 5, 10


def _draws(case, n_eql, seed=31):
    rng = np.random.default_rng(seed)
    fields = rng.standard_normal((n_eql, N_SR, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=(n_eql, N_SR + 1))
    return fields, zetas


def _oracle(case, fields, zetas, n_eql, walkers=None):
    samp = O.Sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    po = case.oracle_prop_data(walkers)
    return O.run_blocks(samp, case.o_prop, case.o_trial, case.o_ham, po, case.sys.mo_coeff,
                        lambda n: fields[n], lambda n: zetas[n], n_eql)


@pytest.mark.parametrize("cfg", [dict(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=16, nw=6),
                                 dict(kind="uhf", restricted=False, norb=9, nelec=(3, 2), nchol=14, nw=5)],
                         ids=["rhf", "uhf"])
def test_equilibration_matches_oracle_fp64(cfg):
    from cs_afqmc_gb300 import driver
    case = Case(**cfg)
    n_eql = 2
    fields, zetas = _draws(case, n_eql)
    e_o, w_o, po = _oracle(case, fields, zetas, n_eql)
    pg = case.gpu_prop_data()
    e_g, w_g, pg = driver.run_equilibration(case.ham, case.ham_data, case.prop, pg, case.trial, case.wave_data,
                                            n_eql, fields=fields, zetas=zetas)
    assert rel_err(to_np(e_g), e_o) < 1e-9
    assert rel_err(to_np(w_g), w_o) < 1e-9
    wg, wo = to_np(pg["walkers"]), po["walkers"]
    if isinstance(wo, list):
        for a, b in zip(wg, wo):
            assert rel_err(a, b) < 1e-9
    else:
        assert rel_err(wg, wo) < 1e-9
    assert abs(float(to_np(pg["e_estimate"])) - po["e_estimate"]) < 1e-9 * abs(po["e_estimate"])


def test_equilibration_mixed_first_sweep():
    from cs_afqmc_gb300 import driver
    cfg = dict(kind="rhf", restricted=True, norb=16, nelec=(4, 4), nchol=30, nw=8)
    case = Case(precision="mixed", orthonormal=True, perturb=0.05, **cfg)
    fields, zetas = _draws(case, 1)
    w0 = case.walkers0.astype(np.complex64).astype(np.complex128)
    e_o, w_o, _ = _oracle(case, fields, zetas, 1, walkers=w0)
    pg = case.gpu_prop_data()
    e_g, w_g, _ = driver.run_equilibration(case.ham, case.ham_data, case.prop, pg, case.trial, case.wave_data, 1,
                                           fields=fields, zetas=zetas)
    assert rel_err(to_np(e_g), e_o) < 5e-5
    assert rel_err(to_np(w_g), w_o) < 5e-5


def test_afqmc_driver_runs_equilibration_then_blocks():
    """driver.afqmc: equilibration sweeps then sampling blocks; the mean is the weighted
    block average and agrees with run_equilibration + run_blocks on the same draws."""
    from cs_afqmc_gb300 import driver, sampling
    case = Case(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=16, nw=6)
    samp = sampling.sampler(n_prop_steps=5, n_ene_blocks=2, n_sr_blocks=1)
    pg = case.gpu_prop_data(seed=5)
    mean, err, be, bw, _ = driver.afqmc(case.ham, case.ham_data, case.prop, pg, case.trial, case.wave_data, samp,
                                        n_eql=1, n_blocks=3)
    pg2 = case.gpu_prop_data(seed=5)
    _, _, pg2 = driver.run_equilibration(case.ham, case.ham_data, case.prop, pg2, case.trial, case.wave_data, 1)
    be2, bw2, _ = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, pg2, case.trial, case.wave_data, 3)
    assert np.allclose(to_np(be), to_np(be2), rtol=1e-12, atol=0)
    e, w = to_np(be), to_np(bw)
    assert abs(mean - np.sum(e * w) / np.sum(w)) < 1e-12 * abs(mean)
    assert err is not None and np.isfinite(err)
