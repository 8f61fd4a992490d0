"""Forward-mode derivative of the FP64 phaseless block (the differentiation pattern,
driver.py:207-215 over sampling.py:266-317) through the C ABI.

Checks, on identical fields and SR uniforms:
* the values the derivative call returns equal those of afq_propagate_phaseless and of
  the oracle (relative 1e-9);
* d energy / d lambda and the per-block derivatives equal the oracle's central finite
  difference of the blocked energy at h1 + lambda D (Richardson-extrapolated, h = 1e-4),
  relative 1e-6 of the largest derivative: the FD truncation (O(h^4)) and rounding
  (1e-15 |E| / h) terms are both far below it;
* the same against a finite difference of the GPU's own value path through
  sampler.propagate_phaseless_ad_norot at coupling +-h (rebuilt intermediates).
"""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=24, nw=8),
    dict(kind="rhf", restricted=False, norb=9, nelec=(3, 3), nchol=17, nw=6),
    dict(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=6),
    dict(kind="rhf", restricted=True, norb=40, nelec=(9, 9), nchol=70, nw=4),
]
IDS = ["rhf-r", "rhf-u", "uhf", "rhf-40"]
N_PROP, N_ENE, N_SR = 3, 2, 2


@pytest.fixture(params=list(range(len(CASES))), ids=IDS)
def case(request):
    return Case(**CASES[request.param])


def _direction(case, seed=7):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((2, case.norb, case.norb)) * 0.1
    return d


def _draws(case, n_sr, seed=3):
    rng = np.random.default_rng(seed)
    fields = rng.standard_normal((n_sr, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=n_sr)
    return fields, zetas


@pytest.mark.parametrize("do_sr", [True, False], ids=["sr", "nosr"])
def test_jvp_against_oracle_fd(case, do_sr):
    from cs_afqmc_gb300 import sampling
    n_sr = N_SR if do_sr else 1
    fields, zetas = _draws(case, n_sr)
    D = _direction(case)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    pg = case.gpu_prop_data()
    e, de, pg = samp.propagate_phaseless_ad_norot_jvp(
        case.ham, case.ham_data, D, case.prop, pg, case.trial, case.wave_data, do_sr=do_sr,
        fields=fields, zetas=zetas if do_sr else None)
    samp_o = O.Sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    raw = {"h0": case.sys.h0, "h1": case.sys.h1, "chol": case.sys.chol}
    e_o, de_o, be_o, dbe_o, bw_o, dbw_o = O.phaseless_derivative_fd(
        samp_o, case.o_prop, case.o_trial, raw, D, case.sys.rdm1, case.sys.mo_coeff,
        case.oracle_prop_data(), fields, zetas, case.restricted, h=1e-4, do_sr=do_sr)
    assert rel_err(e.item(), e_o) < 1e-9
    assert rel_err(to_np(pg["block_energies"]), be_o) < 1e-9
    assert rel_err(to_np(pg["block_weights"]), bw_o) < 1e-9
    scale_e = max(abs(de_o), np.max(np.abs(dbe_o)), 1e-3)
    assert abs(de.item() - de_o) < 1e-6 * scale_e, (de.item(), de_o)
    assert np.max(np.abs(to_np(pg["dblock_energies"]) - dbe_o)) < 1e-6 * scale_e
    scale_w = max(np.max(np.abs(dbw_o)), 1e-3)
    assert np.max(np.abs(to_np(pg["dblock_weights"]) - dbw_o)) < 1e-6 * scale_w


def test_jvp_values_equal_value_path(case):
    """The derivative call leaves walkers, weights and energies as the plain block does."""
    from cs_afqmc_gb300 import sampling
    fields, zetas = _draws(case, N_SR, seed=9)
    D = _direction(case, seed=11)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    pa = case.gpu_prop_data()
    e_a, pa = samp.propagate_phaseless(case.ham, case.ham_data, case.prop, pa, case.trial,
                                       case.wave_data, fields=fields, zetas=zetas)
    pb = case.gpu_prop_data()
    e_b, _, pb = samp.propagate_phaseless_ad_norot_jvp(case.ham, case.ham_data, D, case.prop, pb,
                                                      case.trial, case.wave_data, fields=fields,
                                                      zetas=zetas)
    assert rel_err(e_b.item(), e_a.item()) < 1e-10
    assert rel_err(to_np(pb["weights"]), to_np(pa["weights"])) < 1e-9
    wa, wb = to_np(pa["walkers"]), to_np(pb["walkers"])
    wa = np.concatenate([x.ravel() for x in wa]) if isinstance(wa, list) else wa.ravel()
    wb = np.concatenate([x.ravel() for x in wb]) if isinstance(wb, list) else wb.ravel()
    assert rel_err(wb, wa) < 1e-9
    assert abs(pb["pop_control_ene_shift"].item() - pa["pop_control_ene_shift"].item()) < 1e-9


def test_jvp_against_gpu_value_fd(case):
    """Against a central difference of the GPU value path at coupling +-h, which rebuilds
    exp_h1 and rot_h1 from h1 + coupling D on the device."""
    from cs_afqmc_gb300 import sampling
    fields, zetas = _draws(case, N_SR, seed=13)
    D = _direction(case, seed=17)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    _, de, _ = samp.propagate_phaseless_ad_norot_jvp(case.ham, case.ham_data, D, case.prop,
                                                    case.gpu_prop_data(), case.trial, case.wave_data,
                                                    fields=fields, zetas=zetas)

    def val(c):
        e, _ = samp.propagate_phaseless_ad_norot(case.ham, case.ham_data, c, D, case.prop,
                                                 case.gpu_prop_data(), case.trial, case.wave_data,
                                                 fields=fields, zetas=zetas)
        return e.item()

    h = 1e-4
    d1 = (val(h) - val(-h)) / (2 * h)
    d2 = (val(h / 2) - val(-h / 2)) / h
    fd = (4 * d2 - d1) / 3
    assert abs(de.item() - fd) < 1e-6 * max(abs(fd), 1e-3), (de.item(), fd)


def test_driver_forward_ad_blocks():
    """driver.run_blocks_ad: block energies and weights equal the non-AD driver's on the same
    draws; the block observable is the per-call derivative plus the constant."""
    from cs_afqmc_gb300 import driver, sampling
    case = Case(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=24, nw=8)
    nb = 2
    rng = np.random.default_rng(29)
    fields = rng.standard_normal((nb, 1, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, 2))
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=1)
    e_v, w_v, _ = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                    case.trial, case.wave_data, nb, fields=fields, zetas=zetas)
    e_a, o_a, w_a, _ = driver.run_blocks_ad(samp, case.ham, case.ham_data, case.prop,
                                            case.gpu_prop_data(), case.trial, case.wave_data, nb,
                                            observable=(case.sys.h1, 0.5), fields=fields, zetas=zetas)
    assert rel_err(to_np(e_a), to_np(e_v)) < 1e-10
    assert rel_err(to_np(w_a), to_np(w_v)) < 1e-10
    assert np.all(np.isfinite(to_np(o_a)))
    # the first block starts from the same state in both drivers: its observable is the
    # first call's derivative
    pg = case.gpu_prop_data()
    _, de, _ = samp.propagate_phaseless_ad_norot_jvp(case.ham, case.ham_data, case.sys.h1, case.prop, pg,
                                                    case.trial, case.wave_data, fields=fields[0],
                                                    zetas=zetas[0][:1])
    assert abs(to_np(o_a)[0] - (de.item() + 0.5)) < 1e-10 * max(1.0, abs(de.item()))


def test_jvp_rejects_mixed_precision():
    from cs_afqmc_gb300 import _lib, sampling
    case = Case(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=24, nw=8, precision="mixed")
    samp = sampling.sampler(n_prop_steps=1, n_ene_blocks=1, n_sr_blocks=1)
    with pytest.raises(_lib.AfqError):
        samp.propagate_phaseless_ad_norot_jvp(case.ham, case.ham_data, _direction(case), case.prop,
                                              case.gpu_prop_data(), case.trial, case.wave_data)
