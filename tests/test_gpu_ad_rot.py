"""Forward- and reverse-mode derivatives with orbital rotation (sampler.propagate_phaseless_ad,
sampling.py:173-196, and _ad_nosr 221-254: the trial re-optimised by trial.optimize for
h1 + lambda D; the driver's default options["orbital_rotation"]) through the C ABI.

Checks, on identical fields and SR uniforms:
* the optimised trial equals the oracle's SCF iterations (1e-10);
* the values of the derivative call equal the value path propagate_phaseless_ad (1e-10)
  and the oracle's (1e-9);
* d energy / d lambda and the per-block derivatives equal the oracle's Richardson central
  difference with the trial re-optimised at every lambda (relative 1e-6, as for the
  fixed-trial derivative);
* the driver's forward mode with orbital rotation against its own per-block call, and its
  reverse mode against the forward one;
* the reverse mode (rdm1) against the forward mode along three directions (relative 1e-8).
(The fixed-trial tests of test_gpu_ad.py go through the same entry point with no trial
tangents.)
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
]
IDS = ["rhf-r", "rhf-u", "uhf"]
N_PROP, N_ENE, N_SR = 3, 2, 2


@pytest.fixture(params=list(range(len(CASES))), ids=IDS)
def case(request):
    return Case(**CASES[request.param])


def _draws(case, n_sr, seed=3):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n_sr, N_ENE, N_PROP, case.nw, case.nchol)), rng.uniform(size=n_sr)


def _direction(case, seed=7):
    return np.random.default_rng(seed).standard_normal((2, case.norb, case.norb)) * 0.1


def test_optimize_matches_oracle(case):
    wd = case.trial.optimize(case.ham_data, case.wave_data)
    chol3 = np.asarray(case.sys.chol).reshape(-1, case.norb, case.norb)
    h1 = np.asarray(case.sys.h1)
    h1 = np.stack([h1, h1]) if h1.ndim == 2 else h1
    if case.kind == "rhf":
        want = [O.rhf_optimize(h1, chol3, case.sys.mo_coeff, case.nelec[0], 30)]
        got = [to_np(wd["mo_coeff"])]
    else:
        want = O.uhf_optimize(h1, chol3, case.sys.mo_coeff, case.nelec, 30)
        got = to_np(wd["mo_coeff"])
    for a, b in zip(got, want):
        assert np.max(np.abs(a - b)) < 1e-10
    assert wd["rdm1"] is case.wave_data["rdm1"]


@pytest.mark.parametrize("do_sr", [True, False], ids=["sr", "nosr"])
def test_jvp_rot_against_oracle_fd(case, do_sr):
    from cs_afqmc_gb300 import sampling
    n_sr = N_SR if do_sr else 1
    fields, zetas = _draws(case, n_sr)
    D = _direction(case)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    e, de, pg = samp.propagate_phaseless_ad_jvp(case.ham, case.ham_data, D, case.prop, case.gpu_prop_data(),
                                                case.trial, case.wave_data, do_sr=do_sr, fields=fields,
                                                zetas=zetas if do_sr else None)
    samp_o = O.Sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    raw = {"h0": case.sys.h0, "h1": case.sys.h1, "chol": case.sys.chol}
    e_o, de_o, be_o, dbe_o, bw_o, dbw_o = O.phaseless_derivative_fd(
        samp_o, case.o_prop, case.o_trial, raw, D, case.sys.rdm1, case.sys.mo_coeff,
        case.oracle_prop_data(), fields, zetas, case.restricted, h=1e-4, do_sr=do_sr, orbital_rotation=True)
    assert rel_err(e.item(), e_o) < 1e-9
    assert rel_err(to_np(pg["block_energies"]), be_o) < 1e-9
    scale_e = max(abs(de_o), np.max(np.abs(dbe_o)), 1e-3)
    assert abs(de.item() - de_o) < 1e-6 * scale_e, (de.item(), de_o)
    assert np.max(np.abs(to_np(pg["dblock_energies"]) - dbe_o)) < 1e-6 * scale_e
    scale_w = max(np.max(np.abs(dbw_o)), 1e-3)
    assert np.max(np.abs(to_np(pg["dblock_weights"]) - dbw_o)) < 1e-6 * scale_w
    if do_sr:
        e_v, _ = samp.propagate_phaseless_ad(case.ham, case.ham_data, 0.0, D, case.prop, case.gpu_prop_data(),
                                             case.trial, case.wave_data, fields=fields, zetas=zetas)
        assert rel_err(e.item(), e_v.item()) < 1e-10


def test_driver_forward_rotation():
    from cs_afqmc_gb300 import driver, sampling
    case = Case(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=6)
    nb = 2
    rng = np.random.default_rng(33)
    fields = rng.standard_normal((nb, 1, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, 2))
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=1)
    e_a, o_a, w_a, _ = driver.run_blocks_ad(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                            case.trial, case.wave_data, nb, observable=(case.sys.h1, 0.25),
                                            fields=fields, zetas=zetas, orbital_rotation=True)
    _, de, _ = samp.propagate_phaseless_ad_jvp(case.ham, case.ham_data, case.sys.h1, case.prop, case.gpu_prop_data(),
                                               case.trial, case.wave_data, fields=fields[0], zetas=zetas[0][:1])
    assert abs(to_np(o_a)[0] - (de.item() + 0.25)) < 1e-10 * max(1.0, abs(de.item()))
    assert np.all(np.isfinite(to_np(e_a))) and np.all(np.isfinite(to_np(w_a)))
    e_r, o_r, w_r, pr = driver.run_blocks_ad(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                             case.trial, case.wave_data, nb, observable=(case.sys.h1, 0.25),
                                             fields=fields, zetas=zetas, ad_mode="reverse", orbital_rotation=True)
    assert rel_err(to_np(e_r), to_np(e_a)) < 1e-10
    assert rel_err(to_np(o_r), to_np(o_a)) < 1e-8


@pytest.mark.parametrize("do_sr", [True, False], ids=["sr", "nosr"])
def test_vjp_rot_is_transpose_of_jvp_rot(case, do_sr):
    """Reverse mode with orbital rotation: sum(rdm1 * D) equals the rotated forward-mode
    derivative along three directions (relative 1e-8), and the energy equals
    propagate_phaseless_ad's."""
    from cs_afqmc_gb300 import sampling
    n_sr = N_SR if do_sr else 1
    fields, zetas = _draws(case, n_sr, seed=19)
    z = zetas if do_sr else None
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    e, rdm1, _ = samp.propagate_phaseless_ad_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(), case.trial,
                                                 case.wave_data, do_sr=do_sr, fields=fields, zetas=z)
    r = to_np(rdm1)
    assert np.all(np.isfinite(r))
    if do_sr:
        e_v, _ = samp.propagate_phaseless_ad(case.ham, case.ham_data, 0.0, 0.0 * case.sys.h1, case.prop,
                                             case.gpu_prop_data(), case.trial, case.wave_data, fields=fields,
                                             zetas=zetas)
        assert rel_err(e.item(), e_v.item()) < 1e-10
    rng = np.random.default_rng(53)
    got, want = [], []
    for _ in range(3):
        D = rng.standard_normal((2, case.norb, case.norb)) * 0.1
        _, de, _ = samp.propagate_phaseless_ad_jvp(case.ham, case.ham_data, D, case.prop, case.gpu_prop_data(),
                                                   case.trial, case.wave_data, do_sr=do_sr, fields=fields, zetas=z)
        got.append(float(np.sum(r * D)))
        want.append(de.item())
    scale = max(np.max(np.abs(want)), 1e-3)
    assert np.max(np.abs(np.array(got) - np.array(want))) < 1e-8 * scale, (got, want)


@pytest.mark.parametrize("kind,restricted,nelec", [("rhf", True, (2, 2)), ("uhf", False, (3, 2))],
                         ids=["rhf-r", "uhf"])
def test_two_body_vjp_against_fd(kind, restricted, nelec):
    """ad_mode "2rdm" (sampler.propagate_phaseless_ad_1, sampling.py:198-229): the gradient of
    the block energy with respect to the two-body operator (Cholesky vectors rebuilt by the
    modified Cholesky decomposition, the trial re-optimised) contracted with a random
    8-fold-symmetric direction T equals the Richardson central difference of the value path
    at V +- eps T (relative 1e-6); the energy equals the value path's."""
    from cs_afqmc_gb300 import sampling
    norb, nchol = 6, 8
    case = Case(kind=kind, restricted=restricted, norb=norb, nelec=nelec, nchol=nchol, nw=4)
    ch = np.asarray(case.sys.chol).reshape(nchol, norb * norb)
    V = (ch.T @ ch).reshape(norb, norb, norb, norb)
    rng = np.random.default_rng(61)
    fields = rng.standard_normal((1, 2, 2, case.nw, nchol))
    zetas = rng.uniform(size=1)
    samp = sampling.sampler(n_prop_steps=2, n_ene_blocks=2, n_sr_blocks=1)
    e, rdm2, _ = samp.propagate_phaseless_ad_1_vjp(case.ham, case.ham_data, V, case.prop, case.gpu_prop_data(),
                                                   case.trial, case.wave_data, fields=fields, zetas=zetas)
    r = to_np(rdm2)
    assert r.shape == (norb,) * 4 and np.all(np.isfinite(r))

    def val(eps, T):
        e_, _ = samp.propagate_phaseless_ad_1(case.ham, case.ham_data, 0.0, V + eps * T, case.prop,
                                              case.gpu_prop_data(), case.trial, case.wave_data, fields=fields,
                                              zetas=zetas)
        return e_.item()

    # a direction with the 8-fold symmetry of real-orbital integrals: V's diagonal has exact
    # (ij) / (ji) ties, and the pivoted decomposition is differentiable only along directions
    # that keep them (the reference's argmax picks the first of a tie as torch's does)
    T = rng.standard_normal((norb,) * 4) * 0.05
    T = (T + T.transpose(1, 0, 2, 3)) / 2
    T = (T + T.transpose(0, 1, 3, 2)) / 2
    T = (T + T.transpose(2, 3, 0, 1)) / 2
    assert rel_err(e.item(), val(0.0, T)) < 1e-10
    h = 1e-4
    d1 = (val(h, T) - val(-h, T)) / (2 * h)
    d2 = (val(h / 2, T) - val(-h / 2, T)) / h
    fd = (4 * d2 - d1) / 3
    got = float(np.sum(r * T))
    assert abs(got - fd) < 1e-6 * max(abs(fd), 1e-3), (got, fd)


def test_driver_two_body_mode():
    """driver.run_blocks_ad(ad_mode="2rdm"): block energies equal the value path on the
    rebuilt Hamiltonian, the observable is the trial's value plus the constant, and the
    per-block two-body density matrices are finite [n_blocks, norb, norb, norb, norb]."""
    from cs_afqmc_gb300 import driver, sampling
    norb, nchol = 6, 8
    case = Case(kind="rhf", restricted=True, norb=norb, nelec=(2, 2), nchol=nchol, nw=4)
    nb = 2
    rng = np.random.default_rng(71)
    fields = rng.standard_normal((nb, 1, 2, 2, case.nw, nchol))
    zetas = rng.uniform(size=(nb, 2))
    samp = sampling.sampler(n_prop_steps=2, n_ene_blocks=2, n_sr_blocks=1)
    e_a, o_a, w_a, pa = driver.run_blocks_ad(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                             case.trial, case.wave_data, nb, observable=(case.sys.h1, 0.5),
                                             fields=fields, zetas=zetas, ad_mode="2rdm")
    r2 = to_np(pa["block_rdm2s"])
    assert r2.shape == (nb,) + (norb,) * 4 and np.all(np.isfinite(r2))
    rdm1 = to_np(case.trial.get_rdm1(case.wave_data))
    want = float(np.sum(rdm1 * np.broadcast_to(case.sys.h1, rdm1.shape))) + 0.5
    assert np.allclose(to_np(o_a), want, rtol=1e-12, atol=1e-12)
    assert np.all(np.isfinite(to_np(e_a))) and np.all(np.isfinite(to_np(w_a)))
