"""Reverse-mode derivative of the FP64 phaseless block (ad_mode "reverse", driver.py:217-229
over sampling.py:266-317) through the C ABI: the block's one-body density matrix
rdm1 = d energy / d h1 in one backward sweep.

Checks, on identical fields and SR uniforms:
* the values the call returns equal those of afq_propagate_phaseless (relative 1e-10);
* sum(rdm1 * D) equals the forward-mode derivative along D for several directions D
  (relative 1e-8 of the largest derivative): the vjp is the transpose of the jvp, which
  itself matches the oracle's finite differences;
* sum(rdm1 * D) equals the oracle's Richardson-extrapolated central difference of the
  blocked energy at h1 + lambda D (relative 1e-6, as for the jvp);
* the host-side transposes (expm Frechet derivative, trial rotation, symmetrisation)
  against the forward maps for random cotangents (relative 1e-12);
* the driver's reverse mode against the value driver and its own per-block calls.
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


def _draws(case, n_sr, seed=3):
    rng = np.random.default_rng(seed)
    fields = rng.standard_normal((n_sr, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=n_sr)
    return fields, zetas


@pytest.mark.parametrize("do_sr", [True, False], ids=["sr", "nosr"])
def test_vjp_is_transpose_of_jvp(case, do_sr):
    from cs_afqmc_gb300 import sampling
    n_sr = N_SR if do_sr else 1
    fields, zetas = _draws(case, n_sr)
    z = zetas if do_sr else None
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    e_v, pv = samp.propagate_phaseless_ad_norot(case.ham, case.ham_data, 0.0, 0.0 * case.sys.h1, case.prop,
                                                case.gpu_prop_data(), case.trial, case.wave_data,
                                                fields=fields, zetas=zetas) if do_sr else (None, None)
    e, rdm1, pg = samp.propagate_phaseless_ad_norot_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                                        case.trial, case.wave_data, do_sr=do_sr, fields=fields,
                                                        zetas=z)
    r = to_np(rdm1)
    assert r.shape == (2, case.norb, case.norb)
    assert np.all(np.isfinite(r))
    assert np.max(np.abs(r - r.transpose(0, 2, 1))) < 1e-12 * max(1.0, np.max(np.abs(r)))
    if e_v is not None:
        assert rel_err(e.item(), e_v.item()) < 1e-10
        assert rel_err(to_np(pg["block_energies"]), to_np(pv["block_energies"])) < 1e-10
        assert rel_err(to_np(pg["weights"]), to_np(pv["weights"])) < 1e-10
    rng = np.random.default_rng(41)
    got, want = [], []
    for _ in range(3):
        D = rng.standard_normal((2, case.norb, case.norb)) * 0.1
        _, de, _ = samp.propagate_phaseless_ad_norot_jvp(case.ham, case.ham_data, D, case.prop,
                                                        case.gpu_prop_data(), case.trial, case.wave_data,
                                                        do_sr=do_sr, fields=fields, zetas=z)
        got.append(float(np.sum(r * D)))
        want.append(de.item())
    scale = max(np.max(np.abs(want)), 1e-3)
    assert np.max(np.abs(np.array(got) - np.array(want))) < 1e-8 * scale, (got, want)


def test_vjp_against_oracle_fd(case):
    from cs_afqmc_gb300 import sampling
    fields, zetas = _draws(case, N_SR, seed=5)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    e, rdm1, _ = samp.propagate_phaseless_ad_norot_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                                       case.trial, case.wave_data, fields=fields, zetas=zetas)
    D = np.random.default_rng(43).standard_normal((2, case.norb, case.norb)) * 0.1
    samp_o = O.Sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    raw = {"h0": case.sys.h0, "h1": case.sys.h1, "chol": case.sys.chol}
    e_o, de_o, be_o, dbe_o, _, _ = O.phaseless_derivative_fd(
        samp_o, case.o_prop, case.o_trial, raw, D, case.sys.rdm1, case.sys.mo_coeff,
        case.oracle_prop_data(), fields, zetas, case.restricted, h=1e-4)
    assert rel_err(e.item(), e_o) < 1e-9
    got = float(np.sum(to_np(rdm1) * D))
    scale = max(abs(de_o), np.max(np.abs(dbe_o)), 1e-3)
    assert abs(got - de_o) < 1e-6 * scale, (got, de_o)


@pytest.mark.parametrize("kind,restricted", [("rhf", True), ("rhf", False), ("uhf", False)])
def test_host_transposes(kind, restricted):
    """<sym(exp_cot(gexp) + rot_cot(grot)), D> = <gexp, dexp(D)> + <grot, drot(D)>."""
    import torch
    from cs_afqmc_gb300 import sampling
    case = Case(kind=kind, restricted=restricted, norb=9, nelec=(3, 3) if kind == "rhf" else (4, 2),
                nchol=15, nw=4)
    rng = np.random.default_rng(47)
    D = torch.as_tensor(rng.standard_normal((2, case.norb, case.norb))).cuda()
    dh1 = sampling.h1_direction(D, case.norb)
    dexp = case.prop.exp_h1_tangent(case.ham_data, case.trial, case.wave_data, dh1)
    drot = case.trial.rot_h1_tangent(dh1, case.wave_data)
    gexp = torch.as_tensor(rng.standard_normal(tuple(dexp.shape))).cuda()
    if isinstance(drot, list):
        grot = [torch.as_tensor(rng.standard_normal(tuple(x.shape))).cuda() for x in drot]
        rhs_rot = sum(float(torch.sum(g * d)) for g, d in zip(grot, drot))
    else:
        grot = torch.as_tensor(rng.standard_normal(tuple(drot.shape))).cuda()
        rhs_rot = float(torch.sum(grot * drot))
    rhs = float(torch.sum(gexp * dexp)) + rhs_rot
    g = case.prop.exp_h1_cotangent(case.ham_data, case.trial, case.wave_data, gexp)
    g = g + case.trial.rot_h1_cotangent(grot, case.wave_data)
    lhs = float(torch.sum(sampling._sym(g) * D))
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(rhs)), (lhs, rhs)


def test_driver_reverse_ad_blocks():
    """driver.run_blocks_ad(ad_mode="reverse"): energies and weights equal the non-AD
    driver's; the observable is sum(rdm1 * op) + constant; the first block's rdm1 equals a
    direct vjp call from the same state."""
    from cs_afqmc_gb300 import driver, sampling
    case = Case(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=6)
    nb = 2
    rng = np.random.default_rng(31)
    fields = rng.standard_normal((nb, 1, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, 2))
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=1)
    e_v, w_v, _ = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                    case.trial, case.wave_data, nb, fields=fields, zetas=zetas)
    e_a, o_a, w_a, pa = driver.run_blocks_ad(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                             case.trial, case.wave_data, nb, observable=(case.sys.h1, 0.5),
                                             fields=fields, zetas=zetas, ad_mode="reverse")
    assert rel_err(to_np(e_a), to_np(e_v)) < 1e-10
    assert rel_err(to_np(w_a), to_np(w_v)) < 1e-10
    r = to_np(pa["block_rdm1s"])
    assert r.shape == (nb, 2, case.norb, case.norb)
    h1 = np.broadcast_to(case.sys.h1, (2, case.norb, case.norb))
    assert np.allclose(to_np(o_a), np.sum(r * h1, axis=(1, 2, 3)) + 0.5, rtol=1e-12, atol=1e-12)
    _, r0, _ = samp.propagate_phaseless_ad_norot_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                                     case.trial, case.wave_data, fields=fields[0],
                                                     zetas=zetas[0][:1])
    assert rel_err(r[0], to_np(r0)) < 1e-12


def test_vjp_rejects_mixed_precision():
    from cs_afqmc_gb300 import _lib, sampling
    case = Case(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=24, nw=8, precision="mixed")
    samp = sampling.sampler(n_prop_steps=1, n_ene_blocks=1, n_sr_blocks=1)
    with pytest.raises(_lib.AfqError):
        samp.propagate_phaseless_ad_norot_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                              case.trial, case.wave_data)


def test_vjp_chunked_vhs():
    """n_batch 2: the backward sweep recomputes vhs and runs the Taylor adjoint per walker
    chunk; the result equals the unchunked call's."""
    from cs_afqmc_gb300 import sampling
    a = Case(kind="rhf", restricted=False, norb=9, nelec=(3, 3), nchol=17, nw=6)
    b = Case(kind="rhf", restricted=False, norb=9, nelec=(3, 3), nchol=17, nw=6, n_batch=2)
    fields, zetas = _draws(a, N_SR, seed=51)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    ea, ra, _ = samp.propagate_phaseless_ad_norot_vjp(a.ham, a.ham_data, a.prop, a.gpu_prop_data(), a.trial,
                                                      a.wave_data, fields=fields, zetas=zetas)
    eb, rb, _ = samp.propagate_phaseless_ad_norot_vjp(b.ham, b.ham_data, b.prop, b.gpu_prop_data(), b.trial,
                                                      b.wave_data, fields=fields, zetas=zetas)
    assert rel_err(eb.item(), ea.item()) < 1e-12
    assert rel_err(to_np(rb), to_np(ra)) < 1e-10


@pytest.mark.parametrize("rotation", [False, True], ids=["fixed", "rotated"])
def test_autograd_function(rotation):
    """cs_afqmc_gb300.autograd.phaseless_energy: torch.autograd.grad of the block energy with
    respect to h1 is the adjoint sweep's rdm1; its contraction with a direction equals the
    forward-mode derivative (relative 1e-8)."""
    import torch
    from cs_afqmc_gb300 import autograd, sampling
    case = Case(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=6)
    fields, zetas = _draws(case, N_SR, seed=57)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    h1 = torch.as_tensor(np.asarray(case.ham_data["h1"].cpu()), dtype=torch.float64, device="cuda")
    h1 = h1.clone().requires_grad_(True)
    e = autograd.phaseless_energy(h1, samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(), case.trial,
                                  case.wave_data, fields=fields, zetas=zetas, orbital_rotation=rotation)
    (g,) = torch.autograd.grad(2.0 * e, h1)
    D = np.random.default_rng(59).standard_normal((2, case.norb, case.norb)) * 0.1
    jvp = samp.propagate_phaseless_ad_jvp if rotation else samp.propagate_phaseless_ad_norot_jvp
    e_j, de, _ = jvp(case.ham, case.ham_data, D, case.prop, case.gpu_prop_data(), case.trial, case.wave_data,
                     fields=fields, zetas=zetas)
    assert rel_err(e.item(), e_j.item()) < 1e-10
    got = float(np.sum(to_np(g) * D)) / 2.0
    assert abs(got - de.item()) < 1e-8 * max(abs(de.item()), 1e-3), (got, de.item())
