"""d<E>/dU for the Hubbard model (L_i = sqrt(U) n_i, diagonal Cholesky vectors) by the FP64
reverse-mode sweep: the device returns the cotangents of chol, the mean-field shifts,
h0_prop, exp_h1 and rot_chol, torch autograd carries them to the Cholesky vectors
(sampler.propagate_phaseless_chol_vjp), and dE/dU = <dE/dL, L> / (2U)
(sampler.propagate_phaseless_u_vjp). Checked against the oracle's Richardson-extrapolated
central difference of the blocked energy in U on identical fields and SR uniforms, the
trial fixed and every intermediate rebuilt (relative 1e-6 of the derivative), on a 4 x 4
lattice with restricted and two-slab walkers, with and without SR; and the full chol
cotangent against a central difference of the GPU value path along a random symmetric
direction of the Cholesky vectors (relative 1e-6)."""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

N_PROP, N_ENE, N_SR = 3, 2, 2
U = 4.0


def _case(restricted, nw=6):
    return Case(kind="rhf", restricted=restricted, norb=16, nelec=(5, 5), nchol=16, nw=nw, hubbard=(4, 4, U),
                perturb=0.05)


def _chol_of(case):
    base = case.sys.chol / np.sqrt(U)
    return lambda u: base * np.sqrt(u)


@pytest.mark.parametrize("restricted", [True, False], ids=["restricted", "two-slab"])
@pytest.mark.parametrize("do_sr", [True, False], ids=["sr", "nosr"])
def test_du_matches_oracle_fd(restricted, do_sr):
    from cs_afqmc_gb300 import sampling
    case = _case(restricted)
    n_sr = N_SR if do_sr else 1
    rng = np.random.default_rng(5)
    fields = rng.standard_normal((n_sr, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=n_sr) if do_sr else None
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    e, du, _ = samp.propagate_phaseless_u_vjp(case.ham, case.ham_data, U, case.prop, case.gpu_prop_data(),
                                              case.trial, case.wave_data, do_sr=do_sr, fields=fields, zetas=zetas)
    samp_o = O.Sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=n_sr)
    raw = {"h0": case.sys.h0, "h1": case.sys.h1}
    e_o, du_o = O.phaseless_chol_derivative_fd(samp_o, case.o_prop, case.o_trial, raw, _chol_of(case), U,
                                               case.sys.rdm1, case.sys.mo_coeff, case.oracle_prop_data(), fields,
                                               zetas if do_sr else np.zeros(1), case.restricted, h=1e-3,
                                               do_sr=do_sr)
    assert rel_err(e.item(), e_o) < 1e-9
    assert abs(du.item() - du_o) < 1e-6 * max(abs(du_o), 1e-3), (du.item(), du_o)


def test_chol_cotangent_along_a_direction():
    """<dE/dL, T> against the GPU value path's central difference of the block energy at
    chol + eps T (T symmetric per vector, not diagonal), intermediates rebuilt."""
    import torch
    from cs_afqmc_gb300 import sampling
    case = _case(True, nw=4)
    rng = np.random.default_rng(9)
    fields = rng.standard_normal((N_SR, N_ENE, N_PROP, case.nw, case.nchol))
    zetas = rng.uniform(size=N_SR)
    samp = sampling.sampler(n_prop_steps=N_PROP, n_ene_blocks=N_ENE, n_sr_blocks=N_SR)
    _, gc, _ = samp.propagate_phaseless_chol_vjp(case.ham, case.ham_data, case.prop, case.gpu_prop_data(),
                                                 case.trial, case.wave_data, fields=fields, zetas=zetas)
    n = case.norb
    t = rng.standard_normal((case.nchol, n, n)) * 0.05
    t = (t + t.transpose(0, 2, 1)) / 2
    want = float(np.sum(to_np(gc) * t.reshape(case.nchol, -1)))

    def energy(eps):
        hd = {"h0": case.sys.h0, "h1": case.sys.h1.copy(), "chol": case.sys.chol + eps * t.reshape(case.nchol, -1),
              "ene0": 0.0}
        hd = case.ham.build_measurement_intermediates(hd, case.trial, case.wave_data)
        hd = case.ham.build_propagation_intermediates(hd, case.prop, case.trial, case.wave_data)
        e, _ = samp.propagate_phaseless(case.ham, hd, case.prop, case.gpu_prop_data(), case.trial, case.wave_data,
                                        fields=torch.as_tensor(fields).cuda(), zetas=torch.as_tensor(zetas).cuda())
        return e.item()

    h = 1e-4
    d1 = (energy(h) - energy(-h)) / (2 * h)
    d2 = (energy(h / 2) - energy(-h / 2)) / h
    fd = (4 * d2 - d1) / 3
    assert abs(want - fd) < 1e-6 * max(abs(fd), 1e-3), (want, fd)
