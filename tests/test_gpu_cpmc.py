"""CPMC for the Hubbard model (propagator_cpmc, propagation.py:515-657) through the C ABI,
against the oracle's restatement on identical Gaussian draws: walkers, weights, overlaps,
full Green's functions and the pop-control shift after several steps (relative 1e-9,
FP64 with different summation orders). The oracle's own fast (Sherman-Morrison) and slow
(determinant) forms agree, as the reference's test_propagate_cpmc checks."""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import rel_err, to_np

pytestmark = pytest.mark.gpu


def _system(lx=4, ly=2, nelec=(3, 3), nw=6, dt=0.01, u=4.0, seed=2):
    import torch
    from cs_afqmc_gb300 import hamiltonian, propagation, synthetic, wavefunctions
    s = synthetic.hubbard_2d(lx=lx, ly=ly, u=u, nelec=nelec, real_trial=True)
    n = s.norb
    rng = np.random.default_rng(seed)
    mo = [s.mo_coeff[:, :nelec[0]], s.mo_coeff[:, :nelec[1]]]
    trial = wavefunctions.uhf_cpmc(n, nelec)
    wave = {"mo_coeff": mo, "rdm1": np.stack([mo[0] @ mo[0].T, mo[1] @ mo[1].T])}
    ham = hamiltonian.hamiltonian(n)
    hd = {"h0": 0.0, "h1": s.h1, "chol": s.chol, "ene0": 0.0, "u": u}
    hd = ham.build_measurement_intermediates(hd, trial, wave)
    prop = propagation.propagator_cpmc(dt=dt, n_walkers=nw, precision="fp64")
    hd = ham.build_propagation_intermediates(hd, prop, trial, wave)
    w0 = [np.repeat(mo[0][None], nw, 0) + 0.05 * rng.standard_normal((nw, n, nelec[0])),
          np.repeat(mo[1][None], nw, 0) + 0.05 * rng.standard_normal((nw, n, nelec[1]))]
    pd = prop.init_prop_data(trial, wave, hd, init_walkers=w0)
    return s, trial, wave, hd, prop, pd, w0, mo


def test_cpmc_init_green():
    s, trial, wave, hd, prop, pd, w0, mo = _system()
    g_o = O.cpmc_full_green(w0, mo)
    assert rel_err(to_np(pd["greens"]), g_o) < 1e-12
    assert rel_err(to_np(pd["overlaps"]), O.cpmc_overlap(w0, mo)) < 1e-12


@pytest.mark.parametrize("lx,ly,nelec", [(4, 2, (3, 3)), (4, 4, (7, 5))], ids=["4x2", "4x4"])
def test_cpmc_steps(lx, ly, nelec):
    import torch
    s, trial, wave, hd, prop, pd, w0, mo = _system(lx=lx, ly=ly, nelec=nelec)
    n = s.norb
    exp_h1 = to_np(hd["exp_h1"])
    po = O.cpmc_init(w0, mo)
    e_est = pd["e_estimate"].item()
    pcs = pd["pop_control_ene_shift"].item()
    rng = np.random.default_rng(7)
    for _ in range(4):
        g = rng.standard_normal((prop.n_walkers, n))
        po, pcs = O.cpmc_propagate(exp_h1, prop.dt, 4.0, po, g, mo, e_est, pcs, prop.n_walkers)
        pd = prop.propagate(trial, hd, pd, g, wave)
    torch.cuda.synchronize()
    assert rel_err(to_np(pd["walkers"][0]), po["walkers"][0]) < 1e-9
    assert rel_err(to_np(pd["walkers"][1]), po["walkers"][1]) < 1e-9
    assert rel_err(to_np(pd["weights"]), po["weights"]) < 1e-9
    assert rel_err(to_np(pd["overlaps"]), po["overlaps"]) < 1e-9
    assert rel_err(to_np(pd["greens"]), po["greens"]) < 1e-9
    assert abs(pd["pop_control_ene_shift"].item() - pcs) < 1e-9 * max(1.0, abs(pcs))


def test_cpmc_oracle_fast_equals_slow():
    s, trial, wave, hd, prop, pd, w0, mo = _system()
    exp_h1 = to_np(hd["exp_h1"])
    rng = np.random.default_rng(5)
    a, b = O.cpmc_init(w0, mo), O.cpmc_init(w0, mo)
    for _ in range(2):
        g = rng.standard_normal((prop.n_walkers, s.norb))
        a, pa = O.cpmc_propagate(exp_h1, prop.dt, 4.0, a, g, mo, -5.0, -5.0, prop.n_walkers)
        b, pb = O.cpmc_propagate(exp_h1, prop.dt, 4.0, b, g, mo, -5.0, -5.0, prop.n_walkers, slow=True)
    assert np.allclose(a["walkers"][0], b["walkers"][0]) and np.allclose(a["weights"], b["weights"])
    assert np.allclose(a["overlaps"], b["overlaps"])


def test_cpmc_continuous_steps():
    import torch
    from cs_afqmc_gb300 import propagation
    s, trial, wave, hd, prop, pd, w0, mo = _system(lx=4, ly=4, nelec=(7, 5))
    cprop = propagation.propagator_cpmc_continuous(dt=prop.dt, n_walkers=prop.n_walkers, precision="fp64")
    hd["hs_constant"] = 0.3
    exp_h1 = to_np(hd["exp_h1"])
    po = O.cpmc_init(w0, mo)
    e_est = pd["e_estimate"].item()
    pcs = pd["pop_control_ene_shift"].item()
    rng = np.random.default_rng(8)
    for _ in range(4):
        g = rng.standard_normal((prop.n_walkers, s.norb))
        po, pcs = O.cpmc_continuous_propagate(exp_h1, prop.dt, 0.3, po, g, mo, e_est, pcs, prop.n_walkers)
        pd = cprop.propagate(trial, hd, pd, g, wave)
    torch.cuda.synchronize()
    assert rel_err(to_np(pd["walkers"][0]), po["walkers"][0]) < 1e-9
    assert rel_err(to_np(pd["walkers"][1]), po["walkers"][1]) < 1e-9
    assert rel_err(to_np(pd["weights"]), po["weights"]) < 1e-9
    assert rel_err(to_np(pd["overlaps"]), po["overlaps"]) < 1e-9
    assert abs(pd["pop_control_ene_shift"].item() - pcs) < 1e-9 * max(1.0, abs(pcs))


def _neighbors(lx, ly):
    pairs = {tuple(sorted((x + lx * y, (x + 1) % lx + lx * y))) for y in range(ly) for x in range(lx)} | \
        {tuple(sorted((x + lx * y, x + lx * ((y + 1) % ly)))) for y in range(ly) for x in range(lx)}
    return tuple(p for p in sorted(pairs) if p[0] != p[1])


@pytest.mark.parametrize("lx,ly,nelec", [(4, 2, (3, 3)), (4, 4, (7, 5))], ids=["4x2", "4x4"])
def test_cpmc_nn_steps(lx, ly, nelec):
    """propagator_cpmc_nn (propagation.py:889-1230) against the oracle's fast form on
    identical uniforms: walkers, weights, overlaps, Green's functions and the shift."""
    import torch
    from cs_afqmc_gb300 import propagation
    s, trial, wave, hd, prop, pd, w0, mo = _system(lx=lx, ly=ly, nelec=nelec)
    nbr = _neighbors(lx, ly)
    nprop = propagation.propagator_cpmc_nn(dt=prop.dt, n_walkers=prop.n_walkers, precision="fp64", neighbors=nbr)
    hd["u_1"] = 1.0
    pd = nprop.init_prop_data(trial, wave, hd, init_walkers=w0)
    n = s.norb
    exp_h1 = to_np(hd["exp_h1"])
    po = O.cpmc_init(w0, mo)
    e_est = pd["e_estimate"].item()
    pcs = pd["pop_control_ene_shift"].item()
    rng = np.random.default_rng(11)
    for _ in range(3):
        uni = rng.uniform(size=(prop.n_walkers, n + 4 * len(nbr)))
        po, pcs = O.cpmc_nn_propagate(exp_h1, prop.dt, 4.0, 1.0, nbr, po, uni, mo, e_est, pcs, prop.n_walkers)
        pd = nprop.propagate(trial, hd, pd, None, wave, uniforms=uni)
    torch.cuda.synchronize()
    assert pd["_scalars"][5].item() == 0.0  # no bad neighbour pair
    assert rel_err(to_np(pd["walkers"][0]), po["walkers"][0]) < 1e-9
    assert rel_err(to_np(pd["walkers"][1]), po["walkers"][1]) < 1e-9
    assert rel_err(to_np(pd["weights"]), po["weights"]) < 1e-9
    assert rel_err(to_np(pd["overlaps"]), po["overlaps"]) < 1e-9
    assert rel_err(to_np(pd["greens"]), po["greens"]) < 1e-9
    assert abs(pd["pop_control_ene_shift"].item() - pcs) < 1e-9 * max(1.0, abs(pcs))


def test_cpmc_nn_draws_and_bad_pairs():
    """Uniforms drawn from prop_data["key"] when not given; pairs outside the lattice or of
    one site are refused on the host."""
    from cs_afqmc_gb300 import _lib, propagation
    from cs_afqmc_gb300.propagation import RngKey
    s, trial, wave, hd, prop, pd, w0, mo = _system()
    hd["u_1"] = 1.0
    nprop = propagation.propagator_cpmc_nn(dt=prop.dt, n_walkers=prop.n_walkers, precision="fp64",
                                           neighbors=_neighbors(4, 2))
    pd = nprop.init_prop_data(trial, wave, hd, init_walkers=w0)
    pd["key"] = RngKey(5)
    pd = nprop.propagate(trial, hd, pd, None, wave)
    assert np.all(np.isfinite(to_np(pd["weights"])))
    for bad in (((0, 0),), ((0, s.norb),)):
        p2 = propagation.propagator_cpmc_nn(dt=prop.dt, n_walkers=prop.n_walkers, precision="fp64", neighbors=bad)
        with pytest.raises(_lib.AfqError):
            p2.propagate(trial, hd, pd, None, wave)
