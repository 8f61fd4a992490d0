"""The oracle's CPMC restatements on the CPU: with a nearest-neighbour interaction
(propagator_cpmc_nn, propagation.py:889-1230) the fast form (overlap ratios and
Green's-function updates) agrees with the slow form (determinant ratios,
propagator_cpmc_nn_slow, 1232-1591), as the reference's test_propagate_cpmc_nn asserts
(tests/test_propagation.py:152-179); without neighbour pairs and with the uniforms
(erf(g / sqrt 2) + 1) / 2 it is the on-site CPMC step of cpmc_propagate."""

import numpy as np
import scipy.linalg
import scipy.special

from cs_afqmc_gb300 import synthetic
from oracle import afqmc_oracle as O


def _lattice(lx=4, ly=2, nelec=(3, 3), nw=5, seed=1):
    s = synthetic.hubbard_2d(lx=lx, ly=ly, u=4.0, nelec=nelec, real_trial=True)
    n = s.norb
    mo = [s.mo_coeff[:, :nelec[0]], s.mo_coeff[:, :nelec[1]]]
    rng = np.random.default_rng(seed)
    w0 = [np.repeat(m[None], nw, 0) + 0.05 * rng.standard_normal((nw, n, m.shape[1])) for m in mo]
    h = s.h1[0] if s.h1.ndim == 3 else s.h1
    e = scipy.linalg.expm(-0.01 * h / 2)
    nbr = sorted({tuple(sorted((x + lx * y, (x + 1) % lx + lx * y))) for y in range(ly) for x in range(lx)} |
                 {tuple(sorted((x + lx * y, x + lx * ((y + 1) % ly)))) for y in range(ly) for x in range(lx)})
    nbr = [p for p in nbr if p[0] != p[1]]
    return n, mo, w0, [e, e], nbr, rng


def test_cpmc_nn_fast_equals_slow():
    n, mo, w0, exp_h1, nbr, rng = _lattice()
    nw = w0[0].shape[0]
    a, b = O.cpmc_init(w0, mo), O.cpmc_init(w0, mo)
    for _ in range(3):
        uni = rng.uniform(size=(nw, n + 4 * len(nbr)))
        a, pa = O.cpmc_nn_propagate(exp_h1, 0.01, 4.0, 1.0, nbr, a, uni, mo, -5.0, -5.0, nw)
        b, pb = O.cpmc_nn_propagate(exp_h1, 0.01, 4.0, 1.0, nbr, b, uni, mo, -5.0, -5.0, nw, slow=True)
        assert abs(pa - pb) < 1e-10
    for s in range(2):
        assert np.allclose(a["walkers"][s], b["walkers"][s], rtol=1e-12, atol=0)
    assert np.allclose(a["weights"], b["weights"], rtol=1e-12, atol=0)
    assert np.allclose(a["overlaps"], b["overlaps"], rtol=1e-12, atol=0)


def test_cpmc_nn_two_entry_green_update_is_exact():
    """After one same-spin two-entry update the tracked Green's function equals the one
    recomputed from the updated walkers."""
    n, mo, w0, exp_h1, nbr, rng = _lattice()
    hs = O.cpmc_hs_constant(0.01, 1.0)
    for si, sj in ((0, 0), (1, 1), (0, 1)):
        pd = O.cpmc_init(w0, mo)
        pd = O._cpmc_pair_update(pd, hs, si, 1, sj, 2, rng.uniform(size=w0[0].shape[0]), mo, False)
        g = O.cpmc_full_green(pd["walkers"], mo)
        assert np.max(np.abs(pd["greens"] - g)) < 1e-13
        assert np.allclose(pd["overlaps"], O.cpmc_overlap(pd["walkers"], mo), rtol=1e-12, atol=0)


def test_cpmc_nn_without_pairs_is_onsite_cpmc():
    n, mo, w0, exp_h1, _, rng = _lattice()
    nw = w0[0].shape[0]
    g = rng.standard_normal((nw, n))
    uni = (scipy.special.erf(g / 2 ** 0.5) + 1) / 2
    a, pa = O.cpmc_nn_propagate(exp_h1, 0.01, 4.0, 1.0, [], O.cpmc_init(w0, mo), uni, mo, -5.0, -5.0, nw)
    b, pb = O.cpmc_propagate(exp_h1, 0.01, 4.0, O.cpmc_init(w0, mo), g, mo, -5.0, -5.0, nw)
    assert abs(pa - pb) < 1e-12
    assert np.allclose(a["weights"], b["weights"], rtol=1e-13, atol=0)
    assert np.allclose(a["greens"], b["greens"], rtol=1e-12, atol=1e-14)


def test_cpmc_nn_zero_coupling_is_onsite_step():
    """u_1 = 0: the neighbour constants are all 1, every neighbour ratio is 1 and the weights
    are unchanged, so the step equals the on-site one on the same on-site uniforms."""
    n, mo, w0, exp_h1, nbr, rng = _lattice()
    nw = w0[0].shape[0]
    g = rng.standard_normal((nw, n))
    uni = np.concatenate([(scipy.special.erf(g / 2 ** 0.5) + 1) / 2, rng.uniform(size=(nw, 4 * len(nbr)))], axis=1)
    a, pa = O.cpmc_nn_propagate(exp_h1, 0.01, 4.0, 0.0, nbr, O.cpmc_init(w0, mo), uni, mo, -5.0, -5.0, nw)
    b, pb = O.cpmc_propagate(exp_h1, 0.01, 4.0, O.cpmc_init(w0, mo), g, mo, -5.0, -5.0, nw)
    assert abs(pa - pb) < 1e-12
    assert np.allclose(a["weights"], b["weights"], rtol=1e-13, atol=0)
    for s in range(2):
        assert np.allclose(a["walkers"][s], b["walkers"][s], rtol=1e-13, atol=0)
