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


def _reference_nn_setup():
    """The inputs of the reference's test_propagate_cpmc_nn (tests/test_propagation.py:12-84,
    152-179): numpy's legacy RNG after seed 102 in the file's draw order (RHF h0, h1, chol;
    UHF mo_coeff [10, 5] and [10, 4]; UHF h0, h1 [2, 10, 10], chol [5, 100]), rdm1 = C C^T per
    spin, exp_h1 of the unrestricted propagator at its default dt = 0.01, walkers = the rdm1
    natural orbitals (get_init_walkers, wavefunctions.py:298-355) made real, 10 walkers,
    U = 4, u_1 = 1, ring neighbours (i, i + 1 mod 10). The JAX key's uniforms cannot be
    reproduced; both forms get the same seeded uniforms instead."""
    rs = np.random.RandomState(102)
    norb, nchol, nup, ndn, nw, dt = 10, 5, 5, 4, 10, 0.01
    rs.rand(1), rs.rand(norb, norb), rs.rand(nchol, norb * norb)  # the RHF part of the file
    mo = [rs.rand(norb, nup), rs.rand(norb, ndn)]
    h0 = rs.rand(1)[0]
    h1 = rs.rand(2, norb, norb)
    chol = rs.rand(nchol, norb * norb)
    rdm1 = np.array([mo[0] @ mo[0].T, mo[1] @ mo[1].T])
    ham = O.build_propagation_intermediates({"h0": h0, "h1": h1, "chol": chol}, rdm1, norb, (nup, ndn), dt,
                                            restricted=False)
    nat = [np.linalg.eigh(rdm1[s])[1][:, ::-1][:, :n] for s, n in ((0, nup), (1, ndn))]
    w0 = [np.repeat(x[None], nw, 0) for x in nat]
    nbr = [(i, (i + 1) % norb) for i in range(norb)]
    return norb, mo, w0, list(ham["exp_h1"]), nbr, nw, dt


def test_cpmc_nn_literal_update_on_the_references_own_setup_is_vacuous():
    """On the reference's own test setup (random positive h1 and trial orbitals) every
    walker's weight is zero after the first step in all three forms - exact, literal and
    slow - so that test's np.allclose(fast, slow) checks cannot tell the two readings of the
    update apart: they compare zero weights and identical walkers."""
    norb, mo, w0, exp_h1, nbr, nw, dt = _reference_nn_setup()
    uni = np.random.default_rng(7).uniform(size=(nw, norb + 4 * len(nbr)))
    run = {}
    with np.errstate(divide="ignore"):
        for name, kw in (("exact", {}), ("literal", {"literal": True}), ("slow", {"slow": True})):
            run[name], _ = O.cpmc_nn_propagate(exp_h1, dt, 4.0, 1.0, nbr, O.cpmc_init(w0, mo), uni, mo, -5.0,
                                               -5.0, nw, **kw)
    for name in ("exact", "literal", "slow"):
        assert np.all(run[name]["weights"] == 0.0), name
    for name in ("exact", "literal"):
        assert np.allclose(run["slow"]["overlaps"], run[name]["overlaps"])
        for s in range(2):
            assert np.allclose(run["slow"]["walkers"][s], run[name]["walkers"][s])


def test_cpmc_nn_literal_update_fails_fast_equals_slow():
    """On a lattice where walkers survive (4 x 2, U = 4, u_1 = 1, 3 steps), the reference's
    check np.allclose(fast, slow) (tests/test_propagation.py:174-179) passes for the exact
    rank-two update and fails for the update read literally (wavefunctions.py:916-945, the
    second add built from the once-updated Green's function): its weights leave the slow
    form's by ~1e-3 relative within a step. This is why the kernels implement the exact
    update."""
    n, mo, w0, exp_h1, nbr, rng = _lattice()
    nw = w0[0].shape[0]
    run = {k: O.cpmc_init(w0, mo) for k in ("exact", "literal", "slow")}
    for _ in range(3):
        uni = rng.uniform(size=(nw, n + 4 * len(nbr)))
        for name, kw in (("exact", {}), ("literal", {"literal": True}), ("slow", {"slow": True})):
            run[name], _ = O.cpmc_nn_propagate(exp_h1, 0.01, 4.0, 1.0, nbr, run[name], uni, mo, -5.0, -5.0, nw,
                                               **kw)
        sl, ex, li = run["slow"], run["exact"], run["literal"]
        assert np.allclose(sl["weights"], ex["weights"]) and np.allclose(sl["overlaps"], ex["overlaps"])
        assert all(np.allclose(sl["walkers"][s], ex["walkers"][s]) for s in range(2))
        assert not np.allclose(sl["weights"], li["weights"])
        assert np.max(np.abs(li["weights"] - sl["weights"])) > 1e-4 * np.max(np.abs(sl["weights"]))
