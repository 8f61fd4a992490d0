"""Host-side pieces on the CPU: the Frechet derivative of expm that gives d exp_h1 / d lambda,
the oracle's finite-difference derivative of the blocked energy (its convergence in h), and
the norm bookkeeping of the oracle's free-projection step, and the trial optimisation
(SCF) of the orbital-rotation derivative with its tangent."""

import numpy as np
import pytest
import scipy.linalg
import torch

from oracle import afqmc_oracle as O


def test_expm_frechet_matches_scipy():
    from cs_afqmc_gb300.propagation import expm_frechet
    rng = np.random.default_rng(1)
    for n in (1, 5, 24):
        a = rng.standard_normal((n, n)) * 0.3
        e = rng.standard_normal((n, n))
        want = scipy.linalg.expm_frechet(a, e, compute_expm=False)
        got = expm_frechet(torch.as_tensor(a), torch.as_tensor(e)).numpy()
        assert np.max(np.abs(got - want)) < 1e-12 * max(1.0, np.max(np.abs(want)))


def test_expm_frechet_is_the_derivative():
    from cs_afqmc_gb300.propagation import expm_frechet
    rng = np.random.default_rng(2)
    a = rng.standard_normal((8, 8)) * 0.05
    e = rng.standard_normal((8, 8))
    h = 1e-5
    fd = (scipy.linalg.expm(a + h * e) - scipy.linalg.expm(a - h * e)) / (2 * h)
    got = expm_frechet(torch.as_tensor(a), torch.as_tensor(e)).numpy()
    assert np.max(np.abs(got - fd)) < 1e-8


def test_expm_frechet_transpose():
    """<G, L(A, E)> = <L(A^T, G), E>: the transpose the reverse mode applies to the
    exp_h1 cotangent (A non-symmetric here, so the transpose is exercised)."""
    from cs_afqmc_gb300.propagation import expm_frechet
    rng = np.random.default_rng(4)
    a = torch.as_tensor(rng.standard_normal((7, 7)) * 0.2)
    e = torch.as_tensor(rng.standard_normal((7, 7)))
    g = torch.as_tensor(rng.standard_normal((7, 7)))
    lhs = float(torch.sum(g * expm_frechet(a, e)))
    rhs = float(torch.sum(expm_frechet(a.T.contiguous(), g) * e))
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))


def _small_system(kind="rhf", restricted=True, norb=6, nelec=(2, 2), nchol=8, nw=4, seed=5):
    from cs_afqmc_gb300 import synthetic
    s = synthetic.molecular(norb, nelec, nchol, seed=seed, kind=kind)
    rng = np.random.default_rng(seed + 100)
    trial = O.Trial(kind, norb, nelec)
    ham = {"h0": s.h0, "h1": s.h1.copy(), "chol": s.chol.copy()}
    hd = trial.build_measurement_intermediates(dict(ham), s.mo_coeff)
    dt = 0.005
    hd = O.build_propagation_intermediates(hd, s.rdm1, norb, nelec, dt, restricted)
    prop = O.Propagator(dt=dt, n_walkers=nw, n_exp_terms=6)
    if restricted:
        w = np.repeat(s.mo_coeff[None].astype(np.complex128), nw, 0)
        w = w + 0.2 * (rng.standard_normal(w.shape) + 1j * rng.standard_normal(w.shape))
    else:
        mos = [s.mo_coeff[:, : nelec[0]], s.mo_coeff[:, : nelec[1]]] if kind == "rhf" else s.mo_coeff
        w = [np.repeat(m[None].astype(np.complex128), nw, 0) for m in mos]
        w = [x + 0.2 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape)) for x in w]
    pd = O.init_prop_data(prop, trial, hd, s.mo_coeff, w)
    return s, trial, ham, prop, pd


@pytest.mark.parametrize("kind,restricted", [("rhf", True), ("uhf", False)])
def test_oracle_fd_converges(kind, restricted):
    """The Richardson-extrapolated central difference agrees with itself at h and h/4 (the
    derivative is smooth in lambda for these draws: no clamp or SR index changes)."""
    s, trial, ham, prop, pd = _small_system(kind=kind, restricted=restricted)
    samp = O.Sampler(n_prop_steps=2, n_ene_blocks=2, n_sr_blocks=1)
    rng = np.random.default_rng(3)
    fields = rng.standard_normal((1, 2, 2, prop.n_walkers, s.chol.shape[0]))
    zetas = rng.uniform(size=1)
    D = rng.standard_normal((2, s.norb, s.norb)) * 0.1
    a = O.phaseless_derivative_fd(samp, prop, trial, ham, D, s.rdm1, s.mo_coeff, pd, fields, zetas,
                                  restricted, h=1e-3)
    b = O.phaseless_derivative_fd(samp, prop, trial, ham, D, s.rdm1, s.mo_coeff, pd, fields, zetas,
                                  restricted, h=2.5e-4)
    assert abs(a[1] - b[1]) < 1e-8 * max(1.0, abs(a[1]))
    assert np.max(np.abs(a[3] - b[3])) < 1e-8 * max(1.0, np.max(np.abs(a[3])))
    # zero direction: zero derivative, values unchanged
    z = O.phaseless_derivative_fd(samp, prop, trial, ham, 0 * D, s.rdm1, s.mo_coeff, pd, fields, zetas,
                                  restricted, h=1e-3)
    assert z[1] == 0.0 and z[0] == a[0]


def test_oracle_free_projection_norm_bookkeeping():
    """After free steps, overlap(Q) * norms equals the overlap of the walkers propagated without
    any QR (the norms carry exactly what the orthonormalisation removed)."""
    s, trial, ham, prop, pd = _small_system(kind="uhf", restricted=False)
    hd = trial.build_measurement_intermediates(dict(ham), s.mo_coeff)
    hd = O.build_propagation_intermediates(hd, s.rdm1, s.norb, s.nelec, prop.dt, False)
    pd["norms"] = np.ones(prop.n_walkers, dtype=np.complex128)
    raw = [w.copy() for w in pd["walkers"]]
    rng = np.random.default_rng(9)
    for _ in range(3):
        f = rng.standard_normal((prop.n_walkers, s.chol.shape[0]))
        pd = prop.propagate_free(trial, hd, pd, f, s.mo_coeff)
        # the same step on the raw walkers, without the QR
        sdt = np.sqrt(prop.dt)
        sh = f @ hd["mf_shifts"]
        raw = O.apply_trotprop(hd, raw, f.astype(np.complex128), prop.dt, s.norb, prop.n_exp_terms)
        for i in range(2):
            c = np.exp(-sdt * sh / (2.0 * s.nelec[i])) * np.exp(prop.dt * hd["h0_prop"] / (2.0 * s.nelec[i]))
            raw[i] = c[:, None, None] * raw[i]
    want = trial.overlap(raw, s.mo_coeff)
    assert np.max(np.abs(pd["overlaps"] - want)) < 1e-10 * np.max(np.abs(want))


def _scf_system(kind, norb=8, nelec=(3, 3), nchol=12, seed=6):
    from cs_afqmc_gb300 import synthetic
    s = synthetic.molecular(norb, nelec, nchol, seed=seed, kind=kind)
    h1 = np.asarray(s.h1)
    h1 = np.stack([h1, h1]) if h1.ndim == 2 else h1
    chol3 = np.asarray(s.chol).reshape(-1, norb, norb)
    return s, h1, chol3


@pytest.mark.parametrize("kind,nelec", [("rhf", (3, 3)), ("uhf", (4, 2))])
def test_scf_optimize_value_and_tangent(kind, nelec):
    """The trial optimisation of the orbital-rotation AD variants (rhf/uhf.optimize,
    wavefunctions.py:566-600, 750-813) on the CPU: the torch iterations equal the oracle's,
    and their first-order change along dh1 equals a Richardson central difference of the
    oracle's iterations."""
    from cs_afqmc_gb300.wavefunctions import _scf
    norb = 8
    s, h1, chol3 = _scf_system(kind, norb, nelec)
    mo = s.mo_coeff
    rng = np.random.default_rng(8)
    d = rng.standard_normal((2, norb, norb)) * 0.1
    d = np.stack([(x + x.T) / 2 for x in d])
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x))  # noqa: E731
    if kind == "rhf":
        h = (h1[0] + h1[1]) / 2
        h, dh = [T((h + h.T) / 2)], [T((d[0] + d[1]) / 2)]
        dm0 = [T(2 * mo @ mo.T)]
        ne = (nelec[0],)
        ora = lambda lam: [O.rhf_optimize(h1 + lam * d, chol3, mo, nelec[0], 30)]  # noqa: E731
    else:
        h, dh = [T(h1[0]), T(h1[1])], [T(d[0]), T(d[1])]
        dm0 = [T(mo[0] @ mo[0].T), T(mo[1] @ mo[1].T)]
        ne = nelec
        ora = lambda lam: O.uhf_optimize(h1 + lam * d, chol3, mo, nelec, 30)  # noqa: E731
    mos, dmos = _scf(kind, h, T(chol3), dm0, ne, 30, dh)
    ref = ora(0.0)
    for a, b in zip(mos, ref):
        assert np.max(np.abs(a.numpy() - b)) < 1e-10
    eps = 1e-4
    d1 = [(p - m) / (2 * eps) for p, m in zip(ora(eps), ora(-eps))]
    d2 = [(p - m) / eps for p, m in zip(ora(eps / 2), ora(-eps / 2))]
    for got, a, b in zip(dmos, d1, d2):
        fd = (4 * b - a) / 3
        assert np.max(np.abs(got.numpy() - fd)) < 1e-7 * max(1.0, np.max(np.abs(fd))), np.max(np.abs(got.numpy() - fd))


def test_modified_cholesky_reconstructs_and_differentiates():
    """linalg_utils.modified_cholesky (reference linalg_utils.py:70-106) on the CPU: the
    vectors of a rank-G electron-repulsion matrix rebuild it, and the autograd gradient of a
    function of the vectors matches a central difference along a direction with the 8-fold
    symmetry of real-orbital integrals (the pivots' ties stay ties along it)."""
    from cs_afqmc_gb300.linalg_utils import modified_cholesky
    rng = np.random.default_rng(0)
    n, G = 6, 8
    L = rng.standard_normal((G, n, n))
    L = L + L.transpose(0, 2, 1)
    V = np.einsum("gij,gkl->ijkl", L, L)
    W = torch.as_tensor(rng.standard_normal((G, n * n)))

    def f(v):
        v = (v + v.permute(2, 3, 0, 1) + v.permute(1, 0, 3, 2) + v.permute(3, 2, 1, 0)) / 4
        c = modified_cholesky(v.reshape(n * n, n * n), n, G)
        return torch.sum(W * c), c

    v0 = torch.as_tensor(V).requires_grad_(True)
    val, c = f(v0)
    assert float(torch.max(torch.abs(c.T @ c - torch.as_tensor(V).reshape(n * n, n * n)).detach())) < 1e-12
    (gr,) = torch.autograd.grad(val, v0)
    T = rng.standard_normal((n,) * 4)
    T = (T + T.transpose(1, 0, 2, 3)) / 2
    T = (T + T.transpose(0, 1, 3, 2)) / 2
    T = (T + T.transpose(2, 3, 0, 1)) / 2
    h = 1e-4
    fd = (f(torch.as_tensor(V + h * T))[0].item() - f(torch.as_tensor(V - h * T))[0].item()) / (2 * h)
    assert abs(float(torch.sum(gr * torch.as_tensor(T))) - fd) < 1e-8 * max(1.0, abs(fd))
