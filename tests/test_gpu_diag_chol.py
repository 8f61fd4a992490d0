"""Diagonal Cholesky vectors (lattice models with on-site terms, e.g. the Hubbard model with
L_i = sqrt(U) n_i): the mixed path detects them and replaces the vhs GEMM and the Taylor
products by a per-row polynomial scale of the walkers (exp of a diagonal vhs, 6 terms as
propagation.py:67-92). Checked against the FP64 oracle with the tolerances of the dense
mixed path (one step 2e-5, two driver blocks 5e-5) and against the dense mixed path forced
by an explicit configuration (both within the one-step bound of the oracle, the diagonal
one no less accurate); the device-side diagonality check leaves the status word at zero."""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind="rhf", restricted=True, norb=16, nelec=(5, 5), nchol=16, nw=8, hubbard=(4, 4, 4.0)),
    dict(kind="rhf", restricted=False, norb=16, nelec=(5, 5), nchol=16, nw=6, hubbard=(4, 4, 4.0)),
    dict(kind="rhf", restricted=True, norb=64, nelec=(28, 28), nchol=64, nw=8, hubbard=(8, 8, 4.0)),
]
IDS = ["4x4-r", "4x4-u", "8x8-r"]


@pytest.fixture(params=list(range(len(CASES))), ids=IDS)
def case(request):
    return Case(precision="mixed", orthonormal=True, perturb=0.05, dt=0.01, **CASES[request.param])


def _flat(w):
    return np.concatenate([x.ravel() for x in w]) if isinstance(w, list) else w.ravel()


def _w64(case):
    w = case.walkers0
    return [x.astype(np.complex64).astype(np.complex128) for x in w] if isinstance(w, list) else \
        w.astype(np.complex64).astype(np.complex128)


def test_diagonal_path_selected(case):
    from cs_afqmc_gb300 import _lib
    pg = case.gpu_prop_data()
    pg = case.prop.propagate(case.trial, case.ham_data, pg, np.zeros((case.nw, case.nchol)), case.wave_data)
    eng = case.prop._engine(case.trial, case.ham_data, case.wave_data, pg["walkers"])
    assert eng.dims.mixed_config & _lib.MIXED_DIAG_CHOL
    assert pg["_scalars"][_lib.AFQ_S_STATUS].item() == 0.0


def test_one_step(case):
    rng = np.random.default_rng(3)
    fields = rng.standard_normal((case.nw, case.nchol))
    po = case.oracle_prop_data(_w64(case))
    po = case.o_prop.propagate(case.o_trial, case.o_ham, po, fields, case.sys.mo_coeff)
    pg = case.gpu_prop_data()
    pg = case.prop.propagate(case.trial, case.ham_data, pg, fields, case.wave_data)
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 2e-5
    assert rel_err(to_np(pg["weights"]), po["weights"]) < 2e-5
    assert rel_err(to_np(pg["overlaps"]), po["overlaps"]) < 5e-5


def test_against_dense_mixed_path(case):
    from cs_afqmc_gb300 import _lib, propagation
    rng = np.random.default_rng(4)
    fields = rng.standard_normal((case.nw, case.nchol))
    pa = case.gpu_prop_data()
    pa = case.prop.propagate(case.trial, case.ham_data, pa, fields, case.wave_data)
    P = propagation.propagator_restricted if case.restricted else propagation.propagator_unrestricted
    dense = P(dt=case.dt, n_walkers=case.nw, n_exp_terms=6, precision="mixed",
              mixed_config=_lib.MIXED_DEFAULT | _lib.MIXED_EXPLICIT)
    pb = dense.init_prop_data(case.trial, case.wave_data, case.ham_data, init_walkers=case.gpu_walkers())
    pb = dense.propagate(case.trial, case.ham_data, pb, fields, case.wave_data)
    eng = dense._engine(case.trial, case.ham_data, case.wave_data, pb["walkers"])
    assert not (eng.dims.mixed_config & _lib.MIXED_DIAG_CHOL)
    po = case.oracle_prop_data(_w64(case))
    po = case.o_prop.propagate(case.o_trial, case.o_ham, po, fields, case.sys.mo_coeff)
    wo = _flat(po["walkers"])
    err_diag = rel_err(_flat(to_np(pa["walkers"])), wo)
    err_dense = rel_err(_flat(to_np(pb["walkers"])), wo)
    # both within the one-step bound of the mixed path, the diagonal one (an exact FP32
    # polynomial instead of split-fp16 products) no worse than the dense one
    assert err_diag < 2e-5 and err_dense < 2e-5, (err_diag, err_dense)
    assert err_diag <= err_dense * 1.5 + 1e-7, (err_diag, err_dense)
    assert rel_err(to_np(pa["weights"]), to_np(pb["weights"])) < 4e-5


def test_phaseless_blocks(case):
    from cs_afqmc_gb300 import driver, sampling
    nb, n_sr, n_ene, n_prop = 2, 1, 2, 3
    rng = np.random.default_rng(21)
    fields = rng.standard_normal((nb, n_sr, n_ene, n_prop, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, n_sr + 1))
    samp_o = O.Sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    po = case.oracle_prop_data(_w64(case))
    e_o, w_o, po = O.run_blocks(samp_o, case.o_prop, case.o_trial, case.o_ham, po,
                                case.sys.mo_coeff, lambda n: fields[n], lambda n: zetas[n], nb)
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    e_g, w_g, pg = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, case.gpu_prop_data(), case.trial,
                                     case.wave_data, nb, fields=fields, zetas=zetas)
    assert rel_err(to_np(e_g), e_o) < 5e-5
    assert rel_err(to_np(w_g), w_o) < 5e-5
