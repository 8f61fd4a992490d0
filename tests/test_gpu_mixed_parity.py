"""Mixed-precision CUDA path (complex64 walkers, FP16 split tensor-core contractions,
FP32 small dense algebra, FP64 log-determinants/weights/sums) against the FP64 oracle on
identical inputs, through the C ABI.

Cases up to norb 200 cover the wide propagation kernel (two 128-row M tiles, A operands
streamed from L2) and the Green's-function kernel with two orbital rows per thread.

Tolerances (relative to the largest magnitude of each compared array):
  overlaps 2e-5, force bias 1e-5, local energies 2e-5,
  one-step walkers / weights 2e-5, QR 1e-5, two driver blocks: energies 5e-5.
"""

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind="rhf", restricted=True, norb=12, nelec=(3, 3), nchol=30, nw=8),
    dict(kind="rhf", restricted=False, norb=10, nelec=(4, 4), nchol=17, nw=6),
    dict(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=5),
    dict(kind="rhf", restricted=True, norb=7, nelec=(3, 3), nchol=5, nw=3),
    dict(kind="rhf", restricted=True, norb=40, nelec=(9, 9), nchol=70, nw=14),
    dict(kind="rhf", restricted=True, norb=120, nelec=(20, 20), nchol=600, nw=16),
    dict(kind="uhf", restricted=False, norb=60, nelec=(10, 8), nchol=300, nw=12),
    # norb > 128: two 128-row M tiles, operands streamed through the wide propagation kernel
    dict(kind="rhf", restricted=True, norb=150, nelec=(25, 25), nchol=300, nw=6),
    dict(kind="uhf", restricted=False, norb=140, nelec=(12, 9), nchol=200, nw=5),
    dict(kind="rhf", restricted=True, norb=200, nelec=(32, 32), nchol=400, nw=4),
    dict(kind="rhf", restricted=True, norb=198, nelec=(33, 33), nchol=396, nw=4),  # S 33 x 33
]
IDS = ["rhf-r", "rhf-u", "uhf", "tiny", "rhf-40", "rhf-120", "uhf-60", "rhf-150", "uhf-140", "rhf-200",
       "rhf-198-o33"]


@pytest.fixture(params=list(range(len(CASES))), ids=IDS)
def case(request):
    # orthonormal walkers near the trial: the state at every measurement (the QR precedes it);
    # their overlap matrices have the conditioning of production runs. Far-from-trial walkers
    # (ill-conditioned C^T W) lose accuracy in the FP32 inverse in proportion to its condition.
    return Case(precision="mixed", orthonormal=True, perturb=0.05, **CASES[request.param])


def _flat(w):
    return np.concatenate([x.ravel() for x in w]) if isinstance(w, list) else w.ravel()


def test_measurements(case):
    w = case.gpu_walkers()
    w64 = [x.astype(np.complex64).astype(np.complex128) for x in case.walkers0] if isinstance(
        case.walkers0, list) else case.walkers0.astype(np.complex64).astype(np.complex128)
    ov = to_np(case.trial.calc_overlap(w, case.wave_data))
    fb = to_np(case.trial.calc_force_bias(w, case.ham_data, case.wave_data))
    en = to_np(case.trial.calc_energy(w, case.ham_data, case.wave_data))
    mo = case.sys.mo_coeff
    assert rel_err(ov, case.o_trial.overlap(w64, mo)) < 2e-5
    assert rel_err(fb, case.o_trial.force_bias(w64, case.o_ham, mo)) < 1e-5
    assert rel_err(en, case.o_trial.energy(w64, case.o_ham, mo)) < 2e-5


def test_one_step(case):
    rng = np.random.default_rng(3)
    fields = rng.standard_normal((case.nw, case.nchol))
    w0 = [x.astype(np.complex64).astype(np.complex128) for x in case.walkers0] if isinstance(
        case.walkers0, list) else case.walkers0.astype(np.complex64).astype(np.complex128)
    po = case.oracle_prop_data(w0)
    po = case.o_prop.propagate(case.o_trial, case.o_ham, po, fields, case.sys.mo_coeff)
    pg = case.gpu_prop_data()
    pg = case.prop.propagate(case.trial, case.ham_data, pg, fields, case.wave_data)
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 2e-5
    assert rel_err(to_np(pg["weights"]), po["weights"]) < 2e-5
    assert rel_err(to_np(pg["overlaps"]), po["overlaps"]) < 5e-5


def test_qr(case):
    w0 = [x.astype(np.complex64).astype(np.complex128) for x in case.walkers0] if isinstance(
        case.walkers0, list) else case.walkers0.astype(np.complex64).astype(np.complex128)
    po = case.oracle_prop_data(w0)
    po = case.o_prop.orthonormalize_walkers(po)
    pg = case.gpu_prop_data()
    pg = case.prop.orthonormalize_walkers(pg)
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 1e-5


def test_phaseless_blocks(case):
    from cs_afqmc_gb300 import driver, sampling
    nb, n_sr, n_ene, n_prop = 2, 1, 2, 3
    rng = np.random.default_rng(21)
    fields = rng.standard_normal((nb, n_sr, n_ene, n_prop, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, n_sr + 1))
    samp_o = O.Sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    w0 = [x.astype(np.complex64).astype(np.complex128) for x in case.walkers0] if isinstance(
        case.walkers0, list) else case.walkers0.astype(np.complex64).astype(np.complex128)
    po = case.oracle_prop_data(w0)
    e_o, w_o, po = O.run_blocks(samp_o, case.o_prop, case.o_trial, case.o_ham, po,
                                case.sys.mo_coeff, lambda n: fields[n], lambda n: zetas[n], nb)
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    pg = case.gpu_prop_data()
    e_g, w_g, pg = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, pg, case.trial,
                                     case.wave_data, nb, fields=fields, zetas=zetas)
    assert rel_err(to_np(e_g), e_o) < 5e-5
    assert rel_err(to_np(w_g), w_o) < 5e-5


@pytest.fixture(scope="module")
def wide_case():
    # the benchmark's shapes (norb 120, 20 + 20 electrons, 600 vectors) at 256 walkers: the
    # vhs and force-bias GEMMs run several 128-row M tiles per launch and the persistent
    # kernels loop over more walkers than there are SMs' worth of first assignments
    return Case(precision="mixed", orthonormal=True, perturb=0.05, kind="rhf", restricted=True, norb=120,
                nelec=(20, 20), nchol=600, nw=256)


def test_one_step_many_tiles(wide_case):
    test_one_step(wide_case)


def test_phaseless_blocks_many_tiles(wide_case):
    test_phaseless_blocks(wide_case)


@pytest.mark.parametrize("idx", [0, 2, 5], ids=["rhf-r", "uhf", "rhf-120"])
def test_one_step_legacy_taylor(idx):
    """The separate exp_h1 GEMMs around the Taylor kernel (the path before the fused
    propagation kernel, kept behind a configuration bit) against the oracle."""
    from cs_afqmc_gb300 import _lib
    case = Case(precision="mixed", orthonormal=True, perturb=0.05,
                mixed_config=_lib.MIXED_DEFAULT | _lib.MIXED_LEGACY_TAYLOR, **CASES[idx])
    test_one_step(case)


@pytest.mark.parametrize("n_batch", [1, 2])
def test_fused_matches_legacy_taylor(n_batch):
    """Fused and separate propagation on the same fields: walkers agree to the mixed path's
    own accuracy (both against the oracle at 2e-5)."""
    from cs_afqmc_gb300 import _lib
    kw = dict(kind="uhf", restricted=False, norb=40, nelec=(9, 7), nchol=70, nw=32, n_batch=n_batch)
    a = Case(precision="mixed", orthonormal=True, perturb=0.05, **kw)
    b = Case(precision="mixed", orthonormal=True, perturb=0.05, mixed_config=_lib.MIXED_DEFAULT | _lib.MIXED_LEGACY_TAYLOR,
             **kw)
    fields = np.random.default_rng(8).standard_normal((a.nw, a.nchol))
    pa = a.prop.propagate(a.trial, a.ham_data, a.gpu_prop_data(), fields, a.wave_data)
    pb = b.prop.propagate(b.trial, b.ham_data, b.gpu_prop_data(), fields, b.wave_data)
    assert rel_err(_flat(to_np(pa["walkers"])), _flat(to_np(pb["walkers"]))) < 2e-5
    assert rel_err(to_np(pa["weights"]), to_np(pb["weights"])) < 2e-5


@pytest.mark.parametrize("kw", [dict(kind="rhf", restricted=True, norb=120, nelec=(20, 20), nchol=600, nw=32),
                                dict(kind="uhf", restricted=False, norb=60, nelec=(10, 8), nchol=300, nw=24),
                                dict(kind="rhf", restricted=True, norb=40, nelec=(9, 9), nchol=70, nw=16)],
                         ids=["rhf-120", "uhf-60", "rhf-40"])
def test_symmetric_packing_is_exact(kw):
    """Symmetric Cholesky vectors (detected by the Python layer): the vhs GEMM computes V only
    for q >= 32 floor(p / 32) and the propagation kernel mirrors the rest. Each element is the
    same K sum as in the full product, so walkers and weights after two driver blocks are
    bitwise those of the full vhs GEMM (the configuration given explicitly, without the bit)."""
    from cs_afqmc_gb300 import _lib, driver, sampling
    a = Case(precision="mixed", orthonormal=True, perturb=0.05, **kw)
    b = Case(precision="mixed", orthonormal=True, perturb=0.05,
             mixed_config=_lib.MIXED_DEFAULT | _lib.MIXED_EXPLICIT, **kw)
    rng = np.random.default_rng(12)
    nb, n_prop, n_ene = 2, 3, 2
    fields = rng.standard_normal((nb, 1, n_ene, n_prop, a.nw, a.nchol))
    zetas = rng.uniform(size=(nb, 2))
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=1)
    ea, wa, pa = driver.run_blocks(samp, a.ham, a.ham_data, a.prop, a.gpu_prop_data(), a.trial, a.wave_data, nb,
                                   fields=fields, zetas=zetas)
    eb, wb, pb = driver.run_blocks(samp, b.ham, b.ham_data, b.prop, b.gpu_prop_data(), b.trial, b.wave_data, nb,
                                   fields=fields, zetas=zetas)
    assert int(pa["_engine"].dims.mixed_config) & _lib.MIXED_SYM_CHOL
    assert not int(pb["_engine"].dims.mixed_config) & _lib.MIXED_SYM_CHOL
    assert np.array_equal(_flat(to_np(pa["walkers"])), _flat(to_np(pb["walkers"])))
    assert np.array_equal(to_np(ea), to_np(eb)) and np.array_equal(to_np(wa), to_np(wb))
