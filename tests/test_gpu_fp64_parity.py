"""FP64 CUDA path against the FP64 oracle, through the C ABI, on identical inputs.

Tolerance: FP64 kernels reorder sums relative to NumPy/LAPACK, so results agree to
rounding: relative error <= 1e-9 on every compared array (1e-8 after several steps).
"""

import json
import os

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.golden import seed102_fixture
from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind="rhf", restricted=True, norb=12, nelec=(3, 3), nchol=30, nw=8),
    dict(kind="rhf", restricted=False, norb=10, nelec=(4, 4), nchol=17, nw=6),
    dict(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=5),
    dict(kind="rhf", restricted=True, norb=7, nelec=(3, 3), nchol=5, nw=3),   # odd tiny
    dict(kind="rhf", restricted=True, norb=40, nelec=(9, 9), nchol=70, nw=4),
    dict(kind="rhf", restricted=True, norb=120, nelec=(20, 20), nchol=200, nw=4),
    dict(kind="uhf", restricted=False, norb=60, nelec=(10, 8), nchol=90, nw=4),
]
IDS = ["rhf-r", "rhf-u", "uhf", "tiny", "rhf-40", "rhf-120", "uhf-60"]


@pytest.fixture(params=list(range(len(CASES))), ids=IDS)
def case(request):
    return Case(**CASES[request.param])


def test_measurements(case):
    w = case.gpu_walkers()
    ov = to_np(case.trial.calc_overlap(w, case.wave_data))
    fb = to_np(case.trial.calc_force_bias(w, case.ham_data, case.wave_data))
    en = to_np(case.trial.calc_energy(w, case.ham_data, case.wave_data))
    mo = case.sys.mo_coeff
    assert rel_err(ov, case.o_trial.overlap(case.walkers0, mo)) < 1e-10
    assert rel_err(fb, case.o_trial.force_bias(case.walkers0, case.o_ham, mo)) < 1e-10
    assert rel_err(en, case.o_trial.energy(case.walkers0, case.o_ham, mo)) < 1e-10


def test_one_step(case):
    rng = np.random.default_rng(3)
    fields = rng.standard_normal((case.nw, case.nchol))
    po = case.oracle_prop_data()
    po = case.o_prop.propagate(case.o_trial, case.o_ham, po, fields, case.sys.mo_coeff)
    pg = case.gpu_prop_data()
    pg = case.prop.propagate(case.trial, case.ham_data, pg, fields, case.wave_data)
    assert rel_err(to_np(pg["walkers"]) if not isinstance(pg["walkers"], list) else
                   np.concatenate([x.ravel() for x in to_np(pg["walkers"])]),
                   po["walkers"] if not isinstance(po["walkers"], list) else
                   np.concatenate([x.ravel() for x in po["walkers"]])) < 1e-10
    assert rel_err(to_np(pg["weights"]), po["weights"]) < 1e-10
    assert rel_err(to_np(pg["overlaps"]), po["overlaps"]) < 1e-10
    assert abs(pg["pop_control_ene_shift"].item() - po["pop_control_ene_shift"]) < 1e-9 * max(1, abs(po["pop_control_ene_shift"]))


def _flat(w):
    return np.concatenate([x.ravel() for x in w]) if isinstance(w, list) else w.ravel()


def test_qr_matches_lapack_convention(case):
    po = case.oracle_prop_data()
    po = case.o_prop.orthonormalize_walkers(po)
    pg = case.gpu_prop_data()
    pg = case.prop.orthonormalize_walkers(pg)
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 1e-10


def test_sr_indices_exact(case):
    rng = np.random.default_rng(9)
    wts = rng.uniform(0.2, 2.0, case.nw)
    wts[0] = 0.0
    zeta = 0.37
    po = case.oracle_prop_data()
    po["weights"] = wts.copy()
    po = case.o_prop.stochastic_reconfiguration(po, zeta)
    pg = case.gpu_prop_data()
    pg["weights"].copy_(case.torch.as_tensor(wts))
    pg = case.prop.stochastic_reconfiguration_local(pg, zeta=np.array([zeta]))
    assert np.array_equal(to_np(pg["sr_indices"]), po["sr_indices"])
    assert np.array_equal(_flat(to_np(pg["walkers"])), _flat(po["walkers"]))
    assert rel_err(to_np(pg["weights"]), po["weights"]) < 1e-14


def test_phaseless_blocks(case):
    """Two driver blocks of propagate_phaseless (3 steps x 2 energy blocks, local SR),
    then QR + global SR + e_estimate update, against the oracle's run_blocks."""
    from cs_afqmc_gb300 import driver, sampling
    nb, n_sr, n_ene, n_prop = 2, 1, 2, 3
    rng = np.random.default_rng(21)
    fields = rng.standard_normal((nb, n_sr, n_ene, n_prop, case.nw, case.nchol))
    zetas = rng.uniform(size=(nb, n_sr + 1))
    samp_o = O.Sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    po = case.oracle_prop_data()
    e_o, w_o, po = O.run_blocks(samp_o, case.o_prop, case.o_trial, case.o_ham, po,
                                case.sys.mo_coeff, lambda n: fields[n], lambda n: zetas[n], nb)
    samp = sampling.sampler(n_prop_steps=n_prop, n_ene_blocks=n_ene, n_sr_blocks=n_sr)
    pg = case.gpu_prop_data()
    e_g, w_g, pg = driver.run_blocks(samp, case.ham, case.ham_data, case.prop, pg, case.trial,
                                     case.wave_data, nb, fields=fields, zetas=zetas)
    assert rel_err(to_np(e_g), e_o) < 1e-9
    assert rel_err(to_np(w_g), w_o) < 1e-9
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 1e-8
    assert abs(pg["e_estimate"].item() - po["e_estimate"]) < 1e-9 * abs(po["e_estimate"])


def test_reference_golden_values_through_gpu():
    """The GPU path reproduces the reference's known-answer values directly
    (tests/test_wavefunctions.py:127-183 of the reference)."""
    import torch
    from cs_afqmc_gb300 import wavefunctions
    kat = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))
    fx = seed102_fixture.build()
    r = wavefunctions.rhf(10, (5, 5))
    wd = {"mo_coeff": fx["mo"]}
    hd = {"h0": fx["h0"], "rot_h1": torch.as_tensor(fx["rot_h1"]).cuda(),
          "rot_chol": torch.as_tensor(fx["rot_chol"]).cuda(), "chol": torch.as_tensor(fx["chol"]).cuda()}
    w = torch.as_tensor(fx["walker"][None], dtype=torch.complex128, device="cuda").contiguous()
    assert abs(r.calc_overlap(w, wd)[0].real.item() - kat["rhf_overlap_real"]) < 1e-12
    assert abs(r.calc_force_bias(w, hd, wd)[0].sum().real.item() - kat["rhf_force_bias_sum_real"]) < 1e-11
    assert abs(r.calc_energy(w, hd, wd)[0].real.item() - kat["rhf_energy_real"]) < 1e-10
    u = wavefunctions.uhf(10, (3, 2))
    wdu = {"mo_coeff": fx["mo_u"]}
    hdu = {"h0": fx["h0"], "rot_h1": [torch.as_tensor(x).cuda() for x in fx["rot_h1_u"]],
           "rot_chol": [torch.as_tensor(np.ascontiguousarray(x)).cuda() for x in fx["rot_chol_u"]],
           "chol": torch.as_tensor(fx["chol"]).cuda()}
    wu = [torch.as_tensor(fx["walker_up"][None], dtype=torch.complex128, device="cuda").contiguous(),
          torch.as_tensor(fx["walker_dn"][None], dtype=torch.complex128, device="cuda").contiguous()]
    assert abs(u.calc_overlap(wu, wdu)[0].real.item() - kat["uhf_overlap_real"]) < 1e-12
    assert abs(u.calc_force_bias(wu, hdu, wdu)[0].sum().real.item() - kat["uhf_force_bias_sum_real"]) < 1e-11
    assert abs(u.calc_energy(wu, hdu, wdu)[0].real.item() - kat["uhf_energy_real"]) < 1e-11


def test_rng_counter_based():
    import ctypes
    import torch
    from cs_afqmc_gb300 import _lib
    from cs_afqmc_gb300._engine import stream_ptr
    n = 1 << 20
    a = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.call("afq_fill_normal", a.data_ptr(), n, 1234, 0, stream_ptr())
    b = torch.empty(n // 2, dtype=torch.float64, device="cuda")
    _lib.call("afq_fill_normal", b.data_ptr(), n // 2, 1234, n // 2, stream_ptr())
    assert torch.equal(a[n // 2:], b)
    assert abs(a.mean().item()) < 5e-3 and abs(a.std().item() - 1) < 5e-3
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.call("afq_fill_uniform", u.data_ptr(), n, 7, 0, stream_ptr())
    assert u.min().item() >= 0.0 and u.max().item() < 1.0 and abs(u.mean().item() - 0.5) < 2e-3


def test_errors_are_loud():
    import torch
    from cs_afqmc_gb300 import _lib, wavefunctions
    case = Case(**CASES[0])
    with pytest.raises(_lib.AfqError):
        case.trial.calc_overlap(case.gpu_walkers()[:, :, :2].contiguous(), case.wave_data)
    with pytest.raises(_lib.AfqError):
        case.trial.calc_overlap(torch.zeros(3, 12, 3, dtype=torch.float32, device="cuda"), case.wave_data)
    u = wavefunctions.uhf(12, (3, 3))
    with pytest.raises(_lib.AfqError):
        u.calc_overlap(case.gpu_walkers(), {"mo_coeff": [case.sys.mo_coeff, case.sys.mo_coeff]})


FREE_CASES = [
    dict(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=5),
    dict(kind="rhf", restricted=False, norb=10, nelec=(4, 4), nchol=17, nw=6),
]


@pytest.mark.parametrize("cfg", FREE_CASES, ids=["uhf", "rhf-u"])
def test_free_projection_steps(cfg):
    """Free-projection steps (propagation.py:436-462) against the oracle: walkers, norms,
    overlaps and normed overlaps on identical fields."""
    import torch
    case = Case(**cfg)
    rng = np.random.default_rng(41)
    fields = rng.standard_normal((3, case.nw, case.nchol))
    po = case.oracle_prop_data()
    po["norms"] = np.ones(case.nw, dtype=np.complex128)
    pg = case.gpu_prop_data()
    for f in fields:
        po = case.o_prop.propagate_free(case.o_trial, case.o_ham, po, f, case.sys.mo_coeff)
        pg = case.prop.propagate_free(case.trial, case.ham_data, pg, f, case.wave_data)
    torch.cuda.synchronize()
    assert rel_err(_flat(to_np(pg["walkers"])), _flat(po["walkers"])) < 1e-9
    assert rel_err(to_np(pg["norms"]), po["norms"]) < 1e-9
    assert rel_err(to_np(pg["overlaps"]), po["overlaps"]) < 1e-9
    assert rel_err(to_np(pg["normed_overlaps"]), po["normed_overlaps"]) < 1e-9


def test_free_projection_blocks():
    """sampler.propagate_free (sampling.py:344-360): complex block energies and weights of
    3 blocks x 2 steps against the oracle."""
    from cs_afqmc_gb300 import sampling
    case = Case(kind="uhf", restricted=False, norb=11, nelec=(4, 2), nchol=23, nw=5)
    rng = np.random.default_rng(43)
    fields = rng.standard_normal((3, 2, case.nw, case.nchol))
    samp_o = O.Sampler(n_prop_steps=2)
    po = case.oracle_prop_data()
    po["norms"] = np.ones(case.nw, dtype=np.complex128)
    po, be_o, bw_o = samp_o.propagate_free(case.o_prop, case.o_trial, case.o_ham, po, case.sys.mo_coeff, fields)
    samp = sampling.sampler(n_prop_steps=2, n_blocks=3)
    pg, be, bw, _ = samp.propagate_free(case.ham, case.ham_data, case.prop, case.gpu_prop_data(), case.trial,
                                        case.wave_data, fields=fields)
    assert rel_err(to_np(be), be_o) < 1e-9
    assert rel_err(to_np(bw), bw_o) < 1e-9
    assert rel_err(to_np(pg["norms"]), po["norms"]) < 1e-9


def test_free_projection_rejects_restricted():
    case = Case(kind="rhf", restricted=True, norb=10, nelec=(3, 3), nchol=12, nw=4)
    with pytest.raises(NotImplementedError):
        case.prop.propagate_free(case.trial, case.ham_data, case.gpu_prop_data(),
                                 np.zeros((case.nw, case.nchol)), case.wave_data)
