"""The benchmark's algorithmic work model (no GPU): the dense work per walker-step that the
bench line's whole-step roofline uses, against hand-counted values of the benchmark
configurations (propagation.py:67-165 per step, wavefunctions.py:529-561, 711-743 per
measurement)."""

import pytest

import bench


@pytest.mark.parametrize("w,meas_every,step_mf,meas_mf", [
    # norb 20, 5 + 5 electrons, 100 vectors (restricted walkers)
    (dict(norb=20, nelec=(5, 5), nchol=100, kind="rhf"), 5, 0.305, 0.231),
    # norb 120, 20 + 20, 600 vectors: vhs 34.56 + Taylor 11.52 + exp_h1 2.30 + force bias 5.76
    # + Green 0.64 + overlap 0.21 per step; exchange 117.1 of the 118.1 per measurement
    (dict(norb=120, nelec=(20, 20), nchol=600, kind="rhf"), 5, 55.0, 118.1),
    # norb 60, 10 + 8 electrons, 300 vectors, two slabs
    (dict(norb=60, nelec=(10, 8), nchol=300, kind="uhf"), 50, 8.90, 12.41),
])
def test_work_per_walker_step(w, meas_every, step_mf, meas_mf):
    f = bench.flops_per_walker_step(w, meas_every)
    assert f["step"] / 1e6 == pytest.approx(step_mf, abs=0.006)
    assert f["measurement"] / 1e6 == pytest.approx(meas_mf, abs=0.06)
    assert f["per_walker_step"] == pytest.approx(f["step"] + f["measurement"] / meas_every)


def test_vhs_term_dominates_the_step():
    """At norb 120 / 600 vectors the vhs contraction (4 G norb^2) is 63 % of the step."""
    w = dict(norb=120, nelec=(20, 20), nchol=600, kind="rhf")
    f = bench.flops_per_walker_step(w, 5)
    assert 4.0 * 600 * 120 * 120 / f["step"] == pytest.approx(0.628, abs=0.002)
