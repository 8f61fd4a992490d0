"""Serving loop: a job's result is the same alone and in a mix of concurrent jobs, and the
same with and without CUDA-graph replay (tolerance: bitwise; the kernels are deterministic
and jobs share nothing)."""

import numpy as np
import pytest

from cs_afqmc_gb300 import serving

pytestmark = pytest.mark.gpu


def _specs(precision):
    sizes = [(20, 3, 64), (30, 5, 64), (42, 7, 128)]
    return [serving.JobSpec(job_id=i, norb=n, nocc=o, nchol=5 * n, n_walkers=nw, n_steps=20,
                            n_prop_steps=5, seed=50 + i, precision=precision)
            for i, (n, o, nw) in enumerate(sizes)]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_alone_equals_mix(precision):
    specs = _specs(precision)
    payloads = [serving.job_input(s) for s in specs]
    srv = serving.AfqmcServer(max_active=8)
    alone = {}
    for s, p in zip(specs, payloads):
        res, _ = srv.run([(0.0, s, p)])
        alone[s.job_id] = res[0]
    mix, _ = srv.run([(0.0, s, p) for s, p in zip(specs, payloads)])
    assert len(mix) == len(specs)
    for r in mix:
        a = alone[r.job_id]
        assert np.array_equal(r.block_energies, a.block_energies), r.job_id
        assert np.array_equal(r.block_weights, a.block_weights), r.job_id
        assert np.all(np.isfinite(r.block_energies))


def test_graph_replay_equals_eager():
    spec = _specs("mixed")[1]
    payload = serving.job_input(spec)
    g, _ = serving.AfqmcServer(use_graphs=True).run([(0.0, spec, payload)])
    e, _ = serving.AfqmcServer(use_graphs=False).run([(0.0, spec, payload)])
    assert np.array_equal(g[0].block_energies, e[0].block_energies)
    assert g[0].graph and not e[0].graph


def test_admission_respects_budget():
    """With a budget equal to the largest job's footprint, jobs resident at the same time
    never hold more than the budget together, and the largest job shares the device with no
    other job: it is admitted only after the jobs before it completed."""
    specs = _specs("mixed")
    payloads = [serving.job_input(s) for s in specs]
    needs = {s.job_id: serving.footprint_bytes(s) for s in specs}
    budget = max(needs.values())
    srv = serving.AfqmcServer(hbm_budget=budget)
    res, _ = srv.run([(0.0, s, p) for s, p in zip(specs, payloads)])
    assert sorted(r.job_id for r in res) == [0, 1, 2]

    def overlap(a, b):
        return a.t_admitted < b.t_done and b.t_admitted < a.t_done

    for i, a in enumerate(res):
        for b in res[i + 1:]:
            if overlap(a, b):
                assert needs[a.job_id] + needs[b.job_id] <= budget, (a.job_id, b.job_id)
    big = max(res, key=lambda r: needs[r.job_id])
    for r in res:
        if r.job_id != big.job_id:
            assert not overlap(r, big), (r.job_id, big.job_id)
            if r.job_id < big.job_id:  # arrived earlier (same arrival time, queue order)
                assert big.t_admitted >= r.t_done
