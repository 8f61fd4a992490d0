"""Host-side logic of the serving loop (no GPU): footprints and the Poisson workload."""

from cs_afqmc_gb300 import serving


def test_footprint_grows_with_size():
    a = serving.footprint_bytes(serving.JobSpec(0, norb=20, nocc=3, nchol=100, n_walkers=64))
    b = serving.footprint_bytes(serving.JobSpec(1, norb=120, nocc=20, nchol=600, n_walkers=1024))
    assert 0 < a < b


def test_poisson_requests_shapes():
    reqs = serving.poisson_requests(rate=20.0, duration=1.0, seed=3, norb_range=(20, 40))
    assert len(reqs) > 5
    ts = [t for t, _, _ in reqs]
    assert ts == sorted(ts) and ts[-1] <= 1.0
    for _, s, p in reqs:
        assert 20 <= s.norb <= 40 and s.nocc == s.norb // 6 and s.nchol == 5 * s.norb
        assert s.n_walkers in (64, 256, 1024)
        assert p.chol.shape == (s.nchol, s.norb * s.norb)
