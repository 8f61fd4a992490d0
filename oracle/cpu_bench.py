"""Timed CPU runs of the FP64 oracle: the `cpu_baseline` leg and the `--impl reference` arm
of bench.py.

Test/benchmark infrastructure only (see oracle/afqmc_oracle.py). The reference itself is
JAX, which is not installed and cannot be compiled here, so its CPU path is represented by
this NumPy restatement, laid out as the reference runs on CPU: one process per core, one
BLAS thread each, walkers split evenly between processes (config.py:77-79 and
run_afqmc.py:51-53 of the reference).
"""

from __future__ import annotations

import multiprocessing as mp
import os
import time

_STATE = {}
_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _init(norb, nocc, nchol, nw, dt, kind, seed):
    import numpy as np

    from cs_afqmc_gb300 import synthetic
    from oracle import afqmc_oracle as O

    if kind == "hubbard":  # the square periodic lattice with norb sites, real trial
        side = int(round(norb ** 0.5))
        s = synthetic.hubbard_2d(side, side, 1.0, 4.0, (nocc, nocc), real_trial=True)
        kind = "rhf"
    else:
        s = synthetic.molecular(norb, (nocc, nocc), nchol, seed=1, kind=kind)
    tr = O.Trial(kind, norb, (nocc, nocc))
    ham = {"h0": 0.0, "h1": s.h1.copy(), "chol": s.chol.copy()}
    ham = tr.build_measurement_intermediates(ham, s.mo_coeff)
    ham = O.build_propagation_intermediates(ham, s.rdm1, norb, (nocc, nocc), dt, True)
    prop = O.Propagator(dt=dt, n_walkers=nw)
    pd = O.init_prop_data(prop, tr, ham, s.mo_coeff, s.init_walkers(nw, True))
    _STATE.update(s=s, tr=tr, ham=ham, prop=prop, pd=pd, nw=nw, nchol=nchol,
                  rng=np.random.default_rng(seed + os.getpid()), O=O)


def _sample(args):
    n_steps, n_meas = args
    st = _STATE
    O, tr, ham, prop, s = st["O"], st["tr"], st["ham"], st["prop"], st["s"]
    fields = st["rng"].standard_normal((n_steps, st["nw"], st["nchol"]))
    pd = st["pd"]
    t0 = time.perf_counter()
    per = max(1, n_steps // max(1, n_meas))
    for k in range(n_steps):
        pd = prop.propagate(tr, ham, pd, fields[k], s.mo_coeff)
        if (k + 1) % per == 0:
            pd = prop.orthonormalize_walkers(pd)
            pd["overlaps"] = tr.overlap(pd["walkers"], s.mo_coeff)
            tr.energy(pd["walkers"], ham, s.mo_coeff)
    st["pd"] = pd
    return st["nw"] * n_steps, time.perf_counter() - t0


class CpuPool:
    """Spawned worker pool, one process per core (safe to create after CUDA
    initialisation); each process holds its own walkers of the same synthetic system."""

    def __init__(self, procs: int, norb: int, nocc: int, nchol: int, nw_per_proc: int,
                 dt: float, kind: str = "rhf", seed: int = 0):
        self.procs = procs
        saved = {k: os.environ.get(k) for k in _THREAD_VARS}
        os.environ.update({k: "1" for k in _THREAD_VARS})  # inherited by the spawned children
        try:
            self.pool = mp.get_context("spawn").Pool(
                procs, initializer=_init, initargs=(norb, nocc, nchol, nw_per_proc, dt, kind, seed))
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def run(self, n_steps: int, n_meas: int, timeout: float = 600.0):
        """One bounded sample per process: n_steps propagation steps of its walkers and n_meas
        QR + energy measurements. Returns (walker_steps, wall_seconds of the whole map)."""
        t0 = time.perf_counter()
        # a timeout instead of map(): a worker whose initialiser failed is respawned forever
        res = self.pool.map_async(_sample, [(n_steps, n_meas)] * self.procs, chunksize=1).get(timeout)
        return sum(r[0] for r in res), time.perf_counter() - t0

    def close(self):
        self.pool.terminate()
        self.pool.join()
