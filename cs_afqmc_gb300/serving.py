"""Serving loop: independent AFQMC jobs admitted as they arrive, on one GB300.

A request is one phaseless-AFQMC job (Hamiltonian, trial, walker count, step count). The
server keeps every admitted job's Hamiltonian, walkers, weights and operand workspace
resident in HBM and runs the jobs concurrently:

* admission by HBM footprint: a job is admitted when its measured-size footprint (the
  library's workspace size plus the Hamiltonian, walker and field buffers) fits in the
  memory budget next to the jobs already resident, and a slot is free; otherwise it waits
  in arrival order;
* continuous batching: each job owns a CUDA stream (one per server slot, created with the
  server, so that no two resident jobs share a stream) and, at admission, all of its blocks
  are enqueued on it (a job's blocks are ordered on its stream, and its draws come from a
  host-side counter, so nothing waits for the device). Blocks of different jobs overlap on
  the device, a job that arrives while others run starts as soon as it is admitted, and
  the host's set-up of a new job never leaves the device without queued work;
* CUDA graphs: after its first (eager) block a job's block - propagate_phaseless plus the
  block end - is captured once and replayed; only the field and SR draws (counter-based
  Philox, so identical to an eager run) are launched outside the graph.

Each job's result depends only on its own inputs and seed: the kernels are deterministic
and nothing is shared between jobs, so a job gives the same energies alone and in a mix
(tests/test_gpu_serving.py).

Job structure (the reference's sampler with n_ene_blocks = n_sr_blocks = 1): blocks of
`n_prop_steps` propagation steps, then QR, overlaps, local energies, block energy, local SR,
then the driver's block end (weight record, QR, global SR, e_estimate update)
(sampling.py:50-144, driver.py:250-308).
"""

from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import _lib, hamiltonian, propagation, sampling, synthetic, wavefunctions
from ._engine import device
from .propagation import RngKey


@dataclass
class JobSpec:
    job_id: int
    norb: int
    nocc: int
    nchol: int
    n_walkers: int
    n_steps: int = 100
    n_prop_steps: int = 10
    seed: int = 0
    dt: float = 0.005
    precision: str = "mixed"


@dataclass
class JobResult:
    job_id: int
    spec: JobSpec
    block_energies: np.ndarray
    block_weights: np.ndarray
    t_arrival: float
    t_admitted: float
    t_done: float
    graph: bool

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival

    @property
    def energy(self) -> float:
        return float(np.sum(self.block_energies * self.block_weights) / np.sum(self.block_weights))


def job_input(spec: JobSpec) -> synthetic.SyntheticSystem:
    """The request payload: a synthetic RHF Hamiltonian of the job's sizes (host arrays)."""
    return synthetic.molecular(spec.norb, (spec.nocc, spec.nocc), spec.nchol, seed=spec.seed, kind="rhf")


def footprint_bytes(spec: JobSpec) -> int:
    """Device bytes a job holds while resident: the context workspace (exact, from
    afq_workspace_size) plus the FP64 Hamiltonian arrays, walkers, fields and small state."""
    lib = _lib.load()
    prec = _lib.AFQ_PREC_MIXED if spec.precision == "mixed" else _lib.AFQ_PREC_FP64
    d = _lib.Dims(norb=spec.norb, n_up=spec.nocc, n_dn=spec.nocc, nchol=spec.nchol,
                  n_walkers=spec.n_walkers, walker_type=_lib.AFQ_WALKERS_RESTRICTED,
                  trial_type=_lib.AFQ_TRIAL_RHF, precision=prec, n_exp_terms=6, n_batch=1,
                  mixed_config=0, dt=spec.dt)
    ws = int(lib.afq_workspace_size(ctypes.byref(d)))
    n, o, g, nw = spec.norb, spec.nocc, spec.nchol, spec.n_walkers
    ham = 8 * (g * n * n + g * o * n + 4 * n * n + 2 * g + o * n)   # chol, rot_chol, h1/exp_h1, mf
    walkers = nw * n * o * (8 if spec.precision == "mixed" else 16)
    fields = 8 * spec.n_prop_steps * nw * g
    return ws + 2 * ham + walkers + fields + 64 * nw + (4 << 20)


class _Job:
    """One admitted job: its stream, device state and captured block graph. Construction
    sets the job up and enqueues every block and the result copy on the job's stream."""

    def __init__(self, spec: JobSpec, system: synthetic.SyntheticSystem, t_arrival: float,
                 use_graph: bool, stream: torch.cuda.Stream):
        self.spec, self.t_arrival, self.use_graph = spec, t_arrival, use_graph
        self.t_admitted = time.perf_counter()
        self.stream = stream
        self.n_blocks = max(1, spec.n_steps // spec.n_prop_steps)
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        with torch.cuda.stream(self.stream):
            self._setup(system)
            for b in range(self.n_blocks):
                self._draw()
                if b > 0 and self.use_graph and self.graph is None:
                    self._capture()
                if self.graph is not None:
                    self.graph.replay()
                else:
                    self._block_body()
                self._record(b)
            self.host_e.copy_(self.hist_e, non_blocking=True)
            self.host_w.copy_(self.hist_w, non_blocking=True)
            self.finished_event = torch.cuda.Event()
            self.finished_event.record(self.stream)

    def _setup(self, s: synthetic.SyntheticSystem):
        sp = self.spec
        self.ham = hamiltonian.hamiltonian(sp.norb)
        self.trial = wavefunctions.rhf(sp.norb, (sp.nocc, sp.nocc))
        self.wave = {"mo_coeff": s.mo_coeff, "rdm1": s.rdm1}
        hd = {"h0": s.h0, "h1": s.h1, "chol": s.chol, "ene0": 0.0}
        hd = self.ham.build_measurement_intermediates(hd, self.trial, self.wave)
        self.prop = propagation.propagator_restricted(dt=sp.dt, n_walkers=sp.n_walkers, n_exp_terms=6,
                                                      n_batch=1, precision=sp.precision)
        self.hd = self.ham.build_propagation_intermediates(hd, self.prop, self.trial, self.wave)
        self.pd = self.prop.init_prop_data(self.trial, self.wave, self.hd,
                                           init_walkers=s.init_walkers(sp.n_walkers, True))
        self.pd["key"] = RngKey(sp.seed)
        self.samp = sampling.sampler(n_prop_steps=sp.n_prop_steps, n_ene_blocks=1, n_sr_blocks=1)
        self.eng = self.prop._engine(self.trial, self.hd, self.wave, self.pd["walkers"])
        dict.__setitem__(self.pd, "_engine", self.eng)
        dev = device()
        self.fields = torch.empty(1, 1, sp.n_prop_steps, sp.n_walkers, sp.nchol, dtype=torch.float64, device=dev)
        self.zeta_local = torch.empty(1, dtype=torch.float64, device=dev)
        self.zeta_global = torch.empty(1, dtype=torch.float64, device=dev)
        self.be = torch.empty(1, dtype=torch.float64, device=dev)
        self.bw = torch.empty(1, dtype=torch.float64, device=dev)
        self.energy = torch.empty(1, dtype=torch.float64, device=dev)
        self.wsum = torch.empty(1, dtype=torch.float64, device=dev)
        self.hist_e = torch.zeros(self.n_blocks, dtype=torch.float64, device=dev)
        self.hist_w = torch.zeros(self.n_blocks, dtype=torch.float64, device=dev)
        self.host_e = torch.empty(self.n_blocks, dtype=torch.float64).pin_memory()
        self.host_w = torch.empty(self.n_blocks, dtype=torch.float64).pin_memory()

    # ---- one block --------------------------------------------------------------------
    def _draw(self):
        """Field and SR draws of the next block, in the sampler's order (fields, local SR
        uniform, then the driver's global SR uniform)."""
        key: RngKey = self.pd["key"]
        n = self.fields.numel()
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("afq_fill_normal", self.fields.data_ptr(), n, key.seed, key.take(n), st)
        _lib.call("afq_fill_uniform", self.zeta_local.data_ptr(), 1, key.seed, key.take(1), st)
        _lib.call("afq_fill_uniform", self.zeta_global.data_ptr(), 1, key.seed, key.take(1), st)

    def _block_body(self):
        """propagate_phaseless (1 SR block x 1 energy block) then the driver's block end."""
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        state = self.pd.state(self.eng)
        self._state = state  # keep the ctypes struct alive for graph replays
        _lib.call("afq_propagate_phaseless", self.eng.ctx, ctypes.byref(state), self.fields.data_ptr(),
                  self.zeta_local.data_ptr(), self.spec.n_prop_steps, 1, 1, self.be.data_ptr(),
                  self.bw.data_ptr(), self.energy.data_ptr(), st)
        _lib.call("afq_block_end", self.eng.ctx, ctypes.byref(state), self.energy.data_ptr(),
                  self.zeta_global.data_ptr(), self.wsum.data_ptr(), st)

    def _record(self, b: int):
        self.hist_e[b].copy_(self.energy[0])
        self.hist_w[b].copy_(self.wsum[0])

    def _capture(self):
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.stream(self.stream):
                g.capture_begin(capture_error_mode="thread_local")
                try:
                    self._block_body()
                finally:
                    g.capture_end()
            self.graph = g
        except Exception:  # noqa: BLE001 - a context that cannot be captured runs eagerly
            self.graph = None
            self.use_graph = False

    def result(self) -> JobResult:
        return JobResult(self.spec.job_id, self.spec, self.host_e.numpy().copy(), self.host_w.numpy().copy(),
                         self.t_arrival, self.t_admitted, time.perf_counter(), self.graph is not None)


class AfqmcServer:
    """Continuous-batching server for independent jobs on the current GPU.

    hbm_budget: bytes the resident jobs may hold (default: 85 % of the free memory at
    construction). max_active: most jobs resident at once (at most 32: one stream per slot
    from PyTorch's per-device pool of 32, taken in a row so that they are distinct)."""

    def __init__(self, hbm_budget: Optional[int] = None, max_active: int = 16, use_graphs: bool = True):
        if not torch.cuda.is_available():
            raise _lib.AfqError("the serving loop needs a CUDA device")
        if not 1 <= max_active <= 32:
            raise _lib.AfqError("max_active must be in [1, 32]")
        _lib.load()
        # a job's blocks are all enqueued at admission: resident jobs must not share a stream
        self.streams = [torch.cuda.Stream() for _ in range(max_active)]
        if len({st.cuda_stream for st in self.streams}) != max_active:
            raise _lib.AfqError("could not obtain distinct CUDA streams for the serving slots")
        free, _ = torch.cuda.mem_get_info()
        self.budget = int(hbm_budget if hbm_budget is not None else 0.85 * free)
        self.max_active = max_active
        self.use_graphs = use_graphs

    def run(self, requests: List[Tuple[float, JobSpec, synthetic.SyntheticSystem]],
            poll_s: float = 2e-4) -> Tuple[List[JobResult], float]:
        """Serve requests = [(arrival offset in s, spec, payload)], arrivals replayed in real
        time from the call. Returns (results in completion order, wall time in s)."""
        pending = sorted(requests, key=lambda r: r[0])
        queue: List[Tuple[float, JobSpec, synthetic.SyntheticSystem]] = []
        active: List[_Job] = []
        free_streams = list(self.streams)
        used = 0
        held: Dict[int, int] = {}
        results: List[JobResult] = []
        t0 = time.perf_counter()
        i = 0
        while i < len(pending) or queue or active:
            now = time.perf_counter() - t0
            while i < len(pending) and pending[i][0] <= now:
                off, spec, payload = pending[i]
                queue.append((t0 + off, spec, payload))
                i += 1
            # admission in arrival order by footprint
            while queue and len(active) < self.max_active:
                t_arr, spec, payload = queue[0]
                need = footprint_bytes(spec)
                if need > self.budget:
                    raise _lib.AfqError(f"job {spec.job_id} needs {need} B, more than the budget {self.budget} B")
                if used + need > self.budget:
                    break
                queue.pop(0)
                active.append(_Job(spec, payload, t_arr, self.use_graphs, free_streams.pop()))
                held[spec.job_id] = need
                used += need
            # completions: a job's blocks and result copy were enqueued at admission
            progressed = False
            for job in list(active):
                if job.finished_event.query():
                    progressed = True
                    active.remove(job)
                    results.append(job.result())
                    used -= held.pop(job.spec.job_id)
                    free_streams.append(job.stream)
                    del job
            if not progressed:
                time.sleep(poll_s)
        torch.cuda.synchronize()
        return results, time.perf_counter() - t0


def poisson_requests(rate: float, duration: float, seed: int = 0, norb_range=(20, 200),
                     walkers=(64, 256, 1024), n_steps: int = 100, precision: str = "mixed"):
    """The serving workload: a Poisson stream (rate jobs/s over `duration` s) of independent
    jobs, norb uniform in norb_range, nocc = norb // 6, nchol = 5 norb, walkers drawn from
    `walkers`, n_steps steps each. Payloads are generated here, before the clock starts."""
    rng = np.random.default_rng(seed)
    t, out, jid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        norb = int(rng.integers(norb_range[0], norb_range[1] + 1))
        spec = JobSpec(job_id=jid, norb=norb, nocc=max(1, norb // 6), nchol=5 * norb,
                       n_walkers=int(rng.choice(walkers)), n_steps=n_steps, seed=1000 + jid,
                       precision=precision)
        out.append((t, spec, job_input(spec)))
        jid += 1
    return out
