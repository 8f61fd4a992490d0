"""Seeded synthetic Hamiltonians and trials for the benchmark workloads.

The reference measures on molecules prepared with pyscf (ad_afqmc/pyscf_interface.py); pyscf
and its integral files are not available, so every workload here is a synthetic Hamiltonian
drawn from a seed with the shapes and value distributions below. All draws use
``numpy.random.default_rng(seed)`` in a fixed order: Cholesky vectors first, then the h1
noise, then (UHF only) the two orbital rotations.

* Cholesky vector g (g = 0..nchol-1): a real symmetric norb x norb matrix whose upper
  triangle (diagonal included) is N(0,1), mirrored, then scaled by exp(-g/25) and by
  chol_scale (default 0.5/sqrt(norb), see default_chol_scale).
* h1: symmetric N(0, 0.1^2) noise (upper triangle mirrored) + diag(linspace(-2, 2, norb)).
  h0 = 0.
* RHF trial: the lowest nocc eigenvectors of h1.
* UHF trial: for each spin, the h1 eigenvectors rotated by expm(A - A^T), A ~ N(0, 0.1^2),
  then the first n_sigma columns.
* Hubbard: 2D periodic lattice, hopping -t, L_i = sqrt(U) e_i e_i^T (dense layout), trial =
  lowest plane waves with a twist in the trial orbitals only (h1 stays real, because the
  reference symmetrises h1 with (h + h^T)/2, which would strip Peierls phases); the trial
  rdm1 is returned explicitly.

Walkers start at the trial (+0j).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Tuple, Union

import numpy as np
import scipy.linalg


@dataclass
class SyntheticSystem:
    norb: int
    nelec: Tuple[int, int]
    nchol: int
    h0: float
    h1: np.ndarray            # [2, norb, norb]
    chol: np.ndarray          # [nchol, norb*norb]
    mo_coeff: Union[np.ndarray, List[np.ndarray]]   # RHF [norb, nocc] or UHF [C_a, C_b]
    rdm1: np.ndarray          # [2, norb, norb]
    kind: str                 # "rhf" | "uhf"

    def init_walkers(self, n_walkers: int, restricted: bool):
        """Walkers at the trial, complex128."""
        if self.kind == "rhf" and restricted:
            return np.repeat(self.mo_coeff[None].astype(np.complex128), n_walkers, axis=0)
        if self.kind == "rhf":
            c = self.mo_coeff.astype(np.complex128)
            return [np.repeat(c[None, :, : self.nelec[0]], n_walkers, 0),
                    np.repeat(c[None, :, : self.nelec[1]], n_walkers, 0)]
        return [np.repeat(self.mo_coeff[0][None].astype(np.complex128), n_walkers, 0),
                np.repeat(self.mo_coeff[1][None].astype(np.complex128), n_walkers, 0)]


def _sym_from_upper(rng: np.random.Generator, n: int, scale: float = 1.0) -> np.ndarray:
    iu = np.triu_indices(n)
    m = np.zeros((n, n))
    m[iu] = rng.standard_normal(iu[0].size) * scale
    return m + np.triu(m, 1).T


def default_chol_scale(norb: int) -> float:
    """0.5/sqrt(norb). With unit-variance entries (scale 1) every L_g has spectral norm
    ~2 sqrt(norb), |sqrt(dt) sum_g x_g L_g| reaches 2-5 at dt=0.005, the 6-term Taylor
    series of exp(vhs) diverges and the phaseless projection kills every walker within the
    first block (all weights 0, energies NaN). Scaling the draws by 0.5/sqrt(norb) keeps the
    norm of each L_g at ~1 independent of norb, and runs stay stable (no walker killed at
    norb 20 and 120)."""
    return 0.5 / np.sqrt(norb)


def molecular(norb: int, nelec: Tuple[int, int], nchol: int, seed: int = 0,
              kind: str = "rhf", chol_scale: Optional[float] = None) -> SyntheticSystem:
    """chol_scale multiplies the N(0,1) Cholesky draws (default default_chol_scale(norb);
    1.0 is the unscaled reading)."""
    rng = np.random.default_rng(seed)
    scale = default_chol_scale(norb) if chol_scale is None else float(chol_scale)
    iu = np.triu_indices(norb)
    chol = np.empty((nchol, norb, norb))
    for g in range(nchol):
        m = np.zeros((norb, norb))
        m[iu] = rng.standard_normal(iu[0].size)
        m = m + np.triu(m, 1).T
        chol[g] = m * (scale * np.exp(-g / 25.0))
    h1 = _sym_from_upper(rng, norb, 0.1) + np.diag(np.linspace(-2.0, 2.0, norb))
    evals, evecs = np.linalg.eigh(h1)
    if kind == "rhf":
        assert nelec[0] == nelec[1], "RHF needs equal spin counts"
        mo = evecs[:, : nelec[0]].copy()
        rdm1 = np.stack([mo @ mo.T, mo @ mo.T])
    elif kind == "uhf":
        mos = []
        for s in range(2):
            a = rng.standard_normal((norb, norb)) * 0.1
            u = scipy.linalg.expm(a - a.T)
            mos.append((evecs @ u)[:, : nelec[s]].copy())
        mo = mos
        rdm1 = np.stack([mo[0] @ mo[0].T, mo[1] @ mo[1].T])
    else:
        raise ValueError(kind)
    return SyntheticSystem(norb, tuple(nelec), nchol, 0.0, np.stack([h1, h1]),
                           chol.reshape(nchol, norb * norb), mo, rdm1, kind)


def hubbard_2d(lx: int = 8, ly: int = 8, t: float = 1.0, u: float = 4.0,
               nelec: Tuple[int, int] = (28, 28),
               twist: Tuple[float, float] = (0.01, 0.02), real_trial: bool = False) -> SyntheticSystem:
    """Periodic lx x ly Hubbard lattice; L_i = sqrt(U) n_i; complex twisted plane-wave
    RHF trial (lowest nelec[0] of the twisted dispersion).

    real_trial=True: the trial is instead the lowest nelec[0] eigenvectors of the real
    hopping matrix plus a tiny site-dependent shift (1e-3 * linspace(-1, 1) on the diagonal)
    that splits the degenerate shell deterministically. The twist exists to make the
    free-electron determinant closed-shell; the real version does that with the shift, for
    paths that take real trials only."""
    n = lx * ly
    h1 = np.zeros((n, n))
    for x in range(lx):
        for y in range(ly):
            i = x * ly + y
            for dx, dy in ((1, 0), (0, 1)):
                j = ((x + dx) % lx) * ly + (y + dy) % ly
                h1[i, j] -= t
                h1[j, i] -= t
    chol = np.zeros((n, n, n))
    for i in range(n):
        chol[i, i, i] = np.sqrt(u)
    if real_trial:
        evals, evecs = np.linalg.eigh(h1 + np.diag(1e-3 * np.linspace(-1.0, 1.0, n)))
        mo = evecs[:, : nelec[0]].copy()
        rho = mo @ mo.T
        return SyntheticSystem(n, tuple(nelec), n, 0.0, np.stack([h1, h1]),
                               chol.reshape(n, n * n), mo, np.stack([rho, rho]), "rhf")
    ks = []
    for mx in range(lx):
        for my in range(ly):
            kx = 2 * np.pi * (mx + twist[0]) / lx
            ky = 2 * np.pi * (my + twist[1]) / ly
            ks.append((-2 * t * (np.cos(kx) + np.cos(ky)), kx, ky))
    ks.sort(key=lambda e: e[0])
    xs = np.array([x for x in range(lx) for _ in range(ly)])
    ys = np.array([y for _ in range(lx) for y in range(ly)])
    mo = np.stack([np.exp(1j * (kx * xs + ky * ys)) / np.sqrt(n)
                   for _, kx, ky in ks[: nelec[0]]], axis=1)
    rho = mo @ mo.conj().T
    return SyntheticSystem(n, tuple(nelec), n, 0.0, np.stack([h1, h1]),
                           chol.reshape(n, n * n), mo, np.stack([rho, rho]), "rhf")


# ----------------------------------------------------------------------------------------
# named workloads
# ----------------------------------------------------------------------------------------

WORKLOADS = {
    # plain phaseless AFQMC, RHF, runnable on CPU
    "rhf_norb20_nocc5_nchol100_nw50": dict(norb=20, nelec=(5, 5), nchol=100, n_walkers=50,
                                           dt=0.005, kind="rhf"),
    # single large system, precision pattern
    "rhf_norb120_nocc20_nchol600_nw1024": dict(norb=120, nelec=(20, 20), nchol=600,
                                               n_walkers=1024, dt=0.005, kind="rhf"),
    # one 256-walker chunk of the system above: the same per-launch kernel shapes with
    # n_batch=1, a quarter of the device memory (profiling case)
    "rhf_norb120_nocc20_nchol600_nw256": dict(norb=120, nelec=(20, 20), nchol=600,
                                              n_walkers=256, dt=0.005, kind="rhf"),
    # 8 x 8 periodic Hubbard lattice, U = 4, 28 + 28 electrons, diagonal Cholesky vectors
    "hubbard_8x8_u4_n28_nw2048": dict(norb=64, nelec=(28, 28), nchol=64, n_walkers=2048,
                                      dt=0.01, kind="hubbard", lx=8, ly=8, u=4.0),
    # differentiation pattern (UHF)
    "uhf_norb60_nocc10x8_nchol300_nw512": dict(norb=60, nelec=(10, 8), nchol=300,
                                               n_walkers=512, dt=0.005, kind="uhf"),
}


class FieldStream:
    """Seeded host draws of auxiliary fields N(0,1) [steps, nw, nchol] and SR uniforms,
    shared by the oracle and the device path so both consume identical inputs."""

    def __init__(self, seed: int):
        self.rng = np.random.default_rng(np.random.SeedSequence([seed, 7919]))

    def fields(self, shape) -> np.ndarray:
        return self.rng.standard_normal(shape)

    def zetas(self, n: int) -> np.ndarray:
        return self.rng.uniform(size=n)
