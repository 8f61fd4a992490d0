"""Trial wave functions with the reference's measurement API, evaluated by GB300 kernels.

Mirrors ad_afqmc/wavefunctions.py: ``rhf`` (453-635) and ``uhf`` (638-844) with
``calc_overlap``, ``calc_force_bias``, ``calc_energy`` dispatched on the walker container
(one array = restricted walkers, a 2-list = unrestricted walkers, wavefunctions.py:45-241),
``get_rdm1``, ``get_init_walkers`` and ``_build_measurement_intermediates``.

Walkers are CUDA tensors. Their dtype selects the arithmetic: complex128 runs the FP64
kernels, complex64 runs the mixed-precision (BF16 tensor-core) kernels. Results are
complex128 CUDA tensors, as the reference returns complex arrays.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Any, List, Sequence, Tuple

import numpy as np
import torch

from . import _engine, _lib
from ._engine import as_dev, device, stream_ptr


def _out(shape) -> torch.Tensor:
    return torch.empty(shape, dtype=torch.complex128, device=device())


@dataclass
class wave_function:
    norb: int
    nelec: Tuple[int, int]
    n_batch: int = 1
    kind = "base"

    # ---- measurements ---------------------------------------------------------------
    def calc_overlap(self, walkers, wave_data: dict) -> torch.Tensor:
        """<psi_T|walker> per walker (wavefunctions.py:45-96)."""
        eng = _engine.engine_for(self, None, wave_data, walkers)
        wu, wd = eng.walkers(walkers)
        out = _out(eng.nw)
        _lib.call("afq_calc_overlap", eng.ctx, wu, wd, out.data_ptr(), stream_ptr())
        return out

    def calc_force_bias(self, walkers, ham_data: dict, wave_data: dict) -> torch.Tensor:
        """<psi_T|L_g|walker>/<psi_T|walker>, [nw, nchol] (wavefunctions.py:111-165)."""
        eng = _engine.engine_for(self, ham_data, wave_data, walkers)
        wu, wd = eng.walkers(walkers)
        out = _out((eng.nw, eng.nchol))
        _lib.call("afq_calc_force_bias", eng.ctx, wu, wd, out.data_ptr(), stream_ptr())
        return out

    def calc_energy(self, walkers, ham_data: dict, wave_data: dict) -> torch.Tensor:
        """Mixed local energy per walker (wavefunctions.py:186-241)."""
        eng = _engine.engine_for(self, ham_data, wave_data, walkers)
        wu, wd = eng.walkers(walkers)
        out = _out(eng.nw)
        _lib.call("afq_calc_energy", eng.ctx, wu, wd, out.data_ptr(), stream_ptr())
        return out

    # ---- trial data -----------------------------------------------------------------
    def get_rdm1(self, wave_data: dict) -> torch.Tensor:
        """wave_data["rdm1"] if present, else the trial's own (wavefunctions.py:254-270)."""
        if "rdm1" in wave_data:
            return as_dev(wave_data["rdm1"])
        return self._calc_rdm1(wave_data)

    def _calc_rdm1(self, wave_data: dict) -> torch.Tensor:
        raise NotImplementedError(
            "One-body spin RDM not found in wave_data and not implemented for this trial.")

    def get_init_walkers(self, wave_data: dict, n_walkers: int, restricted: bool = False,
                         dtype=torch.complex128):
        """Walkers from the natural orbitals of rdm1 (wavefunctions.py:298-355). The
        equal-spin restricted case and the unrestricted case are supported."""
        rdm1 = self.get_rdm1(wave_data).cpu().numpy()
        nat_up = np.linalg.eigh(rdm1[0])[1][:, ::-1][:, : self.nelec[0]]
        nat_dn = np.linalg.eigh(rdm1[1])[1][:, ::-1][:, : self.nelec[1]]
        dev = device()
        if restricted:
            if self.nelec[0] != self.nelec[1]:
                raise NotImplementedError("restricted walkers need equal spin counts here")
            det_overlap = np.linalg.det(nat_up.T @ nat_dn)
            if abs(det_overlap) <= 1e-3:
                raise ValueError("Cannot find a set of RHF orbitals with good trial overlap.")
            w = torch.as_tensor(np.ascontiguousarray(nat_up), dtype=dtype, device=dev)
            return w.unsqueeze(0).repeat(n_walkers, 1, 1).contiguous()
        return [torch.as_tensor(np.ascontiguousarray(nat_up), dtype=dtype, device=dev)
                .unsqueeze(0).repeat(n_walkers, 1, 1).contiguous(),
                torch.as_tensor(np.ascontiguousarray(nat_dn), dtype=dtype, device=dev)
                .unsqueeze(0).repeat(n_walkers, 1, 1).contiguous()]

    def optimize(self, ham_data: dict, wave_data: dict) -> dict:
        return wave_data

    def __hash__(self) -> int:
        return hash((self.kind, self.norb, tuple(self.nelec), self.n_batch))


def _sym(h1: torch.Tensor) -> torch.Tensor:
    return torch.stack([(h1[0] + h1[0].T) / 2.0, (h1[1] + h1[1].T) / 2.0])


def _eigh_fixed_sign(f: torch.Tensor, df: Optional[torch.Tensor] = None):
    """eigh with every eigenvector's first largest-magnitude component made non-negative
    (wavefunctions.py:582-586, 788-792), and with df the eigenvectors' first-order change
    dV = V (F o V^T df V), F_ij = 1 / (e_j - e_i) off the diagonal (distinct eigenvalues)."""
    e, v = torch.linalg.eigh(f)
    n = v.shape[1]
    ar = torch.arange(n, device=v.device)
    idx = torch.argmax(torch.abs(v), dim=0)
    v = v * torch.where(v[idx, ar] < 0, -1.0, 1.0).to(v.dtype)[None, :]
    if df is None:
        return e, v, None
    gap = e[None, :] - e[:, None]
    off = ~torch.eye(n, dtype=torch.bool, device=v.device)
    inv = torch.where(off, 1.0 / torch.where(off, gap, torch.ones_like(gap)), torch.zeros_like(gap))
    return e, v, v @ (inv * (v.T @ df @ v))


def _jk(chol3: torch.Tensor, dm: torch.Tensor):
    """Coulomb and exchange matrices of a density matrix (wavefunctions.py:577-580)."""
    f = torch.einsum("gij,ik->gjk", chol3, dm)
    c = torch.einsum("gii->g", f)
    return torch.einsum("g,gij->ij", c, chol3), torch.einsum("glj,gjk->lk", f, chol3)


def _scf(kind: str, h: list, chol3: torch.Tensor, dm0: list, nelec, n_iter: int, dh: Optional[list] = None):
    """The fixed-point iterations of rhf.optimize (wavefunctions.py:566-600; h = [(h_a + h_b)/2],
    fock = h + J - K/2, occupation 2) and uhf.optimize (750-813; fock_s = h_s + J_up + J_dn -
    K_s, occupation 1), with the first-order change along dh when given. Returns the lowest
    nelec eigenvectors of the last Fock matrix per spin, and their changes."""
    nsp = 1 if kind == "rhf" else 2
    occf = 2.0 if kind == "rhf" else 1.0
    dm = list(dm0)
    ddm = [torch.zeros_like(x) for x in dm] if dh is not None else None
    v = dv = None
    for _ in range(n_iter):
        jk = [_jk(chol3, dm[s]) for s in range(nsp)]
        djk = [_jk(chol3, ddm[s]) for s in range(nsp)] if dh is not None else None
        vj = sum(x[0] for x in jk)
        dvj = sum(x[0] for x in djk) if dh is not None else None
        v, dv, ndm, nddm = [], [], [], []
        for s in range(nsp):
            kfac = 0.5 if kind == "rhf" else 1.0
            fock = h[s] + vj - kfac * jk[s][1]
            dfock = dh[s] + dvj - kfac * djk[s][1] if dh is not None else None
            e, vs, dvs = _eigh_fixed_sign(fock, dfock)
            o = torch.argsort(e)[: nelec[s]]
            occ = vs[:, o]
            ndm.append(occf * occ @ occ.T)
            if dh is not None:
                docc = dvs[:, o]
                nddm.append(occf * (docc @ occ.T + occ @ docc.T))
            v.append(vs)
            dv.append(dvs)
        dm, ddm = ndm, (nddm if dh is not None else None)
    mos = [v[s][:, : nelec[s]].contiguous() for s in range(nsp)]
    dmos = [dv[s][:, : nelec[s]].contiguous() for s in range(nsp)] if dh is not None else None
    return mos, dmos


@dataclass
class rhf(wave_function):
    """Restricted Hartree-Fock trial; wave_data["mo_coeff"] is [norb, nocc], real
    (wavefunctions.py:453-635)."""

    norb: int
    nelec: Tuple[int, int]
    n_opt_iter: int = 30
    n_batch: int = 1
    kind = "rhf"

    def __post_init__(self):
        assert self.nelec[0] == self.nelec[1], "RHF requires equal number of up and down electrons."

    def _calc_rdm1(self, wave_data: dict) -> torch.Tensor:
        # mo @ mo.T without conjugation, as wavefunctions.py:563-565
        mo = as_dev(wave_data["mo_coeff"])
        return torch.stack([mo @ mo.T, mo @ mo.T])

    def _build_measurement_intermediates(self, ham_data: dict, wave_data: dict) -> dict:
        """h1 <- (h1 + h1^T)/2 per spin; rot_h1 = C^H (h1_a + h1_b)/2; rot_chol_g = C^H L_g
        (wavefunctions.py:602-619)."""
        mo = as_dev(wave_data["mo_coeff"])
        h1 = _sym(as_dev(ham_data["h1"]))
        ham_data["h1"] = h1
        ham_data["rot_h1"] = (mo.T @ ((h1[0] + h1[1]) / 2.0)).contiguous()
        chol = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        ham_data["rot_chol"] = torch.einsum("pi,gij->gpj", mo.T, chol).contiguous()
        return ham_data

    def rot_h1_tangent(self, dh1, wave_data: dict) -> torch.Tensor:
        """d rot_h1 / d lambda for h1 -> h1 + lambda dh1 (dh1 symmetrised per spin)."""
        mo = as_dev(wave_data["mo_coeff"])
        dh1 = as_dev(dh1)
        return (mo.T @ ((dh1[0] + dh1[1]) / 2.0)).contiguous()

    def rot_h1_cotangent(self, grot, wave_data: dict) -> torch.Tensor:
        """Transpose of rot_h1_tangent: d energy / d h1 per spin [2, norb, norb] (before the
        symmetrisation) from d energy / d rot_h1 [nocc, norb]."""
        mo = as_dev(wave_data["mo_coeff"])
        g = mo @ as_dev(grot) / 2.0
        return torch.stack([g, g])

    def optimize(self, ham_data: dict, wave_data: dict) -> dict:
        """rhf.optimize (wavefunctions.py:566-600): n_opt_iter restricted SCF iterations from
        dm = 2 C C^T with ham_data["h1"] (spin average, symmetrised) and ham_data["chol"].
        Returns a copy of wave_data with the new mo_coeff (the other keys, rdm1 included,
        unchanged)."""
        return self.optimize_tangent(ham_data, wave_data, None)[0]

    def optimize_tangent(self, ham_data: dict, wave_data: dict, dh1):
        """(optimize(ham_data, wave_data), d mo_coeff) for h1 -> h1 + lambda dh1
        ([2, norb, norb]; None: value only)."""
        h1 = as_dev(ham_data["h1"])
        h = (h1[0] + h1[1]) / 2.0
        h = (h + h.T) / 2.0
        dh = None
        if dh1 is not None:
            d = as_dev(dh1)
            d = (d[0] + d[1]) / 2.0
            dh = [(d + d.T) / 2.0]
        chol3 = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        mo = as_dev(wave_data["mo_coeff"])
        mos, dmos = _scf("rhf", [h], chol3, [2.0 * mo @ mo.T], (self.nelec[0],), self.n_opt_iter, dh)
        out = dict(wave_data)
        out["mo_coeff"] = mos[0]
        return out, (dmos[0] if dmos is not None else None)

    def rotation_tangents(self, ham_data: dict, wave_data: dict, dmo, dh1):
        """d rot_h1 and d rot_chol for a trial tangent dmo and dh1: rot_h1 = C^T (h_a + h_b)/2
        and rot_chol_g = C^T L_g of the measurement intermediates (wavefunctions.py:602-619)."""
        mo, dmo, dh1 = as_dev(wave_data["mo_coeff"]), as_dev(dmo), as_dev(dh1)
        h1 = _sym(as_dev(ham_data["h1"]))
        drot = dmo.T @ ((h1[0] + h1[1]) / 2.0) + mo.T @ ((dh1[0] + dh1[1]) / 2.0)
        chol = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        return drot.contiguous(), torch.einsum("pi,gij->gpj", dmo.T, chol).contiguous()

    def __hash__(self) -> int:
        return super().__hash__()


@dataclass
class uhf(wave_function):
    """Unrestricted Hartree-Fock trial; wave_data["mo_coeff"] = [C_a [norb, n_a],
    C_b [norb, n_b]], real (wavefunctions.py:638-844)."""

    norb: int
    nelec: Tuple[int, int]
    n_opt_iter: int = 30
    n_batch: int = 1
    kind = "uhf"

    def _calc_rdm1(self, wave_data: dict) -> torch.Tensor:
        mo = wave_data["mo_coeff"]
        a, b = as_dev(mo[0]), as_dev(mo[1])
        return torch.stack([a @ a.T, b @ b.T])

    def _build_measurement_intermediates(self, ham_data: dict, wave_data: dict) -> dict:
        """(wavefunctions.py:817-841)."""
        mo = wave_data["mo_coeff"]
        a, b = as_dev(mo[0]), as_dev(mo[1])
        h1 = _sym(as_dev(ham_data["h1"]))
        ham_data["h1"] = h1
        ham_data["rot_h1"] = [(a.T @ h1[0]).contiguous(), (b.T @ h1[1]).contiguous()]
        chol = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        ham_data["rot_chol"] = [torch.einsum("pi,gij->gpj", a.T, chol).contiguous(),
                                torch.einsum("pi,gij->gpj", b.T, chol).contiguous()]
        return ham_data

    def rot_h1_tangent(self, dh1, wave_data: dict) -> list:
        """d rot_h1 / d lambda per spin for h1 -> h1 + lambda dh1 (dh1 symmetrised per spin)."""
        mo = wave_data["mo_coeff"]
        a, b = as_dev(mo[0]), as_dev(mo[1])
        dh1 = as_dev(dh1)
        return [(a.T @ dh1[0]).contiguous(), (b.T @ dh1[1]).contiguous()]

    def rot_h1_cotangent(self, grot, wave_data: dict) -> torch.Tensor:
        """Transpose of rot_h1_tangent: [2, norb, norb] from the per-spin d energy / d rot_h1."""
        mo = wave_data["mo_coeff"]
        a, b = as_dev(mo[0]), as_dev(mo[1])
        return torch.stack([a @ as_dev(grot[0]), b @ as_dev(grot[1])])

    def optimize(self, ham_data: dict, wave_data: dict) -> dict:
        """uhf.optimize (wavefunctions.py:750-813): n_opt_iter unrestricted SCF iterations
        from the trial's own density matrices. Returns a copy of wave_data with the new
        mo_coeff (the other keys, rdm1 included, unchanged)."""
        return self.optimize_tangent(ham_data, wave_data, None)[0]

    def optimize_tangent(self, ham_data: dict, wave_data: dict, dh1):
        """(optimize(ham_data, wave_data), [d C_a, d C_b]) for h1 -> h1 + lambda dh1."""
        h1 = _sym(as_dev(ham_data["h1"]))
        dh = None if dh1 is None else list(_sym(as_dev(dh1)))
        chol3 = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        mo = wave_data["mo_coeff"]
        a, b = as_dev(mo[0]), as_dev(mo[1])
        mos, dmos = _scf("uhf", [h1[0], h1[1]], chol3, [a @ a.T, b @ b.T], self.nelec, self.n_opt_iter, dh)
        out = dict(wave_data)
        out["mo_coeff"] = mos
        return out, dmos

    def rotation_tangents(self, ham_data: dict, wave_data: dict, dmo, dh1):
        """([d rot_h1_a, d rot_h1_b], [d rot_chol_a, d rot_chol_b]) (wavefunctions.py:817-841)."""
        mo, dh1 = wave_data["mo_coeff"], _sym(as_dev(dh1))
        h1 = _sym(as_dev(ham_data["h1"]))
        chol = as_dev(ham_data["chol"]).reshape(-1, self.norb, self.norb)
        drot, drc = [], []
        for s in range(2):
            c, dc = as_dev(mo[s]), as_dev(dmo[s])
            drot.append((dc.T @ h1[s] + c.T @ dh1[s]).contiguous())
            drc.append(torch.einsum("pi,gij->gpj", dc.T, chol).contiguous())
        return drot, drc

    def __hash__(self) -> int:
        return super().__hash__()


@dataclass
class uhf_cpmc(uhf):
    """UHF trial of the CPMC propagator (wavefunctions.py:848-955): real walkers and full
    Green's functions G_s = (W_s (C_s^T W_s)^-1 C_s^T)^T."""

    kind = "uhf"

    def calc_full_green_vmap(self, walkers, wave_data: dict) -> torch.Tensor:
        """[nw, 2, norb, norb] (wavefunctions.py:894-914)."""
        return cpmc_overlap_green(self, walkers, wave_data)[1]

    def __hash__(self) -> int:
        return super().__hash__()


def cpmc_overlap_green(trial, walkers, wave_data: dict):
    """(overlaps [nw] float64, greens [nw, 2, norb, norb] float64) of real walkers
    ([nw, norb, n_up], [nw, norb, n_dn]) for a real UHF trial, on the device."""
    wu = as_dev(walkers[0]).contiguous()
    wd = as_dev(walkers[1]).contiguous()
    mo = wave_data["mo_coeff"]
    cu, cd = as_dev(mo[0]).contiguous(), as_dev(mo[1]).contiguous()
    nw, norb = int(wu.shape[0]), trial.norb
    ovl = torch.empty(nw, dtype=torch.float64, device=device())
    greens = torch.empty(nw, 2, norb, norb, dtype=torch.float64, device=device())
    _lib.call("afq_cpmc_init", norb, trial.nelec[0], trial.nelec[1], nw, cu.data_ptr(), cd.data_ptr(),
              wu.data_ptr(), wd.data_ptr(), ovl.data_ptr(), greens.data_ptr(), stream_ptr())
    return ovl, greens
