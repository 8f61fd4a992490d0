"""Device context management: turns the reference-style dicts (ham_data, wave_data) into an
afq_ctx of the C ABI, with device-resident copies of every array it points to.

An engine is cached inside ham_data (or wave_data for overlap-only use) under a private
key, keyed by everything the context depends on. Torch provides the device memory and the
stream; all arithmetic happens in libafqmc_gb300.so.
"""

from __future__ import annotations

import ctypes
import math
from typing import Any, Optional, Sequence

import numpy as np
import torch

from . import _lib

_CACHE_KEY = "_afq_engines"

PRECISIONS = {"fp64": _lib.AFQ_PREC_FP64, "mixed": _lib.AFQ_PREC_MIXED}


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise _lib.AfqError("no CUDA device: the AFQMC kernels run on the GPU only")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def as_dev(x: Any, dtype: torch.dtype = torch.float64) -> torch.Tensor:
    """Contiguous device tensor of `dtype` (numpy arrays, lists and tensors accepted)."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if t.is_complex() and not dtype.is_complex:
        if torch.any(t.imag != 0):
            raise _lib.AfqError("complex input where a real array is required (complex trials "
                                "are not supported by this build)")
        t = t.real
    return t.to(device=device(), dtype=dtype).contiguous()


def walker_precision(walkers) -> int:
    w = walkers[0] if isinstance(walkers, (list, tuple)) else walkers
    if not isinstance(w, torch.Tensor) or not w.is_cuda:
        raise _lib.AfqError("walkers must be CUDA tensors")
    if w.dtype == torch.complex128:
        return _lib.AFQ_PREC_FP64
    if w.dtype == torch.complex64:
        return _lib.AFQ_PREC_MIXED
    raise _lib.AfqError(f"walkers must be complex128 (fp64) or complex64 (mixed), got {w.dtype}")


def walker_ptrs(walkers, restricted: bool, nw: int, norb: int, nelec) -> tuple:
    if restricted:
        if isinstance(walkers, (list, tuple)):
            raise _lib.AfqError("restricted propagator/trial call got a walker list")
        w = walkers
        if tuple(w.shape) != (nw, norb, max(nelec)) or not w.is_contiguous():
            raise _lib.AfqError(f"restricted walkers must be contiguous [{nw},{norb},{max(nelec)}], got {tuple(w.shape)}")
        return w.data_ptr(), None
    if not isinstance(walkers, (list, tuple)) or len(walkers) != 2:
        raise NotImplementedError("Walker type not supported")
    for s, w in enumerate(walkers):
        if tuple(w.shape) != (nw, norb, nelec[s]) or not w.is_contiguous():
            raise _lib.AfqError(f"walker slab {s} must be contiguous [{nw},{norb},{nelec[s]}], got {tuple(w.shape)}")
    if walkers[0].dtype != walkers[1].dtype:
        raise _lib.AfqError("walker slabs must share a dtype")
    return walkers[0].data_ptr(), walkers[1].data_ptr()


class Engine:
    """Owns one afq_ctx, its workspace and the device arrays it points to."""

    def __init__(self, *, norb: int, nelec, nchol: int, n_walkers: int, restricted: bool,
                 uhf: bool, precision: int, dt: float, n_exp_terms: int, n_batch: int,
                 arrays: dict, h0: float, h0_prop: complex, mixed_config: int = 0):
        self.lib = _lib.load()
        self.norb, self.nelec, self.nchol, self.nw = norb, tuple(nelec), nchol, n_walkers
        self.restricted, self.uhf, self.precision = restricted, uhf, precision
        self.arrays = arrays  # keeps every pointed-to tensor alive
        d = _lib.Dims(norb=norb, n_up=nelec[0], n_dn=nelec[1], nchol=nchol, n_walkers=n_walkers,
                      walker_type=_lib.AFQ_WALKERS_RESTRICTED if restricted else _lib.AFQ_WALKERS_UNRESTRICTED,
                      trial_type=_lib.AFQ_TRIAL_UHF if uhf else _lib.AFQ_TRIAL_RHF,
                      precision=precision, n_exp_terms=n_exp_terms, n_batch=n_batch,
                      mixed_config=int(mixed_config), dt=dt)
        self.dims = d
        nbytes = self.lib.afq_workspace_size(ctypes.byref(d))
        if nbytes == 0:
            raise _lib.AfqError("afq_workspace_size: " + self.lib.afq_last_error().decode())
        self.workspace = torch.empty(nbytes + 256, dtype=torch.uint8, device=device())
        off = (-self.workspace.data_ptr()) % 256
        a = arrays
        h = _lib.Hamiltonian(
            h0=float(h0), h0_prop_re=float(np.real(h0_prop)), h0_prop_im=float(np.imag(h0_prop)),
            trial_up=ptr(a["trial_up"]), trial_dn=ptr(a.get("trial_dn")), chol=ptr(a["chol"]),
            rot_chol_up=ptr(a["rot_chol_up"]), rot_chol_dn=ptr(a.get("rot_chol_dn")),
            rot_h1_up=ptr(a["rot_h1_up"]), rot_h1_dn=ptr(a.get("rot_h1_dn")),
            exp_h1_up=ptr(a["exp_h1_up"]), exp_h1_dn=ptr(a.get("exp_h1_dn")),
            mf_shifts=ptr(a["mf_shifts"]))
        self.ham_struct = h
        ctx = ctypes.c_void_p()
        _lib.check(self.lib.afq_ctx_create(ctypes.byref(d), ctypes.byref(h),
                                           ctypes.c_void_p(self.workspace.data_ptr() + off),
                                           ctypes.c_size_t(nbytes), stream_ptr(), ctypes.byref(ctx)),
                   "afq_ctx_create")
        self.ctx = ctx

    def __del__(self):
        try:
            if getattr(self, "ctx", None) is not None and self.ctx.value:
                self.lib.afq_ctx_destroy(self.ctx)
                self.ctx = None
        except Exception:
            pass

    def walkers(self, walkers):
        return walker_ptrs(walkers, self.restricted, self.nw, self.norb, self.nelec)


def _zeros(n, dtype=torch.float64):
    return torch.zeros(n, dtype=dtype, device=device())


def engine_for(trial, ham_data: Optional[dict], wave_data: dict, walkers, *, dt: float = 1.0,
               n_exp_terms: int = 6, n_batch: int = 1, need_propagation: bool = False,
               mixed_config: int = 0) -> Engine:
    """Find or build the engine for these walkers (shape, dtype) and intermediates."""
    restricted = not isinstance(walkers, (list, tuple))
    w0 = walkers if restricted else walkers[0]
    nw = int(w0.shape[0])
    prec = walker_precision(walkers)
    uhf = trial.kind == "uhf"
    if uhf and restricted:
        raise _lib.AfqError("the UHF trial needs unrestricted (two-slab) walkers")
    store = ham_data if ham_data is not None else wave_data
    cache = store.setdefault(_CACHE_KEY, {})
    mo = wave_data["mo_coeff"]
    have_prop = ham_data is not None and "exp_h1" in ham_data and "mf_shifts" in ham_data
    if need_propagation and not have_prop:
        raise _lib.AfqError("ham_data lacks propagation intermediates: call "
                            "hamiltonian.build_propagation_intermediates first")
    if ham_data is not None and "rot_chol" not in ham_data:
        raise _lib.AfqError("ham_data lacks measurement intermediates: call "
                            "hamiltonian.build_measurement_intermediates first")

    def ident(x):
        if x is None:
            return None
        if isinstance(x, (list, tuple)):
            return tuple(ident(y) for y in x)
        return (id(x), x.data_ptr() if isinstance(x, torch.Tensor) else None)

    key = (nw, restricted, prec, float(dt) if have_prop else None, n_exp_terms, n_batch,
           int(mixed_config),
           ident(mo),
           ident(ham_data.get("rot_chol")) if ham_data is not None else None,
           ident(ham_data.get("exp_h1")) if have_prop else None,
           ident(ham_data.get("chol")) if ham_data is not None else None)
    eng = cache.get(key)
    if eng is not None:
        return eng
    norb = trial.norb
    nelec = trial.nelec
    a = {}
    if uhf:
        a["trial_up"], a["trial_dn"] = as_dev(mo[0]), as_dev(mo[1])
    else:
        a["trial_up"] = as_dev(mo)
    if ham_data is not None:
        nchol = int(ham_data["chol"].shape[0])
        a["chol"] = as_dev(ham_data["chol"]).reshape(nchol, norb * norb)
        rc, rh = ham_data["rot_chol"], ham_data["rot_h1"]
        if uhf:
            a["rot_chol_up"], a["rot_chol_dn"] = as_dev(rc[0]), as_dev(rc[1])
            a["rot_h1_up"], a["rot_h1_dn"] = as_dev(rh[0]), as_dev(rh[1])
        else:
            a["rot_chol_up"], a["rot_h1_up"] = as_dev(rc), as_dev(rh)
        h0 = float(np.real(_scalar(ham_data["h0"])))
    else:
        nchol = 1
        a["chol"] = _zeros(norb * norb)
        a["rot_chol_up"] = _zeros(max(nelec) * norb)
        a["rot_h1_up"] = _zeros(max(nelec) * norb)
        if uhf:
            a["rot_chol_dn"], a["rot_h1_dn"] = a["rot_chol_up"], a["rot_h1_up"]
        h0 = 0.0
    if have_prop:
        e = ham_data["exp_h1"]
        e = e if isinstance(e, torch.Tensor) else torch.as_tensor(np.asarray(e))
        if e.dim() == 3:
            a["exp_h1_up"], a["exp_h1_dn"] = as_dev(e[0]), as_dev(e[1])
        else:
            a["exp_h1_up"] = as_dev(e)
            a["exp_h1_dn"] = a["exp_h1_up"]
        mf = ham_data["mf_shifts"]
        a["mf_shifts"] = torch.view_as_real(as_dev(mf, torch.complex128)).contiguous()
        h0p = complex(_scalar(ham_data["h0_prop"]))
    else:
        a["exp_h1_up"] = torch.eye(norb, dtype=torch.float64, device=device())
        a["exp_h1_dn"] = a["exp_h1_up"]
        a["mf_shifts"] = _zeros(2 * nchol)
        h0p = 0.0
    if restricted:
        a.pop("exp_h1_dn", None)
    if prec == _lib.AFQ_PREC_MIXED and ham_data is not None and have_prop and \
            not (int(mixed_config) & _lib.MIXED_EXPLICIT) and _diagonal_chol(a["chol"], norb):
        # on-site lattice terms: the library replaces the vhs GEMM and the Taylor products by
        # a per-row polynomial scale (and checks the diagonality itself)
        mixed_config = (int(mixed_config) or _lib.MIXED_DEFAULT) | _lib.MIXED_DIAG_CHOL
    elif prec == _lib.AFQ_PREC_MIXED and ham_data is not None and have_prop and \
            not (int(mixed_config) & _lib.MIXED_EXPLICIT) and _symmetric_chol(a["chol"], norb):
        # L_g = L_g^T exactly: V is symmetric, so the vhs GEMM computes about two thirds of it
        # and the propagation kernel mirrors the rest (the same numbers as the full product)
        mixed_config = (int(mixed_config) or _lib.MIXED_DEFAULT) | _lib.MIXED_SYM_CHOL
    eng = Engine(norb=norb, nelec=nelec, nchol=nchol, n_walkers=nw, restricted=restricted, uhf=uhf,
                 precision=prec, dt=dt, n_exp_terms=n_exp_terms, n_batch=n_batch, arrays=a, h0=h0,
                 h0_prop=h0p, mixed_config=mixed_config)
    cache[key] = eng
    return eng


def _diagonal_chol(chol: torch.Tensor, norb: int) -> bool:
    """True when every Cholesky vector [norb, norb] is a diagonal matrix."""
    c = chol.reshape(-1, norb, norb)
    off = c - torch.diag_embed(torch.diagonal(c, dim1=1, dim2=2))
    return bool(torch.count_nonzero(off).item() == 0)


def _symmetric_chol(chol: torch.Tensor, norb: int) -> bool:
    """True when every Cholesky vector [norb, norb] equals its transpose exactly."""
    c = chol.reshape(-1, norb, norb)
    return bool(torch.equal(c, c.transpose(1, 2)))


def _scalar(x):
    if isinstance(x, torch.Tensor):
        return x.item()
    return np.asarray(x).item() if np.ndim(x) == 0 else np.asarray(x).reshape(-1)[0].item()
