"""ctypes binding of libafqmc_gb300.so, the C ABI declared in include/afqmc_gb300.h.

The shared library is the product: there is no CPU or PyTorch fallback. Loading fails
loudly when the library has not been built (``python -c "import __graft_entry__ as g;
g.build()"``) or when no CUDA device is present at call time.
"""

from __future__ import annotations

import ctypes
import os
from typing import Optional

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libafqmc_gb300.so")

AFQ_WALKERS_RESTRICTED, AFQ_WALKERS_UNRESTRICTED = 0, 1
AFQ_TRIAL_RHF, AFQ_TRIAL_UHF = 0, 1
AFQ_PREC_FP64, AFQ_PREC_MIXED = 0, 1
AFQ_S_E_ESTIMATE, AFQ_S_POP_CONTROL_SHIFT, AFQ_S_N_KILLED = 0, 1, 2
AFQ_S_BLOCK_ENERGY, AFQ_S_BLOCK_WEIGHT, AFQ_S_STATUS = 3, 4, 5
AFQ_NSCALARS = 8
AFQ_JVP_NO_SR = 1
MIXED_DEFAULT = 767          # the library's default accuracy options (afq_dims.mixed_config)
MIXED_DIAG_CHOL = 1 << 15    # every Cholesky vector diagonal: per-row exp(vhs), no Taylor MMA
MIXED_EXPLICIT = 1 << 30     # the caller's configuration as given (no automatic diagonal path)
MIXED_LEGACY_TAYLOR = 1 << 16  # separate exp_h1 GEMMs and Taylor kernel instead of the fused kernel
MIXED_SYM_CHOL = 1 << 17     # every Cholesky vector symmetric: packed vhs GEMM, V mirrored on load

_vp = ctypes.c_void_p


class Dims(ctypes.Structure):
    _fields_ = [
        ("norb", ctypes.c_int32), ("n_up", ctypes.c_int32), ("n_dn", ctypes.c_int32),
        ("nchol", ctypes.c_int32), ("n_walkers", ctypes.c_int32),
        ("walker_type", ctypes.c_int32), ("trial_type", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("n_exp_terms", ctypes.c_int32),
        ("n_batch", ctypes.c_int32), ("mixed_config", ctypes.c_int32), ("dt", ctypes.c_double),
    ]


class Hamiltonian(ctypes.Structure):
    _fields_ = [
        ("h0", ctypes.c_double), ("h0_prop_re", ctypes.c_double), ("h0_prop_im", ctypes.c_double),
        ("trial_up", _vp), ("trial_dn", _vp), ("chol", _vp),
        ("rot_chol_up", _vp), ("rot_chol_dn", _vp), ("rot_h1_up", _vp), ("rot_h1_dn", _vp),
        ("exp_h1_up", _vp), ("exp_h1_dn", _vp), ("mf_shifts", _vp),
    ]


class JvpInputs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("dexp_h1_up", "dexp_h1_dn", "drot_h1_up", "drot_h1_dn",
                                              "dtrial_up", "dtrial_dn", "drot_chol_up", "drot_chol_dn")]


class VjpOutputs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("gexp_h1_up", "gexp_h1_dn", "grot_h1_up", "grot_h1_dn",
                                              "gtrial_up", "gtrial_dn", "grot_chol", "gchol", "gmf_shifts",
                                              "gh0_prop")]


class WalkerState(ctypes.Structure):
    _fields_ = [("walkers_up", _vp), ("walkers_dn", _vp), ("weights", _vp),
                ("overlaps", _vp), ("scalars", _vp)]


_SIGS = {
    "afq_abi_version": (ctypes.c_int, []),
    "afq_last_error": (ctypes.c_char_p, []),
    "afq_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(Dims)]),
    "afq_ctx_create": (ctypes.c_int, [ctypes.POINTER(Dims), ctypes.POINTER(Hamiltonian), _vp,
                                      ctypes.c_size_t, _vp, ctypes.POINTER(_vp)]),
    "afq_ctx_destroy": (None, [_vp]),
    "afq_calc_overlap": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "afq_calc_force_bias": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "afq_calc_energy": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "afq_propagate": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp]),
    "afq_orthonormalize_walkers": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp]),
    "afq_stochastic_reconfiguration": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp, _vp]),
    "afq_propagate_phaseless": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp,
                                               ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                               _vp, _vp, _vp, _vp]),
    "afq_block_end": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp, _vp, _vp]),
    "afq_propagate_free": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, ctypes.c_double, _vp, _vp, _vp]),
    "afq_propagate_free_blocks": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, ctypes.c_int32,
                                                 ctypes.c_int32, ctypes.c_double, _vp, _vp, _vp, _vp, _vp]),
    "afq_cpmc_init": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _vp, _vp,
                                     _vp, _vp, _vp, _vp, _vp]),
    "afq_cpmc_propagate": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                          _vp, _vp, _vp, _vp, _vp]),
    "afq_cpmc_continuous_propagate": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_double, ctypes.c_double, _vp,
                                                     _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "afq_cpmc_nn_propagate": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double, _vp, ctypes.c_int32,
                                             _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "afq_tangent_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(Dims)]),
    "afq_propagate_phaseless_jvp": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp, _vp, _vp,
                                                   _vp, ctypes.c_size_t, _vp, _vp, ctypes.c_int32,
                                                   ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _vp, _vp,
                                                   _vp, _vp, _vp, _vp, _vp]),
    "afq_propagate_phaseless_jvp_ex": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, _vp,
                                                      ctypes.c_size_t, _vp, _vp, ctypes.c_int32, ctypes.c_int32,
                                                      ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp,
                                                      _vp, _vp]),
    "afq_propagate_phaseless_vjp_ex": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, ctypes.c_size_t,
                                                      _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                      ctypes.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "afq_vjp_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(Dims), ctypes.c_int32, ctypes.c_int32,
                                                 ctypes.c_int32]),
    "afq_propagate_phaseless_vjp": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, ctypes.c_size_t, _vp,
                                                   _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "afq_field_block": (ctypes.c_int, [_vp, ctypes.POINTER(WalkerState), _vp, ctypes.c_int32, _vp, _vp,
                                       _vp, _vp]),
    "afq_cs_outlier_removal": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_double, _vp,
                                              _vp]),
    "afq_calc_force_bias_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "afq_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "afq_profile_reset": (ctypes.c_int, []),
    "afq_profile_read": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_int64)]),
    "afq_profile_class_name": (ctypes.c_char_p, [ctypes.c_int]),
    "afq_profile_num_classes": (ctypes.c_int, []),
    "afq_fill_normal": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64, _vp]),
    "afq_fill_uniform": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64, _vp]),
}

# include/afqmc_gb300_testing.h: single-kernel hooks for the numerics tests
_TEST_SIGS = {
    "afq_test_gemm_f16": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_long, ctypes.c_long, _vp,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         _vp, _vp]),
    "afq_test_gemm_split": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, _vp, _vp]),
    "afq_test_split_pairs": (ctypes.c_int, [ctypes.c_int]),
}
_SIGS.update(_TEST_SIGS)

EXPORTED = tuple(_SIGS)

_lib: Optional[ctypes.CDLL] = None


class AfqError(RuntimeError):
    pass


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Load (once) and return the library; raises AfqError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise AfqError(
            f"{path} not found: build it with `python -c \"import __graft_entry__ as g; g.build()\"`"
        )
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        msg = load().afq_last_error().decode(errors="replace")
        raise AfqError(f"{what} failed (rc={rc}): {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def profile_read_all() -> dict:
    """{class name: (total ms, launches)} since the last afq_profile_enable/reset."""
    lib = load()
    out = {}
    for c in range(lib.afq_profile_num_classes()):
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(lib.afq_profile_read(c, ctypes.byref(ms), ctypes.byref(n)), "afq_profile_read")
        out[lib.afq_profile_class_name(c).decode()] = (ms.value, n.value)
    return out
