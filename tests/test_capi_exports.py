"""The C-ABI library builds, loads without a GPU and exports every function the public
header declares (no compute calls here)."""

import glob
import os
import re

import pytest

from cs_afqmc_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(afq_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared()
    for n in ["afq_propagate", "afq_calc_force_bias", "afq_calc_energy", "afq_calc_overlap",
              "afq_orthonormalize_walkers", "afq_propagate_phaseless"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.afq_abi_version() == 1


def test_binding_table_matches_header():
    assert set(_lib.EXPORTED) == declared()


def test_workspace_size_and_validation_without_gpu():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    import ctypes
    lib = _lib.load()
    d = _lib.Dims(norb=120, n_up=20, n_dn=20, nchol=600, n_walkers=1024, walker_type=0,
                  trial_type=0, precision=0, n_exp_terms=6, n_batch=4, dt=0.005)
    assert lib.afq_workspace_size(ctypes.byref(d)) > 0
    d.n_dn = 19  # RHF needs equal spins
    assert lib.afq_workspace_size(ctypes.byref(d)) == 0
    assert b"RHF" in lib.afq_last_error()
    d.n_dn, d.n_batch = 20, 3  # must divide n_walkers
    assert lib.afq_workspace_size(ctypes.byref(d)) == 0


def test_derivative_and_cpmc_entry_validation_without_gpu():
    """The derivative and CPMC entry points refuse NULL or inconsistent arguments before
    any device work: -1 and a message."""
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    import ctypes
    lib = _lib.load()
    d = _lib.Dims(norb=12, n_up=3, n_dn=3, nchol=20, n_walkers=8, walker_type=0, trial_type=0, precision=0,
                  n_exp_terms=6, n_batch=1, dt=0.005)
    big = lib.afq_vjp_workspace_size(ctypes.byref(d), 5, 4, 2)
    small = lib.afq_vjp_workspace_size(ctypes.byref(d), 5, 4, 1)
    assert big > small > 0  # the recorded sweep grows with the block count
    assert lib.afq_vjp_workspace_size(ctypes.byref(d), 0, 4, 1) == 0
    assert lib.afq_tangent_workspace_size(ctypes.byref(d)) > 0
    outs = _lib.VjpOutputs()
    assert lib.afq_propagate_phaseless_vjp_ex(None, None, None, 0, None, None, 1, 1, 1, 0, None, None, None,
                                              ctypes.byref(outs), None) == -1
    assert b"NULL" in lib.afq_last_error()
    tin = _lib.JvpInputs()
    assert lib.afq_propagate_phaseless_jvp_ex(None, None, ctypes.byref(tin), None, 0, None, None, 1, 1, 1, 0,
                                              None, None, None, None, None, None, None) == -1
    assert lib.afq_cpmc_nn_propagate(8, 3, 3, 4, 0.01, 4.0, 1.0, None, 2, None, None, None, None, None, None,
                                     None, None, None, None, None, None) == -1
    assert b"NULL" in lib.afq_last_error()
