"""The FP64 oracle against the reference's own known-answer values
(tests/test_wavefunctions.py:127-183 of the reference)."""

import json
import os

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.golden import seed102_fixture

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))
FX = seed102_fixture.build()


def close(a, key):
    assert np.allclose(a, KAT[key], rtol=KAT["rtol"], atol=KAT["atol"]), (key, a, KAT[key])
    # the restatement reproduces them far below the reference's own tolerance
    assert abs(a - KAT[key]) <= 1e-12 * max(1.0, abs(KAT[key])), (key, a, KAT[key])


def test_rhf_overlap():
    close(np.real(O.rhf_overlap_restricted(FX["walker"][None], FX["mo"])[0]), "rhf_overlap_real")


def test_rhf_green():
    g = O.rhf_green(FX["walker"][None], FX["mo"])[0]
    assert g.shape == (5, 10)
    close(np.real(np.sum(g)), "rhf_green_sum_real")


def test_rhf_force_bias():
    fb = O.rhf_force_bias_restricted(FX["walker"][None], FX["rot_chol"], FX["mo"])[0]
    assert fb.shape == (5,)
    close(np.real(np.sum(fb)), "rhf_force_bias_sum_real")


def test_rhf_energy():
    e = O.rhf_energy_restricted(FX["walker"][None], FX["h0"], FX["rot_h1"], FX["rot_chol"], FX["mo"])[0]
    close(np.real(e), "rhf_energy_real")


def test_uhf_overlap():
    o = O.uhf_overlap(FX["walker_up"][None], FX["walker_dn"][None], FX["mo_u"])[0]
    close(np.real(o), "uhf_overlap_real")


def test_uhf_green():
    g = O.uhf_green(FX["walker_up"][None], FX["walker_dn"][None], FX["mo_u"])
    assert g[0].shape == (1, 3, 10) and g[1].shape == (1, 2, 10)
    close(np.real(np.sum(g[0]) + np.sum(g[1])), "uhf_green_sum_real")


def test_uhf_force_bias():
    fb = O.uhf_force_bias(FX["walker_up"][None], FX["walker_dn"][None], FX["rot_chol_u"], FX["mo_u"])[0]
    assert fb.shape == (5,)
    close(np.real(np.sum(fb)), "uhf_force_bias_sum_real")


def test_uhf_energy():
    e = O.uhf_energy(FX["walker_up"][None], FX["walker_dn"][None], FX["h0"], FX["rot_h1_u"],
                     FX["rot_chol_u"], FX["mo_u"])[0]
    close(np.real(e), "uhf_energy_real")


def test_oracle_detects_planted_error():
    """A mistake planted in the oracle's inputs must break the pin (the KAT is sensitive)."""
    rc = FX["rot_chol"].copy()
    rc[0, 0, 0] += 1e-6
    fb = O.rhf_force_bias_restricted(FX["walker"][None], rc, FX["mo"])[0]
    assert abs(np.real(np.sum(fb)) - KAT["rhf_force_bias_sum_real"]) > 1e-9
