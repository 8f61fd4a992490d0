"""Cholesky-integral file I/O (cs_afqmc_gb300.integrals) on the CPU: the HDF5 subset reader
and writer round trip, the FCIDUMP_chol field mapping of _prep_afqmc (mpi_jax.py:39-60), and
the reader on the reference's own fixture file (tests/FCIDUMP_chol of the reference, an
HDF5 file written by h5py; a byte-for-byte copy is kept as tests/golden/FCIDUMP_chol): its
header and structural identities (symmetric hcore and Cholesky vectors, identity /
orthogonal trial orbitals) pin the decoding."""

import os

import numpy as np
import pytest

from cs_afqmc_gb300 import integrals as I

REF_FCIDUMP = os.environ.get(
    "AFQ_REFERENCE_FCIDUMP", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "FCIDUMP_chol"))


def test_h5_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    d = {"a": rng.standard_normal((3, 4)), "b": np.arange(7, dtype=np.int64), "c": np.float64(2.5),
         "long_dataset_name": rng.standard_normal(1000)}
    p = str(tmp_path / "x.h5")
    I.write_h5(p, d)
    g = I.read_h5(p)
    assert sorted(g) == sorted(d)
    for k in d:
        assert g[k].shape == np.asarray(d[k]).shape
        assert np.array_equal(g[k], d[k])


def test_fcidump_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    nmo, nchol = 5, 7
    h1 = rng.standard_normal((nmo, nmo))
    h1 = h1 + h1.T
    chol = rng.standard_normal((nchol, nmo, nmo))
    mo = [np.eye(nmo), np.linalg.qr(rng.standard_normal((nmo, nmo)))[0]]
    p = str(tmp_path / "FCIDUMP_chol")
    I.write_fcidump_chol(p, h1, h1 - 0.1, chol, nelec=5, nmo=nmo, enuc=1.25, ms=1, mo_coeffs=mo)
    f = I.read_fcidump_chol(p)
    assert (f["nelec"], f["nmo"], f["ms"], f["nchol"]) == (5, nmo, 1, nchol)
    assert f["h0"] == 1.25
    assert np.array_equal(f["h1"], h1) and np.array_equal(f["h1_mod"], h1 - 0.1)
    assert np.array_equal(f["chol"], chol)
    assert np.array_equal(f["mo_coeffs"][1], mo[1])
    h = I.ham_data_from_fcidump(p)
    assert h["nelec"] == (3, 2) and h["norb"] == nmo and h["nchol"] == nchol
    assert h["ham_data"]["h1"].shape == (2, nmo, nmo)
    assert np.array_equal(h["ham_data"]["chol"], chol.reshape(nchol, nmo * nmo))


def test_not_hdf5(tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(b"not an hdf5 file at all")
    with pytest.raises(I.H5FormatError):
        I.read_h5(str(p))


@pytest.mark.skipif(not os.path.exists(REF_FCIDUMP), reason="fixture file not present")
def test_reference_fixture():
    f = I.read_fcidump_chol(REF_FCIDUMP)
    assert (f["nelec"], f["nmo"], f["ms"], f["nchol"]) == (6, 6, 0, 15)
    assert abs(f["h0"] - 4.35) < 1e-12
    assert np.allclose(f["h1"], f["h1"].T, atol=1e-12)
    assert np.allclose(f["h1_mod"], f["h1_mod"].T, atol=1e-12)
    for L in f["chol"]:
        assert np.allclose(L, L.T, atol=1e-12)
    up, dn = f["mo_coeffs"]
    assert np.allclose(up, np.eye(6), atol=1e-12)
    assert np.allclose(dn.T @ dn, np.eye(6), atol=1e-10)
    h = I.ham_data_from_fcidump(REF_FCIDUMP)
    assert h["nelec"] == (3, 3)
