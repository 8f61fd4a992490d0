"""Rebuilds the seed-102 fixture of the reference's wavefunction unit tests.

The reference (zh-yichi/cs_afqmc, tests/test_wavefunctions.py:12-72) draws its inputs with
numpy's legacy global RNG after ``np.random.seed(102)``, in this order: RHF walker real and
imaginary parts [10,5]; h0; rot_h1 [5,10]; rot_chol [5,5,10]; h1 [10,10]; chol [5,10,10];
UHF mo_coeff [10,3] and [10,2]; UHF walker up real/imag [10,3], down real/imag [10,2].
The trial is the identity's first 5 columns (RHF); the UHF intermediates are slices of the
RHF ones. The known-answer values these inputs produce are in reference_kat.json.
"""

import numpy as np


def build():
    rs = np.random.RandomState(102)
    norb, nocc, nchol = 10, 5, 5
    walker = rs.rand(norb, nocc) + 1.0j * rs.rand(norb, nocc)
    h0 = rs.rand(1)[0]
    rot_h1 = rs.rand(nocc, norb)
    rot_chol = rs.rand(nchol, nocc, norb)
    h1 = rs.rand(norb, norb)
    chol = rs.rand(nchol, norb, norb)
    mo = np.eye(norb)[:, :nocc]
    nup, ndn = 3, 2
    mo_u = [rs.rand(norb, nup), rs.rand(norb, ndn)]
    wu = rs.rand(norb, nup) + 1.0j * rs.rand(norb, nup)
    wd = rs.rand(norb, ndn) + 1.0j * rs.rand(norb, ndn)
    return dict(
        norb=norb, nocc=nocc, nchol=nchol, walker=walker, h0=h0, rot_h1=rot_h1,
        rot_chol=rot_chol, h1=np.stack([h1, h1]), chol=chol.reshape(nchol, -1), mo=mo,
        nelec_u=(nup, ndn), mo_u=mo_u, walker_up=wu, walker_dn=wd,
        rot_h1_u=[rot_h1[:nup], rot_h1[:ndn]], rot_chol_u=[rot_chol[:, :nup], rot_chol[:, :ndn]],
    )
