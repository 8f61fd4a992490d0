"""The allocation-free force bias (afq_calc_force_bias_noalloc) against the context-based
afq_calc_force_bias, through the C ABI.

The entry point exists for callers that cannot allocate device memory, such as code that
runs inside another runtime's memory arena and only receives pre-allocated buffers: it
keeps its Green's-function scratch in a static device array of the library. This file is
collected last so that a failure here cannot hide the rest of the suite; it must pass both
alone in a fresh process and after the other tests. Tolerance: both paths run the same FP64
kernels, so results agree to 1e-10 relative, as in the other FP64 parity tests.
"""

import numpy as np
import pytest

from tests.helpers import Case, rel_err, to_np

pytestmark = pytest.mark.gpu


def _noalloc(case, walkers, out):
    import torch

    from cs_afqmc_gb300 import _lib
    from cs_afqmc_gb300._engine import stream_ptr

    trial = torch.as_tensor(np.ascontiguousarray(case.sys.mo_coeff), dtype=torch.float64, device="cuda")
    rc = case.ham_data["rot_chol"].contiguous()
    _lib.call("afq_calc_force_bias_noalloc", case.norb, case.nelec[0], case.nchol, case.nw,
              trial.data_ptr(), rc.data_ptr(), walkers.data_ptr(), out.data_ptr(), stream_ptr())


def test_noalloc_matches_context_path_twice():
    import torch

    case = Case(kind="rhf", restricted=True, norb=40, nelec=(9, 9), nchol=70, nw=16)
    w = case.gpu_walkers()
    ref = to_np(case.trial.calc_force_bias(w, case.ham_data, case.wave_data))
    for _ in range(2):  # the second call reuses the scratch left by the first
        out = torch.full((case.nw, case.nchol), float("nan"), dtype=torch.complex128, device="cuda")
        _noalloc(case, w, out)
        torch.cuda.synchronize()
        assert rel_err(to_np(out), ref) < 1e-10
    # different walkers on the same scratch
    w2 = case.gpu_walkers(case.walkers0 * 1.1 + 0.01)
    ref2 = to_np(case.trial.calc_force_bias(w2, case.ham_data, case.wave_data))
    out = torch.full((case.nw, case.nchol), float("nan"), dtype=torch.complex128, device="cuda")
    _noalloc(case, w2, out)
    torch.cuda.synchronize()
    assert rel_err(to_np(out), ref2) < 1e-10


def test_noalloc_rejects_sizes_beyond_the_scratch():
    import torch

    from cs_afqmc_gb300 import _lib
    from cs_afqmc_gb300._engine import stream_ptr

    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    lib = _lib.load()
    rc = lib.afq_calc_force_bias_noalloc(128, 32, 8, 4096, dummy.data_ptr(), dummy.data_ptr(),
                                         dummy.data_ptr(), dummy.data_ptr(), stream_ptr())
    assert rc < 0
    assert b"static scratch" in lib.afq_last_error()


def test_noalloc_at_the_scratch_limit():
    """n_walkers * nocc * norb exactly at the 2,621,440-element capacity (1024 walkers, 20
    electrons, 128 orbitals): accepted, and the last walker's force bias - computed from the
    last bytes of the scratch - equals the context path's; one walker more is rejected."""
    import torch

    from cs_afqmc_gb300 import _lib
    from cs_afqmc_gb300._engine import stream_ptr

    case = Case(kind="rhf", restricted=True, norb=128, nelec=(20, 20), nchol=24, nw=1024)
    assert case.nw * case.nelec[0] * case.norb == 2_621_440
    w = case.gpu_walkers()
    ref = to_np(case.trial.calc_force_bias(w, case.ham_data, case.wave_data))
    out = torch.full((case.nw, case.nchol), float("nan"), dtype=torch.complex128, device="cuda")
    _noalloc(case, w, out)
    torch.cuda.synchronize()
    got = to_np(out)
    assert rel_err(got, ref) < 1e-10
    assert rel_err(got[-1], ref[-1]) < 1e-10

    lib = _lib.load()
    trial = torch.as_tensor(np.ascontiguousarray(case.sys.mo_coeff), dtype=torch.float64, device="cuda")
    rc = lib.afq_calc_force_bias_noalloc(case.norb, case.nelec[0], case.nchol, case.nw + 1, trial.data_ptr(),
                                         case.ham_data["rot_chol"].data_ptr(), w.data_ptr(), out.data_ptr(),
                                         stream_ptr())
    assert rc < 0
    assert b"static scratch" in lib.afq_last_error()
