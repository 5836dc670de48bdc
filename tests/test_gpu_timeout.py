"""Bounded device waits: a wait that runs out is reported as MMR_ERR_TIMEOUT, the context stays
usable, and callers with device arrays see it through mmr_check_device_error.  The test lowers the
gridding kernels' poll limit to 0 (mmr_debug_set_wait_polls), so every TMA wait of the forward
interpolation gives up at once; the kernel still lets its copy land before returning, so nothing is
left in flight and no GPU fault is involved."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case():
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    N = 64
    kloc = synth.spiral(N, 4, 1024, 2.0)
    S = mm.nufftOp([N, N], kloc, None, 1, 2.0, 4)
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    return mm, S, x


def test_wait_timeout_reported_and_recovered():
    import torch
    from matmri_gb300 import _lib
    mm, S, x = _case()
    lib = _lib.load()
    ref = S * x
    try:
        _lib.check(lib.mmr_debug_set_wait_polls(0))
        # host arrays: the call itself reports the timeout
        with pytest.raises(mm.MatmriError) as ei:
            S * x
        assert ei.value.code == 4
        # device arrays: the call returns, the check reports it once
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda().T
        S * xd
        stream = torch.cuda.current_stream().cuda_stream
        with pytest.raises(mm.MatmriError) as ei:
            mm.check_device_error(stream)
        assert ei.value.code == 4
        mm.check_device_error(stream)      # cleared
    finally:
        _lib.check(lib.mmr_debug_set_wait_polls(1 << 22))
    # the context is usable and results are unchanged
    again = S * x
    assert np.array_equal(again, ref)
    mm.check_device_error()
