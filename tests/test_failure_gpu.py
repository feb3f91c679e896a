"""The device-side failure path: a bounded wait that runs out.

Every mbarrier wait in the library's TMA / tensor-core pipelines gives up
after a bounded number of SM cycles, records a code in the per-device error
word and leaves, so a copy that never lands turns into a status the host can
read instead of a hung GPU.  scir_selftest_pipeline runs that path on
purpose, without any fault: its producer stops issuing copies (a host flag),
so the consumer waits on a barrier that nothing completes until its short
limit passes.  Nothing here faults, traps or hangs the GPU."""
import ctypes

import numpy as np
import pytest

import scir_gb300 as S

pytestmark = pytest.mark.gpu

LIMIT = 2_000_000  # SM cycles (about 1 ms at 2 GHz)


def _run(cuda, n_chunks, issue):
    import torch
    g = torch.Generator(device=cuda).manual_seed(11)
    x = torch.randn(n_chunks * 1024, device=cuda, generator=g)
    out = torch.full((n_chunks,), float("nan"), device=cuda)
    rc = S.load().scir_selftest_pipeline(x.data_ptr(), n_chunks, issue, LIMIT,
                                               out.data_ptr(),
                                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0, S.last_error()
    torch.cuda.synchronize()
    return x.view(n_chunks, 1024).double().sum(1).cpu().numpy(), out.cpu().numpy()


def test_pipeline_completes_without_error(cuda):
    ref, out = _run(cuda, 64, 64)
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-3)
    assert S.device_errors() == 0


@pytest.mark.parametrize("issue", [0, 1, 5, 63])
def test_starved_wait_times_out_and_is_reported(cuda, issue):
    ref, out = _run(cuda, 64, issue)
    # the chunks that arrived were consumed; the first missing one was waited
    # for until the limit, then the kernel gave up and reported it
    np.testing.assert_allclose(out[:issue], ref[:issue], rtol=0, atol=1e-3)
    assert np.isnan(out[issue:]).all()
    assert S.device_errors() == 1  # kErrMbarTimeout, read and cleared
    assert S.device_errors() == 0
    # the context stays usable: a normal call runs afterwards
    ref2, out2 = _run(cuda, 8, 8)
    np.testing.assert_allclose(out2, ref2, rtol=0, atol=1e-3)
    assert S.device_errors() == 0


def test_selftest_validates_arguments(cuda):
    L = S.load()
    f = ctypes.c_void_p(256)
    assert L.scir_selftest_pipeline(f, 4, 5, LIMIT, f, None) == S.ERR_INVALID_ARG
    assert L.scir_selftest_pipeline(f, 4, 4, 10, f, None) == S.ERR_INVALID_ARG
    assert L.scir_selftest_pipeline(ctypes.c_void_p(260), 4, 4, LIMIT, f, None) == S.ERR_ALIGN
