"""The allocation-free entry point ps_fit_batch_noalloc.

Callers that cannot let the library allocate device memory at call time
(hosts that give all GPU memory to their own pool, jobs under a fixed memory
budget, pipelines that cannot take the synchronisation of cudaMalloc/cudaFree)
use this variant: work lists and outputs are the caller's device buffers, and
the kernel's work counter and per-slot scratch live in a file-scope device
array.  This test allocates the caller's buffers itself (with torch), calls the
entry point through the C ABI twice in a row, and checks both results against
the allocating entry point ps_fit_batch with the FP64 tolerance of the other
parity tests.  The file name sorts last so that a run stopping at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL = 1e-6


@pytest.mark.parametrize("case", ["tiny_mix", "golden"])
def test_noalloc_matches_fit_batch(engine_lib, case):
    import torch

    from periodsearch_gb300 import FIT_DTYPE, Engine, _abi, read_input

    path = GOLDEN / "period_search_in" if case == "golden" else GOLDEN / case / "period_search_in"
    eng = Engine(read_input(path))
    conw_r = eng.info.conw_r0
    periods = np.repeat(np.arange(1, 4), 10).astype(np.int64)
    poles = np.tile(np.arange(1, 11), 3).astype(np.int32)
    want = eng.fit_batch(conw_r, periods, poles)

    dev = torch.device("cuda", 0)
    d_p = torch.from_numpy(periods).to(dev)
    d_m = torch.from_numpy(poles).to(dev)
    n = len(periods)
    # both calls' output buffers exist before the first call, so that the
    # device's free memory can only change if the entry point allocates
    outs = [torch.full((n * FIT_DTYPE.itemsize,), 0xFF, dtype=torch.uint8, device=dev) for _ in range(2)]
    torch.cuda.synchronize(dev)
    free_after = []
    for call in range(2):
        d_out = outs[call]
        stream = torch.cuda.current_stream(dev)
        st = engine_lib.ps_fit_batch_noalloc(eng._ctx, conw_r, n, C.c_void_p(d_p.data_ptr()),
                                             C.c_void_p(d_m.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        _abi.check(st, "ps_fit_batch_noalloc", eng._ctx)
        torch.cuda.synchronize(dev)
        free_after.append(torch.cuda.mem_get_info(dev)[0])
        got = np.frombuffer(d_out.cpu().numpy().tobytes(), FIT_DTYPE)
        for f in ("dev", "chisq", "period_h", "totarea", "dark"):
            np.testing.assert_allclose(got[f], want[f], rtol=RTOL, err_msg=f"call {call}: {f}")
        np.testing.assert_allclose(got["lambda_deg"], want["lambda_deg"], atol=1e-6)
        np.testing.assert_allclose(got["beta_deg"], want["beta_deg"], atol=1e-6)
        assert np.array_equal(got["niter"], want["niter"])
    # the second call (the array's address already looked up) takes no
    # device memory
    assert free_after[1] == free_after[0], free_after
    eng.close()


def test_noalloc_refuses_mixed_form(engine_lib):
    """The entry point serves the FP64 form only: a mixed-form context is
    refused with PS_ERR_ARG before anything is launched."""
    import torch

    from periodsearch_gb300 import FIT_DTYPE, PS_FORM_MIXED, Engine, read_input
    from periodsearch_gb300._abi import PS_ERR_ARG

    eng = Engine(read_input(GOLDEN / "tiny_mix" / "period_search_in"), form=PS_FORM_MIXED)
    dev = torch.device("cuda", 0)
    d_p = torch.ones(10, dtype=torch.int64, device=dev)
    d_m = torch.arange(1, 11, dtype=torch.int32, device=dev)
    d_out = torch.zeros(10 * FIT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    st = engine_lib.ps_fit_batch_noalloc(eng._ctx, eng.info.conw_r0, 10, C.c_void_p(d_p.data_ptr()),
                                         C.c_void_p(d_m.data_ptr()), C.c_void_p(d_out.data_ptr()), None)
    assert st == PS_ERR_ARG
    eng.close()
