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
    for call in range(2):
        d_out = torch.full((n * FIT_DTYPE.itemsize,), 0xFF, dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev)
        st = engine_lib.ps_fit_batch_noalloc(eng._ctx, conw_r, n, C.c_void_p(d_p.data_ptr()),
                                             C.c_void_p(d_m.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        _abi.check(st, "ps_fit_batch_noalloc", eng._ctx)
        torch.cuda.synchronize(dev)
        got = np.frombuffer(d_out.cpu().numpy().tobytes(), FIT_DTYPE)
        for f in ("dev", "chisq", "period_h", "totarea", "dark"):
            np.testing.assert_allclose(got[f], want[f], rtol=RTOL, err_msg=f"call {call}: {f}")
        np.testing.assert_allclose(got["lambda_deg"], want["lambda_deg"], atol=1e-6)
        np.testing.assert_allclose(got["beta_deg"], want["beta_deg"], atol=1e-6)
        assert np.array_equal(got["niter"], want["niter"])
    eng.close()
