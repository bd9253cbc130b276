"""The allocation-free Whittle entry point (pes_whittle_lnl_noalloc).

It serves callers that may not allocate device memory (stream capture into a
CUDA graph, host runtimes that own the memory pool).  Checked through the C ABI
against pes_whittle_lnl with a caller workspace, on two calls in a row with
different inputs (the shared scratch keeps the previous call's contents).
This file is collected last so that a failure here stops a run only after
every other test has run.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _call_pair(lib, _lib, d, h, s, df):
    C, n = d.shape
    ws = torch.empty(int(lib.pes_whittle_workspace_len(n)), dtype=torch.float64, device="cuda")
    ref = torch.empty(1, dtype=torch.float64, device="cuda")
    got = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    _lib.check(lib.pes_whittle_lnl(_lib.ptr(d), _lib.ptr(h), _lib.ptr(s), C, n, df, _lib.ptr(ws), ws.numel(),
                                   _lib.ptr(ref), None))
    _lib.check(lib.pes_whittle_lnl_noalloc(_lib.ptr(d), _lib.ptr(h), _lib.ptr(s), C, n, df, _lib.ptr(got), None))
    torch.cuda.synchronize()
    return float(ref.item()), float(got.item())


@pytest.mark.parametrize("n,C", [(300_001, 3), (125_410, 2), (7, 1)])
def test_noalloc_matches_workspace_entry_point(cuda_lib, n, C):
    from pespace_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(n + C)
    values = []
    for call in range(2):  # two calls in a row, different inputs
        d = torch.as_tensor(rng.normal(size=(C, n)) + 1j * rng.normal(size=(C, n)), device="cuda")
        h = torch.as_tensor(rng.normal(size=(C, n)) + 1j * rng.normal(size=(C, n)), device="cuda")
        s = torch.as_tensor(rng.uniform(0.1, 3.0, size=(C, n)), device="cuda")
        ref, got = _call_pair(lib, _lib, d, h, s, 1e-3 * (call + 1))
        assert abs(got - ref) <= 1e-12 * abs(ref), (call, got, ref)
        values.append(got)
    assert values[0] != values[1]


def test_noalloc_rejects_bad_sizes(cuda_lib):
    from pespace_gb300 import _lib

    lib = _lib.load()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    assert lib.pes_whittle_lnl_noalloc(None, None, None, 4, 10, 1.0, _lib.ptr(out), None) == _lib.PES_EINVAL
    assert b"n_chan" in lib.pes_last_error()
    assert lib.pes_whittle_lnl_noalloc(None, None, None, 3, 2 ** 31, 1.0, _lib.ptr(out), None) == _lib.PES_EINVAL
    assert b"outside" in lib.pes_last_error()
    # empty input: lnL = 0 without touching the data pointers
    _lib.check(lib.pes_whittle_lnl_noalloc(None, None, None, 3, 0, 1.0, _lib.ptr(out), None))
    torch.cuda.synchronize()
    assert out.item() == 0.0
