"""pqc_run_static, the forward entry point that allocates no device memory.

It serves callers that cannot allocate on the GPU (a host framework that owns
all device memory, a loop that must not risk an allocation); its scratch is a
fixed array inside the library.  Called here through the C ABI and compared
with pqc_run, which takes a caller workspace, on two calls in a row (the
second call reuses the array the first one left behind).  This file is
collected last so that a stop at the first failure has already run the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib, engine

pytestmark = pytest.mark.gpu
AMP_TOL = 1e-10  # the amplitude tolerance of the other GPU parity tests


def _static(lib, prog, theta, out):
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.pqc_run_static(prog.handle, C.c_void_p(theta.data_ptr()), theta.shape[1], theta.shape[0], None, 0,
                              C.c_void_p(out.data_ptr()), stream)


def test_run_static_matches_run_on_two_calls_in_a_row(cuda):
    lib = _lib.load()
    assert lib.pqc_run_static_capacity() == 16 << 20
    c = pq.templates.hardware_efficient_ladder(15, 4)  # N = 15 > 13: a multi-sweep plan
    prog = c.program
    rs = np.random.default_rng(7)
    for call in range(2):
        theta = torch.from_numpy(rs.random((6, c.n_columns())) * 2 * np.pi).to(cuda)
        ref = prog.run(theta, 0)
        out = torch.full_like(ref, complex(np.nan, np.nan))
        rc = _static(lib, prog, theta, out)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        assert float((out - ref).abs().max()) < AMP_TOL, f"call {call}"
    # the second batch's states are not the first batch's: the shared scratch was rewritten
    assert float((out[0] - prog.run(theta[:1] * 0.5, 0)[0]).abs().max()) > 1e-3


def test_run_static_rejects_batches_beyond_its_scratch(cuda):
    lib = _lib.load()
    c = pq.templates.hardware_efficient_ladder(10, 10)
    prog = c.program
    per_row = c.n_columns() * 4 * (8 + 8)  # f64 + double-float sine/cosine tables
    B = (16 << 20) // per_row + 8
    theta = torch.zeros((B, c.n_columns()), dtype=torch.float64, device=cuda)
    out = torch.empty((B, 1 << 10), dtype=torch.complex128, device=cuda)
    rc = _static(lib, prog, theta, out)
    assert rc == -2
    assert "static array holds" in _lib.last_error()
    small = prog.run(theta[:2], 0)
    rc = _static(lib, prog, theta[:2], out[:2])
    assert rc == 0
    torch.cuda.synchronize()
    assert float((out[:2] - small).abs().max()) < AMP_TOL
