"""Failure detection on the device without a GPU fault: the bounded waits of the persistent
batch give up after about a second, record the timeout in an error word the host reads, and
leave the CUDA context usable. A flag that nothing sets makes the wait run out."""
import time

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import assert_close, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_bounded_wait_reports_its_timeout_and_the_context_survives(gpu_lib):
    lib = R.load()
    t0 = time.time()
    st = lib.casadi_gb300_check_wait_timeout(R._stream_handle(None))
    elapsed = time.time() - t0
    assert st == -4, lib.casadi_gb300_last_error()
    assert b"bounded wait ran out" in lib.casadi_gb300_last_error()
    assert 0.2 < elapsed < 60.0
    # the context is still usable: a sweep runs and is right
    f = W.cartpole_step()
    n = 257
    args = W.cartpole_inputs(n, steps=1, seed=9)
    ct = R.CudaTape(f)
    got = ct.eval([torch.from_numpy(a).cuda() for a in args])
    want = O.eval(f.tape, args, n)
    assert_close(got[0].cpu().numpy(), want[0], "eval after the timeout",
                 bound=value_bounds(f.tape, args, n)[0])
    ct.sync()
