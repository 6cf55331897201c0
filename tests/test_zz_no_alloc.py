"""The no-alloc surrogate inference entry point, called through the C-ABI.

izem_mlp_forward_noalloc serves callers that cannot allocate device memory
while they run (a solver whose own arena already holds the GPU's memory, or
that calls the surrogate inside its time-step loop, where cudaMalloc would
synchronise the device).  It keeps its activations in one fixed device array
shared by every call, so these tests check that two calls in a row -- the
second smaller than the first, with the first call's data still in the array
-- give the same outputs as izem_mlp_forward (both run the tensor-core
inference kernel on the same BF16 inputs, so the outputs are compared bit
for bit), and that requests above the array's capacity are refused.

This file is collected last so that it also runs after every other test."""
import ctypes as C

import numpy as np
import pytest

from phd_gb300 import capi
from phd_gb300.izem import load_library
from phd_gb300.surrogate import Surrogate

pytestmark = pytest.mark.gpu

MAX_ROWS = 4096   # IZEM_MLP_NOALLOC_MAX_ROWS in include/izem_gpu.h


def _entry():
    f = load_library().izem_mlp_forward_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_forward_matches_forward_on_two_calls():
    torch = pytest.importorskip("torch")
    s = Surrogate(seed=21)
    f = _entry()
    rng = np.random.Generator(np.random.PCG64(5))
    for M in (MAX_ROWS, 1500):
        x = rng.standard_normal((M, 12)).astype(np.float32)
        ref = s.forward(x)
        dx = torch.from_numpy(x).to("cuda:0")
        dy = torch.full((M, 10), float("nan"), dtype=torch.float32, device="cuda:0")
        torch.cuda.synchronize()
        rc = f(s.h, M, dx.data_ptr(), dy.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == capi.OK, rc
        y = dy.cpu().numpy()
        assert np.isfinite(y).all()
        assert np.array_equal(y, ref), (M, np.abs(y - ref).max())


def test_noalloc_forward_refuses_sizes_above_capacity():
    torch = pytest.importorskip("torch")
    s = Surrogate(seed=22)
    f = _entry()
    dx = torch.zeros((8, 12), dtype=torch.float32, device="cuda:0")
    dy = torch.zeros((8, 10), dtype=torch.float32, device="cuda:0")
    assert f(s.h, MAX_ROWS + 1, dx.data_ptr(), dy.data_ptr(), None) == capi.ERR_TOO_LARGE
    assert f(s.h, 0, dx.data_ptr(), dy.data_ptr(), None) == capi.ERR_ARG
