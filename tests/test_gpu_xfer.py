"""State transfers through the C ABI: izem_gpu_upload_state and
izem_gpu_download_state move pinned host arrays with the SMs (16-byte
loads and stores over the host link) and pageable or unaligned ones with
cudaMemcpyAsync.  Every path must give the same bytes."""
import numpy as np
import pytest

import workloads as W
from phd_gb300.izem import IzemGPU

pytestmark = pytest.mark.gpu


def _pinned(shape, dtype, offset=0):
    """A Fortran-ordered host array in page-locked memory, starting `offset`
    bytes into its allocation."""
    torch = pytest.importorskip("torch")
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    buf = torch.empty(n + offset, dtype=torch.uint8).pin_memory().numpy()
    return np.ndarray(shape, dtype=dtype, buffer=buf, offset=offset, order="F")


def _gpu(cfg, thd, adi, dxi, st):
    g = IzemGPU(cfg, thd, adi)
    g.set_grid(*dxi)
    g.upload(**st)
    return g


@pytest.mark.parametrize("offset", [0, 8])
def test_pinned_transfers_give_the_same_bytes(offset):
    """Upload from pinned arrays (SM copy when 16-byte aligned, copy engine at
    an 8-byte offset), download into pinned arrays, against the pageable
    path; the sensor's byte count (18 x 18 x 14 = 4536) leaves a tail that is
    not a multiple of 16."""
    cfg, thd, adi, dxi, st, info, orc = W.case("mix", 12)
    rng = np.random.Generator(np.random.PCG64(3))
    st["shock_sensor"][...] = (rng.random(st["shock_sensor"].shape) < 0.3).astype(np.uint8)
    g = _gpu(cfg, thd, adi, dxi, st)
    ref = g.download()
    # a different state on the device, then the pinned upload over it
    g.upload(**{k: (np.zeros_like(a)) for k, a in st.items()})
    pinned = {}
    for k, a in ref.items():
        pinned[k] = _pinned(a.shape, a.dtype, offset)
        pinned[k][...] = a
    g.set_kernel_timing(True)
    g.upload(**pinned)
    out = {k: _pinned(a.shape, a.dtype, offset) for k, a in ref.items()}
    got = g.download(out=out)
    kt = g.kernel_times()
    g.close()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k
    if offset == 0:
        assert "host_xfer" in kt and kt["host_xfer"][0] == 12   # six arrays each way
    else:
        assert "host_xfer" not in kt


def test_pinned_round_trip_after_steps():
    """Two RK3 steps between a pinned upload and a pinned download give the
    bytes that the pageable path gives."""
    cfg, thd, adi, dxi, st, info, orc = W.case("tgv", 12)
    dt4, dt = orc.timestep(W.copy(st))
    out = []
    for pinned in (False, True):
        g = IzemGPU(cfg, thd, adi)
        g.set_grid(*dxi)
        src = {k: a for k, a in st.items()}
        if pinned:
            src = {}
            for k, a in st.items():
                src[k] = _pinned(a.shape, a.dtype)
                src[k][...] = a
        g.upload(**src)
        for _ in range(2):
            g.rk3(dt)
        dst = None
        if pinned:
            dst = {k: _pinned(a.shape, a.dtype) for k, a in st.items()}
        out.append(g.download(out=dst))
        g.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
