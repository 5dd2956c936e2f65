"""glasma_gauss_noalloc: the Gauss-law measurement for callers that cannot allocate device memory
(inside another framework's graph capture, pool-owned memory, real-time loops).  Called through
the C ABI on device buffers the test owns, and checked against the handle-based glasma_gauss on
two calls in a row.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from soerenpragya3dglasma_gb300 import Lattice, _lib, build

pytestmark = pytest.mark.gpu


def device_layout(f, torch, dev):
    """Reference host layout (numpy) -> the library's device layout (component-major), on the GPU."""
    S = f["U"].shape[0] * f["U"].shape[1] * f["U"].shape[2]
    U = np.ascontiguousarray(f["U"].reshape(S, 27).T)              # [mu*9+k][s] complex
    E = np.ascontiguousarray(f["E"].reshape(S, 24).T)              # [mu*8+a][s]
    Jp = np.ascontiguousarray(f["JpStat"].reshape(S, 8).T)
    Jm = np.ascontiguousarray(f["JmStat"].reshape(S, 8).T)
    return [torch.from_numpy(x.view(np.float64) if x.dtype == np.complex128 else x).to(dev) for x in (U, E, Jp, Jm)]


def test_gauss_noalloc_matches_handle_twice():
    torch = pytest.importorskip("torch")
    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    N, a = (12, 10, 16), (1.0, 0.9, 1.1)
    for call, seed in enumerate((71, 72)):
        f = O.random_fields(N, seed)
        with Lattice(N, a) as lat:
            lat.upload_fields(f)
            mx, avg, prof = lat.gauss(profile=True)
        bufs = device_layout(f, torch, dev)
        res = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
        zp = torch.zeros(N[2], dtype=torch.float64, device=dev)
        st = lib.glasma_gauss_noalloc(*[b.data_ptr() for b in bufs], N[0], N[1], N[2], a[0], a[1], a[2], 1.0,
                                      res.data_ptr(), zp.data_ptr(), None)
        assert st == 0, call
        torch.cuda.synchronize()
        got = res.cpu().numpy()
        assert abs(got[0] - mx) <= 1e-12 * mx, call
        assert abs(got[1] - avg) <= 1e-12 * avg, call
        assert np.allclose(zp.cpu().numpy(), prof, rtol=1e-12, atol=0), call


def test_gauss_noalloc_rejects_oversized_lattice():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    st = lib.glasma_gauss_noalloc(p, p, p, p, 4, 4, 993, 1.0, 1.0, 1.0, 1.0, p, None, None)
    assert st == 2
    assert b"exceeds the maximum" in lib.glasma_last_error()


def test_gauss_noalloc_inside_graph_capture():
    """The use the entry point exists for: after one warm-up call, a call captured into a CUDA graph on
    the caller's stream (a capture fails on any allocation or synchronisation), replayed on new field
    data written into the same buffers, equals glasma_gauss on that data."""
    torch = pytest.importorskip("torch")
    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    N, a = (12, 10, 16), (1.0, 0.9, 1.1)
    f1, f2 = O.random_fields(N, 81), O.random_fields(N, 82)
    bufs = device_layout(f1, torch, dev)
    res = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    zp = torch.zeros(N[2], dtype=torch.float64, device=dev)
    s = torch.cuda.Stream(dev)
    args = [b.data_ptr() for b in bufs] + [N[0], N[1], N[2], a[0], a[1], a[2], 1.0, res.data_ptr(), zp.data_ptr(),
                                           ctypes.c_void_p(s.cuda_stream)]
    with torch.cuda.stream(s):
        assert lib.glasma_gauss_noalloc(*args) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = lib.glasma_gauss_noalloc(*args)
    assert st == 0
    for b, n in zip(bufs, device_layout(f2, torch, dev)):
        b.copy_(n)
    res.fill_(-1.0)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    with Lattice(N, a) as lat:
        lat.upload_fields(f2)
        mx, avg, prof = lat.gauss(profile=True)
    got = res.cpu().numpy()
    assert abs(got[0] - mx) <= 1e-12 * mx
    assert abs(got[1] - avg) <= 1e-12 * avg
    assert np.allclose(zp.cpu().numpy(), prof, rtol=1e-12, atol=0)
