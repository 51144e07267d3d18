"""The allocation-free chi2 reduction (galario_reduce_chi2_noalloc_d).

It exists for callers that cannot let the library allocate GPU memory (device
memory owned by another allocator such as PyTorch's caching allocator, or
loops that cannot afford cudaFree's device-wide synchronisation).  The test
calls it through the C ABI on caller-owned device buffers, twice in a row with
different sizes (the second call must not see what the first left in the
shared scratch), and compares each result with the regular entry point
galario_reduce_chi2_d.  It also checks the size limit.  Kept in its own file,
collected last, so a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative chi2 tolerance of the double-precision tests
MAX_ND = 4096 * 4096


def _lib():
    from galario_gb300 import _lib
    L = _lib.lib()
    f = L.galario_reduce_chi2_noalloc_d
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _case(nd, seed):
    rng = np.random.default_rng(seed)
    re, im = rng.normal(0, 1e-3, nd), rng.normal(0, 1e-3, nd)
    w = rng.uniform(0.5, 1.5, nd) * 1e6
    vis = (rng.normal(0, 1e-3, nd) + 1j * rng.normal(0, 1e-3, nd)).astype(np.complex128)
    return re, im, w, vis


def test_no_alloc_reduce_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    g.double.use_gpu(0)
    L, f = _lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    for nd, seed in ((1_000_003, 1), (5_000, 2)):
        re, im, w, vis = _case(nd, seed)
        expected = g.double.reduce_chi2(re, im, w, vis)   # regular entry point, host buffers
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (re, im, w)]
        tv = torch.from_numpy(vis.view(np.float64).copy()).to(dev)
        st = f(nd, t[0].data_ptr(), t[1].data_ptr(), tv.data_ptr(), t[2].data_ptr(), out.data_ptr(),
               C.c_void_p(stream.cuda_stream))
        assert st == 0, L.galario_last_error()
        stream.synchronize()
        got = float(out.item())
        assert abs(got - expected) / abs(expected) <= TOL, (nd, got, expected)


def test_no_alloc_reduce_edge_sizes_and_cleanup():
    """nd = 0 writes 0; sizes that fill the last 4096-visibility block exactly
    agree with the regular entry point; a call after galario_cleanup() (which
    forgets the cached scratch address) looks the address up again."""
    torch = pytest.importorskip("torch")
    import galario_gb300 as g
    g.double.use_gpu(0)
    L, f = _lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    out = torch.full((1,), 7.0, dtype=torch.float64, device=dev)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    assert f(0, p, p, p, p, out.data_ptr(), C.c_void_p(stream.cuda_stream)) == 0, L.galario_last_error()
    stream.synchronize()
    assert float(out.item()) == 0.0
    for nd, seed, cleanup in ((4096, 3, False), (4096 * 5, 4, True), (4096 * 37, 5, False)):
        if cleanup:
            assert L.galario_cleanup() == 0
        re, im, w, vis = _case(nd, seed)
        expected = g.double.reduce_chi2(re, im, w, vis)
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (re, im, w)]
        tv = torch.from_numpy(vis.view(np.float64).copy()).to(dev)
        st = f(nd, t[0].data_ptr(), t[1].data_ptr(), tv.data_ptr(), t[2].data_ptr(), out.data_ptr(),
               C.c_void_p(stream.cuda_stream))
        assert st == 0, L.galario_last_error()
        stream.synchronize()
        got = float(out.item())
        assert abs(got - expected) / abs(expected) <= TOL, (nd, got, expected)


def test_no_alloc_reduce_rejects_misaligned_vis():
    """vis_dev is read 16 bytes at a time: a view starting at an odd double is
    rejected on the host, before anything is enqueued."""
    torch = pytest.importorskip("torch")
    L, f = _lib()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    assert p % 16 == 0
    st = f(4, p, p, p + 8, p, out.data_ptr(), None)
    assert st == 1  # GALARIO_EINVAL
    assert b"16-byte aligned" in L.galario_last_error()


def test_no_alloc_reduce_rejects_sizes_beyond_the_maximum():
    torch = pytest.importorskip("torch")
    L, f = _lib()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    st = f(MAX_ND + 1, p, p, p, p, p, None)
    assert st == 1  # GALARIO_EINVAL, nothing launched
    assert b"exceeds the maximum" in L.galario_last_error()
