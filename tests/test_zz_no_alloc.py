"""qcmg_multidot_noalloc against qcmg_multidot, through the C ABI.

The allocation-free entry point serves callers that may not allocate device
memory (a framework owning the GPU through its own pool or a memory cap, or
code that must not allocate while other work runs); its partial sums live in
a fixed device array of the library.  The file name sorts last so the test
also runs after every other GPU test of the suite, and it builds everything
it needs itself, so it passes alone in a fresh process as well.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pyqcm_gb300 as pg
    from pyqcm_gb300 import _lib
    return torch, pg.lib(), _lib


def test_noalloc_multidot_matches_allocating_entry_point_twice_in_a_row():
    torch, lib, _lib = _setup()
    gen = torch.Generator(device="cuda").manual_seed(2024)
    stream = torch.cuda.Stream()
    for n, m in ((3_000_017, 9), (65_537, 64)):
        V = [torch.randn(n, dtype=torch.float64, device="cuda", generator=gen) for _ in range(m)]
        w = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        ptrs = torch.tensor([v.data_ptr() for v in V], dtype=torch.int64, device="cuda")
        ref = np.zeros(m)
        _lib.check(lib.qcmg_multidot(m, ptrs.data_ptr(), w.data_ptr(), n, _lib.ptr(ref), None))
        outs = [torch.full((m,), np.nan, dtype=torch.float64, device="cuda") for _ in range(2)]
        torch.cuda.synchronize()  # inputs and the NaN-filled outputs are ready for the other stream
        for out in outs:  # two calls in a row on one stream, no wait between them
            _lib.check(lib.qcmg_multidot_noalloc(m, ptrs.data_ptr(), w.data_ptr(), n,
                                                 out.data_ptr(), stream.cuda_stream))
        stream.synchronize()
        tol = 1e-12 * np.sqrt(n) * max(1.0, float(np.max(np.abs(ref))))
        for out in outs:
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert np.max(np.abs(got - ref)) <= tol, (n, m)


def test_noalloc_multidot_rejects_more_vectors_than_its_scratch():
    torch, lib, _lib = _setup()
    n, m = 1024, 65
    V = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(m)]
    ptrs = torch.tensor([v.data_ptr() for v in V], dtype=torch.int64, device="cuda")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = lib.qcmg_multidot_noalloc(m, ptrs.data_ptr(), w.data_ptr(), n, out.data_ptr(), None)
    assert rc == -1
    assert "at most 64 vectors" in _lib.last_error()
