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
    """Both entry points run the same kernels in the same fixed order, so the
    results agree bit for bit; after the first call (which may load the
    module and so reserve the scratch), further calls leave the device's free
    memory unchanged."""
    torch, lib, _lib = _setup()
    gen = torch.Generator(device="cuda").manual_seed(2024)
    stream = torch.cuda.Stream()
    for n, m in ((3_000_017, 9), (65_537, 64)):
        V = [torch.randn(n, dtype=torch.float64, device="cuda", generator=gen) for _ in range(m)]
        w = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        ptrs = torch.tensor([v.data_ptr() for v in V], dtype=torch.int64, device="cuda")
        ref = np.zeros(m)
        _lib.check(lib.qcmg_multidot(m, ptrs.data_ptr(), w.data_ptr(), n, _lib.ptr(ref), None))
        outs = [torch.full((m,), np.nan, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()  # inputs and the NaN-filled outputs are ready for the other stream
        _lib.check(lib.qcmg_multidot_noalloc(m, ptrs.data_ptr(), w.data_ptr(), n,
                                             outs[0].data_ptr(), stream.cuda_stream))
        stream.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for out in outs[1:]:  # two more calls in a row on one stream, no wait between them
            _lib.check(lib.qcmg_multidot_noalloc(m, ptrs.data_ptr(), w.data_ptr(), n,
                                                 out.data_ptr(), stream.cuda_stream))
        stream.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        for out in outs:
            got = out.cpu().numpy()
            assert np.array_equal(got, ref), (n, m)


def test_noalloc_multidot_accepts_an_empty_list():
    torch, lib, _lib = _setup()
    assert lib.qcmg_multidot_noalloc(0, None, None, 0, None, None) == 0


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
