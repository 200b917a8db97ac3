"""idrs_rinprod_noalloc: the inner product for callers that cannot allocate
device memory (their GPU memory belongs to another allocator, or they forbid
allocation after start-up).  Checked through the C ABI against the
allocating entry point idrs_rinprod on the same device vectors, on two calls
in a row.  This file is collected last so that a failure here comes after
every other test has run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rinprod_noalloc_matches_rinprod(gpu):
    import torch
    lib = gpu.lib()
    n = 3_000_017  # not a multiple of the 4096-element chunk
    # an n x n handle for idrs_rinprod (identity pattern; only its size is used)
    rp = np.arange(1, n + 2, dtype=np.int32)
    ci = np.arange(1, n + 1, dtype=np.int32)
    A = gpu.Matrix(gpu.crs_format(n, n, rp, ci))
    A.set_pointer_mode(gpu.POINTER_DEVICE)
    gen = torch.Generator(device="cuda").manual_seed(4)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        u = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        v = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        torch.cuda.synchronize()
        st = lib.idrs_rinprod_noalloc(n, u.data_ptr(), v.data_ptr(), out.data_ptr(), None)
        assert st == 0, lib.idrs_last_error()
        torch.cuda.synchronize()
        ref = np.zeros(2)
        assert lib.idrs_rinprod(A.handle, u.data_ptr(), v.data_ptr(), ref.ctypes.data) == 0
        got = float(out.item())
        assert abs(got - ref[0]) <= 1e-12 * float(torch.linalg.norm(u) * torch.linalg.norm(v)), (call, got, ref[0])
        assert abs(got - float(torch.dot(u, v))) <= 1e-10 * abs(got) + 1e-9


def test_rinprod_noalloc_rejects_oversize(gpu):
    import torch
    lib = gpu.lib()
    small = torch.zeros(8, dtype=torch.float64, device="cuda")
    # rejected on the host before any launch: the buffers are never read
    st = lib.idrs_rinprod_noalloc((1 << 26) + 1, small.data_ptr(), small.data_ptr(), small.data_ptr(), None)
    assert st == 1 and b"no-allocation limit" in lib.idrs_last_error()


def test_rinprod_noalloc_rejects_host_pointers(gpu):
    """Pointers the GPU cannot use as device memory are refused on the host
    (cudaPointerGetAttributes) before any launch."""
    import torch
    lib = gpu.lib()
    host = np.ones(16)
    dev = torch.ones(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for args in ((host.ctypes.data, dev.data_ptr(), out.data_ptr()),
                 (dev.data_ptr(), dev.data_ptr(), host.ctypes.data)):
        st = lib.idrs_rinprod_noalloc(16, *args, None)
        assert st == 1 and b"device (or managed) pointers" in lib.idrs_last_error()
    # the entry point still works afterwards
    assert lib.idrs_rinprod_noalloc(16, dev.data_ptr(), dev.data_ptr(), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert float(out.item()) == 16.0
