"""sphx_exclusive_scan_u32_noalloc: the exclusive scan for callers that cannot allocate
device memory while they run (their device memory belongs to another allocator, or their
loop must not pay cudaMalloc's device-wide synchronisation).  It keeps its scratch in a
fixed device array of the library, shared by every call.

Checked through the C ABI against the allocating sphx_exclusive_scan_u32 (exact integer
equality) on two calls in a row, the second smaller than the first so that stale scratch
contents of the first call would show; sizes past the fixed maximum are rejected.  This
file is collected last, and passes alone in a fresh process as well as after the rest.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_scan_matches_allocating_scan_on_two_calls():
    torch = pytest.importorskip("torch")
    from sphinxsys_gb300 import native as N

    lib = N.load()
    ctx = C.c_void_p()
    N.call("sphx_ctx_create", 0, None, C.byref(ctx))
    try:
        stream = C.c_void_p()
        N.call("sphx_ctx_stream", ctx, C.byref(stream))
        rng = np.random.default_rng(7)
        for n in (3_000_001, 4_097):
            v = torch.tensor(rng.integers(0, 50, size=n).astype(np.int32), device="cuda")
            out_ref = torch.empty_like(v)
            out_new = torch.full_like(v, -1)
            torch.cuda.synchronize()
            t_ref, t_new = C.c_uint32(), C.c_uint32()
            N.call("sphx_exclusive_scan_u32", ctx, C.c_void_p(v.data_ptr()), C.c_void_p(out_ref.data_ptr()), n,
                   C.byref(t_ref))
            N.call("sphx_exclusive_scan_u32_noalloc", stream, C.c_void_p(v.data_ptr()),
                   C.c_void_p(out_new.data_ptr()), n, C.byref(t_new))
            N.call("sphx_ctx_synchronize", ctx)
            assert torch.equal(out_ref, out_new)
            assert t_new.value == t_ref.value == int(v.sum().item())
        too_big = 67_108_864 + 1
        st = lib.sphx_exclusive_scan_u32_noalloc(stream, C.c_void_p(v.data_ptr()), C.c_void_p(out_new.data_ptr()),
                                                 too_big, None)
        assert st == 1 and b"at most" in lib.sphx_last_error()
    finally:
        N.call("sphx_ctx_destroy", ctx)
