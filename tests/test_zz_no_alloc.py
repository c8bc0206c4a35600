"""bt_sample_noalloc: the allocation-free sampling entry point.

Some callers cannot let a library allocate device memory: a host framework's
memory pool (CUDA.jl, PyTorch) may own nearly all of HBM, so a library-side
cudaMalloc can fail and a cudaFree stalls every stream, and code being recorded
into a CUDA graph cannot have cudaMalloc/cudaFree captured.  This entry point
takes the state, the draws and the output as the caller's device buffers and
keeps its own scratch in a fixed device array.  The test calls it through the C
ABI twice in a row (different sizes, precisions and draws) and requires the
same shots as bt_sample, which is exact for given uniforms.  Collected last so
that a failure here does not hide the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def test_sample_noalloc_matches_bt_sample_twice(ctx):
    import torch

    import bluetangle_gpu as bt
    from bluetangle_gpu import _lib as L

    lib = L.lib()
    own = bt.Context(0, seed=777)
    try:
        rng = np.random.default_rng(808)
        stream = torch.cuda.current_stream().cuda_stream
        for call, (n, prec, shots) in enumerate([(12, "c128", 4096), (10, "c64", 3000)]):
            psi = rstate(rng, n)
            st = bt.state_from(psi, prec, ctx=own)
            u = rng.random(shots)
            d_u = torch.tensor(u, dtype=torch.float64, device="cuda")
            d_out = torch.empty(shots, dtype=torch.int64, device="cuda")
            own.synchronize()
            rc = lib.bt_sample_noalloc(lib.bt_state_device_ptr(st.h), n, L.BT_PREC_C64 if prec == "c64" else L.BT_PREC_C128,
                                       shots, ctypes.c_void_p(d_u.data_ptr()), 777, 0,
                                       ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream))
            L.check(rc)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            ref = np.empty(shots, dtype=np.int64)
            uu = np.ascontiguousarray(u)
            own.check(lib.bt_sample(st.h, 0, shots, uu.ctypes.data_as(ctypes.c_void_p), 0,
                                    ref.ctypes.data_as(ctypes.c_void_p)))
            assert np.array_equal(got, ref), f"call {call}: shots differ"
            # the on-device Philox path with the ctx's key reproduces bt_sample's stream
            rc = lib.bt_sample_noalloc(lib.bt_state_device_ptr(st.h), n, L.BT_PREC_C64 if prec == "c64" else L.BT_PREC_C128,
                                       shots, None, 777, 31 + call, ctypes.c_void_p(d_out.data_ptr()),
                                       ctypes.c_void_p(stream))
            L.check(rc)
            torch.cuda.synchronize()
            assert np.array_equal(d_out.cpu().numpy(), bt.sample(st, shots, seed=31 + call))
            st.free()
        # sizes beyond the static scratch are rejected with a clear error
        rc = lib.bt_sample_noalloc(ctypes.c_void_p(d_u.data_ptr()), 29, L.BT_PREC_C64, 1, None, 0, 0,
                                   ctypes.c_void_p(d_out.data_ptr()), None)
        assert rc == L.BT_ERR_BAD_ARG
        assert b"28" in lib.bt_last_error(None)
    finally:
        own.close()
