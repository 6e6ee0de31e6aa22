"""The allocation-free Gram entry point (ithaca_gpu_pod_gram_noalloc) against ithaca_gpu_pod_gram.

Callers that cannot allocate device memory where they need S^T S (a host whose device
memory is reserved up front in its own pool, or a loop that must not stall on the
device-wide synchronisation of cudaFree) call the
no-allocation variant with their own device input and output; its split-K scratch is a
fixed 2 MiB device array inside the library (ns <= 128). This file is collected last so
that a run stopping at the first failure has already run every other test; it passes alone
in a fresh process and after the others. Both entry points compute the same FP64 product
with different split counts, so they agree to 1e-13 relative.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _call_noalloc(S, C, stream):
    from ithaca_gpu import _capi
    lib = _capi.lib()
    fn = lib.ithaca_gpu_pod_gram_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    N, ns = S.shape[1], S.shape[0]  # S is stored snapshot-major: row j of S is snapshot j
    rc = fn(N, ns, ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(stream))
    return rc


def test_noalloc_gram_matches_gram_twice():
    from ithaca_gpu import _capi, pod
    from ithaca_gpu.operators import Context
    ctx = Context(0)
    rng = np.random.default_rng(12)
    for N, ns in ((70001, 96), (3001, 128)):
        Sh = rng.standard_normal((N, ns))
        ref = pod.gram(ctx, Sh)  # the existing entry point (allocates its scratch)
        S = torch.from_numpy(np.ascontiguousarray(Sh.T)).cuda()  # column-major N x ns on the device
        stream = torch.cuda.current_stream().cuda_stream
        for _ in range(2):  # two calls in a row share the scratch array
            C = torch.full((ns, ns), float("nan"), dtype=torch.float64, device="cuda")
            assert _call_noalloc(S, C, stream) == _capi.OK, _capi.last_error()
            torch.cuda.synchronize()
            got = C.cpu().numpy().T  # column-major result
            assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-13


def test_noalloc_gram_rejects_too_many_snapshots():
    from ithaca_gpu import _capi
    S = torch.zeros((129, 16), dtype=torch.float64, device="cuda")
    C = torch.zeros((129, 129), dtype=torch.float64, device="cuda")
    rc = _call_noalloc(S, C, torch.cuda.current_stream().cuda_stream)
    assert rc == _capi.ERR_ARG
    assert "exceeds" in _capi.last_error()
