"""Tensor-core (tcgen05, 3xTF32) Gram against an FP64 NumPy product.

The kernel stacks point chunks along the 128-row MMA operand and keeps the
diagonal blocks of the accumulator (``csrc/gram_tc.cu``); these cases cover
every stacking factor (a, b padded to 8, 16, 32, 64), ragged point counts
(the last stage partly out of range), one stage only, the unweighted form,
accumulation, row strides wider than the rows, the bench's 2M-point grid,
self-Grams (sums of one sign, where the accumulation error does not average
out) and several host threads at once.
Tolerance: 2e-6 of max |G|, the FP32 Gram tolerance of the eigensolver tests.
"""

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("n,a,b", [(1000, 16, 16), (4133, 5, 9), (100_000, 32, 32), (65_536, 64, 64),
                                   (50_001, 12, 24), (333, 1, 1), (77_777, 64, 8), (40_000, 8, 64),
                                   (2_097_152, 16, 16), (262_147, 33, 17)])
def test_tensor_core_gram_matches_fp64(n, a, b):
    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr, stream_ptr

    rng = np.random.default_rng(n + 7 * a + b)
    ld = (n + 3) // 4 * 4 + 4  # row stride wider than the row, 16-byte multiple
    A = np.zeros((a, ld), dtype=np.float32)
    B = np.zeros((b, ld), dtype=np.float32)
    A[:, :n] = rng.normal(size=(a, n))
    B[:, :n] = rng.normal(size=(b, n))
    A[:, n:] = np.nan  # never read
    B[:, n:] = np.nan
    w = rng.uniform(0.5, 2.0, n)
    Ad, Bd = torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda")
    wd = torch.tensor(w, device="cuda")
    out = torch.full((a, b), 7.0, dtype=torch.float64, device="cuda")
    wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    A64, B64 = A[:, :n].astype(np.float64), B[:, :n].astype(np.float64)
    ref = A64 @ (w[:, None] * B64.T)
    try:
        _lib.check(_lib.call("igd_gram_select", 1), "igd_gram_select")
        _lib.check(_lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(Ad), ld, b, ptr(Bd), ld, ptr(wd), ptr(out), 0,
                             ptr(ws), wsb, stream_ptr()), "igd_block_gram")
        assert _lib.call("igd_gram_last_path") == 1
        assert _rel(out.cpu().numpy(), ref) < 2e-6, _rel(out.cpu().numpy(), ref)
        # accumulate the unweighted product on top
        _lib.check(_lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(Ad), ld, b, ptr(Bd), ld, None, ptr(out), 1,
                             ptr(ws), wsb, stream_ptr()), "igd_block_gram")
        assert _lib.call("igd_gram_last_path") == 1
        assert _rel(out.cpu().numpy(), ref + A64 @ B64.T) < 4e-6
    finally:
        _lib.call("igd_gram_select", 0)
    assert _lib.error_flags(clear=True, stream=stream_ptr()) == 0


@pytest.mark.parametrize("n,a", [(300_000, 16), (2_097_152, 32), (1_000_003, 64)])
def test_tensor_core_self_gram_matches_fp64(n, a):
    """G = A W A^T: the diagonal sums terms of one sign, so errors that are biased
    (truncated splits, a non-nearest accumulation) add up instead of averaging out."""

    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr, stream_ptr

    ld = (n + 3) // 4 * 4
    g = torch.Generator(device="cuda").manual_seed(n + a)
    A = torch.zeros((a, ld), device="cuda")
    A[:, :n] = torch.randn((a, n), device="cuda", generator=g)
    w = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) + 0.5
    out = torch.empty((a, a), dtype=torch.float64, device="cuda")
    wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, a))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(_lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(A), ld, a, ptr(A), ld, ptr(w), ptr(out), 0,
                         ptr(ws), wsb, stream_ptr()), "igd_block_gram")
    assert _lib.call("igd_gram_last_path") == 1
    A64 = A[:, :n].double().cpu().numpy()
    ref = A64 @ (w.cpu().numpy()[:, None] * A64.T)
    print("self-Gram", n, a, _rel(out.cpu().numpy(), ref))
    assert _rel(out.cpu().numpy(), ref) < 2e-6, _rel(out.cpu().numpy(), ref)


def test_tensor_core_gram_same_as_cuda_core_path():
    """The automatic choice on a large grid is the tensor pipe; it and the pipelined
    CUDA-core kernel each stay within 2e-6 of the FP64 product."""

    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr, stream_ptr

    n, a, b = 1 << 20, 24, 24
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(a, n, device="cuda", generator=g)
    B = torch.randn(b, n, device="cuda", generator=g)
    w = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) + 0.5
    wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    outs = []
    for path in (0, 2):
        out = torch.empty((a, b), dtype=torch.float64, device="cuda")
        try:
            _lib.check(_lib.call("igd_gram_select", path), "igd_gram_select")
            _lib.check(_lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(A), n, b, ptr(B), n, ptr(w), ptr(out), 0,
                                 ptr(ws), wsb, stream_ptr()), "igd_block_gram")
            outs.append((_lib.call("igd_gram_last_path"), out.cpu().numpy()))
        finally:
            _lib.call("igd_gram_select", 0)
    assert outs[0][0] == 1 and outs[1][0] == 2
    A64, B64 = A.double().cpu().numpy(), B.double().cpu().numpy()
    ref = A64 @ (w.cpu().numpy()[:, None] * B64.T)
    for _, got in outs:
        assert _rel(got, ref) < 2e-6


def test_tensor_core_gram_concurrent_threads_mixed_shapes():
    """Host threads on their own streams run Grams of different shapes at once.

    The kernel's dynamic shared-memory size depends on the shape, and the limit
    that a launch needs is a process-wide attribute of the kernel: a thread with
    a small shape must not lower it under another thread's larger launch."""

    import concurrent.futures as cf

    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr

    n = 300_000
    shapes = [(8, 8), (64, 64), (16, 16), (32, 32), (5, 9), (64, 8)]
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.randn(64, n, device="cuda", generator=g)
    w = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) + 0.5
    torch.cuda.synchronize()
    A64, w64 = A.double().cpu().numpy(), w.cpu().numpy()

    def worker(t):
        stream = torch.cuda.Stream()
        errs = []
        with torch.cuda.stream(stream):
            for r in range(3):
                a, b = shapes[(t + r) % len(shapes)]
                wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
                ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
                out = torch.empty((a, b), dtype=torch.float64, device="cuda")
                _lib.check(_lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(A), n, b, ptr(A), n, ptr(w), ptr(out),
                                     0, ptr(ws), wsb, stream.cuda_stream), "igd_block_gram")
                assert _lib.call("igd_gram_last_path") == 1
                stream.synchronize()
                ref = A64[:a] @ (w64[:, None] * A64[:b].T)
                errs.append(_rel(out.cpu().numpy(), ref))
            assert _lib.error_flags(clear=True, stream=stream.cuda_stream) == 0
        return errs

    with cf.ThreadPoolExecutor(max_workers=len(shapes)) as ex:
        errs = [e for es in ex.map(worker, range(len(shapes))) for e in es]
    assert max(errs) < 2e-6, errs
