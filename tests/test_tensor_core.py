"""Known-answer tests of the tcgen05 product the radiance-cache kernels are built on:
D[128 x n] = A[128 x k] * B[n x k]^T with BF16 operands and FP32 accumulation, against
numpy in FP64 on the same BF16 values (tolerance: FP32 accumulation error, 1e-5 of the sum
of absolute products)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    from oracle.mlp import bf16
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


@pytest.mark.parametrize("n,k", [(16, 16), (64, 64), (64, 96), (16, 64), (128, 128), (256, 32), (48, 80)])
def test_mma_known_answer(built, n, k):
    import narvalengine_gb300 as ne
    rng = np.random.default_rng(n * 1000 + k)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    ab, bb = bf16_bits(a), bf16_bits(b)
    af = (ab.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    bf = (bb.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    want = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    ctx = ne.Context(0)
    try:
        d = np.empty((128, n), np.float32)
        st = ne.library().ne_debug_mma(ctx._h, ab.ctypes.data, bb.ctypes.data, n, k, d.ctypes.data)
        assert st == 0, ctx.error()
    finally:
        ctx.close()
    err = np.abs(d - want) / (scale + 1e-30)
    assert err.max() < 1e-5, f"max scaled error {err.max():.3e}; first rows:\n{d[:2, :8]}\n{want[:2, :8]}"


def test_mma_rejects_bad_shapes(built):
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    try:
        z = np.zeros(128 * 256, np.uint16)
        d = np.zeros(128 * 256, np.float32)
        for n, k in [(8, 16), (16, 8), (272, 16), (16, 144)]:
            assert ne.library().ne_debug_mma(ctx._h, z.ctypes.data, z.ctypes.data, n, k, d.ctypes.data) == -1
    finally:
        ctx.close()


def test_bounded_wait_gives_up_and_releases_tensor_memory(built):
    """Failure detection without a fault: a block waits on an mbarrier that nothing signals,
    gives up after a short poll limit and reports NE_ERR_TIMEOUT; its tensor memory is
    released, so products on the same context still run and are right afterwards (a block
    that kept its allocation would leave the next allocations on that SM short)."""
    import narvalengine_gb300 as ne
    from narvalengine_gb300 import _abi
    ctx = ne.Context(0)
    try:
        for polls in (1, 64, 4096):
            st = ne.library().ne_debug_wait_timeout(ctx._h, polls)
            assert st == _abi.NE_ERR_TIMEOUT, (polls, st, ctx.error())
            assert "gave up" in ctx.error()
        assert ne.library().ne_debug_wait_timeout(ctx._h, 0) == _abi.NE_ERR_INVALID_ARG
        rng = np.random.default_rng(7)
        for _ in range(3):
            a = rng.normal(size=(128, 64)).astype(np.float32)
            b = rng.normal(size=(256, 64)).astype(np.float32)
            ab, bb = bf16_bits(a), bf16_bits(b)
            af = (ab.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
            bf = (bb.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
            d = np.empty((128, 256), np.float32)
            st = ne.library().ne_debug_mma(ctx._h, ab.ctypes.data, bb.ctypes.data, 256, 64, d.ctypes.data)
            assert st == 0, ctx.error()
            err = np.abs(d - af @ bf.T) / (np.abs(af) @ np.abs(bf).T + 1e-30)
            assert err.max() < 1e-5
    finally:
        ctx.close()


@pytest.mark.parametrize("layout", [1, 2, 3])
@pytest.mark.parametrize("n,k", [(16, 16), (64, 64), (32, 48), (64, 16)])
def test_mma_mn_major_known_answer(built, layout, n, k):
    """Operands staged MN-major (bit 0: A, bit 1: B) and read through transposed descriptors:
    the layout the backward pass uses to read a row-per-sample tile as its transpose."""
    import narvalengine_gb300 as ne
    rng = np.random.default_rng(n * 100 + k + layout)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    ab, bb = bf16_bits(a), bf16_bits(b)
    af = (ab.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    bf = (bb.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    want = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    ctx = ne.Context(0)
    try:
        d = np.empty((128, n), np.float32)
        st = ne.library().ne_debug_mma_layout(ctx._h, ab.ctypes.data, bb.ctypes.data, n, k, layout, d.ctypes.data)
        assert st == 0, ctx.error()
    finally:
        ctx.close()
    err = np.abs(d - want) / (scale + 1e-30)
    assert err.max() < 1e-5, f"max scaled error {err.max():.3e}"
