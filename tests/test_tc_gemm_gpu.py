"""bemgpu_cgemm: the complex64 product of the mixed-precision LU, solve and
trace (the reference's addproduct -> zgemm, src/util/MatrixOperations.cpp:70-74).

The tensor-core engine (tcgen05, bf16x3 slices, six products, FP32
accumulation) and the FP32 FMA engine are both held to the complex128 product
of the same complex64 inputs: every entry within 2e-6 of sum_k |a_ik| |b_kj|
(FP32 class; the FP32 FMA reference itself sits near 1e-7)."""
import ctypes

import numpy as np
import pytest

from bem_gb300 import _lib, api

pytestmark = pytest.mark.gpu
TOL = 2e-6


def _rand(rng, shape, scale=1.0):
    return (scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))).astype(np.complex64)


def _gemm(A, B, C0, accumulate, engine, lda_pad=0, ldb_pad=0, ldc_pad=0):
    import torch
    ctx = api.default_context()
    A, B, C0 = (np.asarray(x, dtype=np.complex64) for x in (A, B, C0))
    m, k = A.shape
    n = B.shape[1]
    assert B.shape[0] == k and C0.shape == (m, n)
    lda, ldb, ldc = m + lda_pad, k + ldb_pad, m + ldc_pad
    dA = torch.zeros((k, lda), dtype=torch.complex64, device="cuda")
    dB = torch.zeros((n, ldb), dtype=torch.complex64, device="cuda")
    dC = torch.zeros((n, ldc), dtype=torch.complex64, device="cuda")
    dA[:, :m] = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB[:, :k] = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC[:, :m] = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
    torch.cuda.synchronize()
    rc = _lib.load().bemgpu_cgemm(ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), lda,
                                  ctypes.c_void_p(dB.data_ptr()), ldb, ctypes.c_void_p(dC.data_ptr()), ldc,
                                  int(accumulate), engine)
    assert rc == 0, _lib.load().bemgpu_ctx_last_error(ctx.handle)
    out = dC.cpu().numpy()
    assert np.all(out[:, m:] == 0), "wrote outside the m rows of C"
    return out[:, :m].T


def _check(A, B, C0, accumulate, got):
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    if accumulate:
        ref = ref + C0.astype(np.complex128)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + (np.abs(C0) if accumulate else 0)
    err = np.max(np.abs(got - ref) / scale)
    return err


@pytest.mark.parametrize("m,n,k", [(64, 64, 16), (100, 130, 37), (257, 129, 200), (1000, 384, 320)])
@pytest.mark.parametrize("engine", [1, 2])
def test_cgemm_engines_match_complex128(m, n, k, engine):
    pytest.importorskip("torch")
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A, B, C0 = _rand(rng, (m, k)), _rand(rng, (k, n)), _rand(rng, (m, n))
    for acc in (0, 1):
        got = _gemm(A, B, C0, acc, engine)
        err = _check(A, B, C0, acc, got)
        assert err < TOL, (engine, acc, err)


def test_tensor_core_gemm_leading_dimensions_and_dynamic_range():
    """Strided operands (lda, ldb, ldc > rows) and entries spanning 1e-6..1e6,
    the spread of an impedance block's L and K terms.  With one dominant term
    per sum, the FP32 accumulator's per-add rounding over the 6 x 2k partial
    products is what remains: held to 1e-5 (the sequential FP32 bound is
    ~2k x 6 x 2^-24 = 1e-4), FMA engine alongside for comparison."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    m, n, k = 300, 200, 150
    A = _rand(rng, (m, k)) * (10.0 ** rng.uniform(-6, 6, (m, k))).astype(np.float32)
    B = _rand(rng, (k, n)) * (10.0 ** rng.uniform(-3, 3, (k, n))).astype(np.float32)
    C0 = _rand(rng, (m, n))
    got = _gemm(A, B, C0, 1, 1, lda_pad=5, ldb_pad=3, ldc_pad=7)
    fma = _gemm(A, B, C0, 1, 2, lda_pad=5, ldb_pad=3, ldc_pad=7)
    assert _check(A, B, C0, 1, fma) < 1e-5
    assert _check(A, B, C0, 1, got) < 1e-5


def test_tensor_core_gemm_is_deterministic():
    pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    A, B, C0 = _rand(rng, (512, 256)), _rand(rng, (256, 256)), _rand(rng, (512, 256))
    a = _gemm(A, B, C0, 1, 1)
    b = _gemm(A, B, C0, 1, 1)
    assert np.array_equal(a, b)


def _gemm64(A, B, C0, accumulate, engine):
    import torch
    ctx = api.default_context()
    A, B = (np.asarray(x, dtype=np.complex64) for x in (A, B))
    C0 = np.asarray(C0, dtype=np.complex128)
    m, k = A.shape
    n = B.shape[1]
    assert B.shape[0] == k and C0.shape == (m, n)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
    torch.cuda.synchronize()
    rc = _lib.load().bemgpu_cgemm_acc64(ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), m,
                                        ctypes.c_void_p(dB.data_ptr()), k, ctypes.c_void_p(dC.data_ptr()), m,
                                        int(accumulate), engine)
    assert rc == 0, _lib.load().bemgpu_ctx_last_error(ctx.handle)
    return dC.cpu().numpy().T


@pytest.mark.parametrize("m,n,k", [(64, 64, 16), (130, 70, 33), (600, 200, 2000)])
@pytest.mark.parametrize("engine", [1, 2])
def test_acc64_residual_product(m, n, k, engine):
    """The refinement residual's product: complex64 operands, complex128
    result.  Tensor cores: operands rounded (to nearest) to 25-bit block fixed
    point, block products summed exactly, so each product carries ~2^-24 of
    its blocks' largest magnitudes, unbiased; FMA engine: FP32 products, short
    FP32 runs.  Short sums sit near 2^-24 of sum |a| |b|, long ones far below
    as the unbiased errors average out."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(m + 11 * n + k)
    A, B = _rand(rng, (m, k)), _rand(rng, (k, n))
    C0 = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n)))
    for acc in (0, 1):
        got = _gemm64(A, B, C0, acc, engine)
        ref = A.astype(np.complex128) @ B.astype(np.complex128) + (C0 if acc else 0)
        scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
        err = np.max(np.abs(got - ref) / scale)
        assert err < (3e-7 if k < 256 else 2e-8), (engine, acc, err)


def test_acc64_beats_fp32_accumulation_on_long_sums():
    """K = 8192: the compensated product's error stays well below the plain
    FP32-accumulated tensor-core product's."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    m, n, k = 256, 128, 8192
    A, B = _rand(rng, (m, k)), _rand(rng, (k, n))
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    e64 = np.max(np.abs(_gemm64(A, B, np.zeros((m, n)), 0, 1) - ref) / scale)
    e32 = np.max(np.abs(_gemm(A, B, np.zeros((m, n), np.complex64), 0, 1) - ref) / scale)
    assert e64 < 2e-8 and e64 < 0.25 * e32, (e64, e32)


def _zgemm_exact(A, B, C0, accumulate, slices):
    import torch
    ctx = api.default_context()
    A, B, C0 = (np.asarray(x, dtype=np.complex128) for x in (A, B, C0))
    m, k = A.shape
    n = B.shape[1]
    assert B.shape[0] == k and C0.shape == (m, n)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
    torch.cuda.synchronize()
    rc = _lib.load().bemgpu_zgemm_exact(ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), m,
                                        ctypes.c_void_p(dB.data_ptr()), k, ctypes.c_void_p(dC.data_ptr()), m,
                                        int(accumulate), slices)
    assert rc == 0, _lib.load().bemgpu_ctx_last_error(ctx.handle)
    return dC.cpu().numpy().T


@pytest.mark.parametrize("m,n,k", [(64, 64, 16), (100, 70, 37), (300, 200, 1000)])
@pytest.mark.parametrize("slices", [4, 5])
def test_exact_gemm_matches_fp64(m, n, k, slices):
    """Block fixed point with `slices` slices: each entry is represented to
    2^(-8 slices - 1) of its 16-entry K-block's largest magnitude and the
    tensor cores sum the slice products exactly, so the product is within a
    few 2^(-8 slices) of sum_k |a| |b| -- far beyond FP32 for 5 slices."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(m * 3 + n + k + slices)
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    C0 = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    scale = np.abs(A) @ np.abs(B)
    tol = {4: 2e-9, 5: 1e-11}[slices]
    for acc in (0, 1):
        got = _zgemm_exact(A, B, C0, acc, slices)
        ref = A @ B + (C0 if acc else 0)
        err = np.max(np.abs(got - ref) / scale)
        assert err < tol, (slices, acc, err)


def test_exact_gemm_dynamic_range_and_scaling():
    """Entries of A spanning 1e-8..1e8 along its rows, an overall scale of
    1e-200 (the per-matrix power-of-two scaling) and a zero block: the error
    stays at 2^-41 of each K-block's largest term."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    m, n, k = 256, 128, 512
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))) * 10.0 ** rng.uniform(-8, 8, (m, k))
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    A[:, 32:64] = 0
    A *= 1e-200
    got = _zgemm_exact(A, B, np.zeros((m, n)), 0, 5)
    ref = A @ B
    scale = np.abs(A) @ np.abs(B)
    assert np.max(np.abs(got - ref) / scale) < 1e-9


@pytest.mark.parametrize("m,n,k", [(64, 64, 16), (130, 70, 300), (300, 200, 1000)])
def test_exact_gemm_with_quantized_b(m, n, k):
    """B quantized in place to its 3-slice block fixed point, A in 5 slices:
    the returned B differs from the input by at most ~2^-25 of its blocks'
    maxima, and A times that quantized B is exact to ~2^-40 of the blocks'
    maxima products (all 12 slice products of level <= 4 kept)."""
    import torch
    rng = np.random.default_rng(m + 7 * n + k)
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * np.exp(rng.uniform(-8, 8, (k, n)))
    C0 = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    ctx = api.default_context()
    for acc in (0, 1):
        dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
        dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
        dC = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
        torch.cuda.synchronize()
        rc = _lib.load().bemgpu_zgemm_exact_quantized(ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), m,
                                                      ctypes.c_void_p(dB.data_ptr()), k,
                                                      ctypes.c_void_p(dC.data_ptr()), m, acc)
        assert rc == 0, _lib.load().bemgpu_ctx_last_error(ctx.handle)
        Bq = dB.cpu().numpy().T
        C = dC.cpu().numpy().T
        assert np.max(np.abs(Bq - B)) <= 2.0 ** -23 * np.max(np.abs(B)), "quantization beyond its bound"
        ref = A @ Bq + (C0 if acc else 0)
        # the bound is per 64-deep K block, relative to the block maxima of a
        # row of A and a column of B (B spans 7 decades here)
        scale = k * np.outer(np.abs(A).max(axis=1), np.abs(Bq).max(axis=0))
        err = np.max(np.abs(C - ref) / scale)
        assert err < 2.0 ** -38, (acc, err)


def test_tensor_flop_counts_per_product():
    """bemgpu_prof_query_tensor reports the bf16 slice products each product
    issued: 6 per complex MAC for the bf16x3 complex64 product, 15 / 10 / 6
    for the exact product of 5 / 4 / 3 slices, 12 for 5 slices times a
    3-slice quantized B; the FMA engine issues none."""
    import torch
    ctx = api.default_context()
    L = _lib.load()
    trace = _lib.K_NAMES.index("trace")
    rng = np.random.default_rng(11)
    m, n, k = 96, 80, 64

    def counts(run):
        L.bemgpu_prof_enable(ctx.handle, 1)
        run()
        nl, ms, fl, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        tf = ctypes.c_double()
        assert L.bemgpu_prof_query(ctx.handle, trace, ctypes.byref(nl), ctypes.byref(ms), ctypes.byref(fl),
                                   ctypes.byref(by)) == 0
        assert L.bemgpu_prof_query_tensor(ctx.handle, trace, ctypes.byref(tf)) == 0
        L.bemgpu_prof_enable(ctx.handle, 0)
        return fl.value, tf.value

    A32, B32 = _rand(rng, (m, k)), _rand(rng, (k, n))
    fl, tf = counts(lambda: _gemm(A32, B32, np.zeros((m, n), np.complex64), 0, 1))
    assert fl == 8.0 * m * n * k and tf == 6 * fl
    fl, tf = counts(lambda: _gemm(A32, B32, np.zeros((m, n), np.complex64), 0, 2))
    assert fl == 8.0 * m * n * k and tf == 0
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    for slices, products in ((5, 15), (4, 10), (3, 6)):
        fl, tf = counts(lambda: _zgemm_exact(A, B, np.zeros((m, n)), 0, slices))
        assert fl == 8.0 * m * n * k and tf == products * fl, (slices, tf / fl)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    fl, tf = counts(lambda: L.bemgpu_zgemm_exact_quantized(ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), m,
                                                           ctypes.c_void_p(dB.data_ptr()), k,
                                                           ctypes.c_void_p(dC.data_ptr()), m, 0))
    assert fl == 8.0 * m * n * k and tf == 12 * fl


@pytest.mark.parametrize("slices", [3, 4, "quantized"])
def test_exact_gemm_wide_and_narrow_tiles_agree(slices):
    """The 128 x 128-tile exact product (BEMGPU_TUNE_EX_WIDE: 3 x 3, 4 x 4,
    5 x 3 and 5 x 2 slices on large grids) against the 128 x 64-tile one on
    ragged shapes with several M and N tiles and many exponent blocks.  The
    quantized 5 x 3 product keeps levels 0..2 exact in both, so they differ
    only by the FP32 rounding of the level-3/4 sums (one buffer or two), far
    below its 2^-40; the wide 3 x 3 and 4 x 4 products sum level 2 in FP32
    too (2^-40 of the block maxima products, below their own truncation at
    2^-24 and 2^-32)."""
    quantized = slices == "quantized"
    import torch
    L = _lib.load()
    ctx = api.default_context()
    rng = np.random.default_rng(11 + quantized)
    m, n, k = 300, 200, 1000
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * np.exp(rng.uniform(-4, 4, (k, n)))
    C0 = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    scale = k * np.outer(np.abs(A).max(axis=1), np.abs(B).max(axis=0))

    def run():
        dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
        dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
        dC = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
        torch.cuda.synchronize()
        args = (ctx.handle, m, n, k, ctypes.c_void_p(dA.data_ptr()), m, ctypes.c_void_p(dB.data_ptr()), k,
                ctypes.c_void_p(dC.data_ptr()), m, 1)
        rc = L.bemgpu_zgemm_exact_quantized(*args) if quantized else L.bemgpu_zgemm_exact(*args, slices)
        assert rc == 0, L.bemgpu_ctx_last_error(ctx.handle)
        return dC.cpu().numpy().T

    try:
        assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_EX_WIDE, 0) == _lib.OK
        narrow = run()
        # 2: wide tiles whatever the grid (this one is below the 4-wave threshold)
        assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_EX_WIDE, 2) == _lib.OK
        wide = run()
    finally:
        L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_EX_WIDE, 1)
    assert np.max(np.abs(wide - narrow) / scale) < (2.0 ** -44 if quantized else 2.0 ** -36)
    assert not np.array_equal(wide, np.asarray(C0, dtype=np.complex128))
