"""Tensor-core building blocks (tcgen05.mma, TMEM, bulk-copied SW128 weight
images, split-BF16 products) against an FP64 matrix product."""
import ctypes as C

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def _bf16(x):
    x32 = np.asarray(x, np.float32)
    b = x32.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


@pytest.mark.parametrize("N,K", [(256, 64), (256, 256), (64, 256), (128, 100)])
def test_tc_gemm_single_and_split(lib, N, K):
    rng = np.random.default_rng(N + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    W = (rng.standard_normal((N, K)) / np.sqrt(K)).astype(np.float32)
    fp = C.POINTER(C.c_float)
    D0 = np.zeros((128, N), np.float32)
    D1 = np.zeros((128, N), np.float32)
    rc0 = lib.gbnde_tc_selftest(A.ctypes.data_as(fp), W.ctypes.data_as(fp), N, K, 0, D0.ctypes.data_as(fp))
    rc1 = lib.gbnde_tc_selftest(A.ctypes.data_as(fp), W.ctypes.data_as(fp), N, K, 1, D1.ctypes.data_as(fp))
    assert rc0 == 0 and rc1 == 0
    ref_bf16 = _bf16(A) @ _bf16(W).T
    ref = A.astype(np.float64) @ W.astype(np.float64).T
    scale = np.abs(ref).max()
    # one product: exact bf16 operands, FP32 accumulation
    assert np.abs(D0 - ref_bf16).max() / scale < 1e-5
    # five split products, emulated exactly (pieces are exact bf16 values):
    # W = Wh + Wl, A = Ah + Am + Al; products Wh.Ah + Wh.Am + Wl.Ah + Wh.Al + Wl.Am
    Wh = _bf16(W); Wl = _bf16(W - Wh)
    Ah = _bf16(A); Am = _bf16(A - Ah); Al = _bf16(A - Ah - Am)
    emul = Ah @ Wh.T + Am @ Wh.T + Ah @ Wl.T + Al @ Wh.T + Am @ Wl.T
    # (the tensor core accumulates with FP32 alignment truncation: ~2e-6 at K=256)
    assert np.abs(D1 - emul).max() / scale < 1e-5
    # and within the 16-bit weight truncation of the FP64 product
    assert np.abs(D1 - ref).max() / scale < 2e-5


@pytest.mark.parametrize("N", [64, 256])
def test_tc_gemm_mn_major_weight_gradient_form(lib, N):
    """D = G^T A with both operands stored trajectory-major (MN-major for the MMA),
    the layout of the weight-gradient products of the adjoint."""
    rng = np.random.default_rng(N)
    G = rng.standard_normal((128, 128)).astype(np.float32)
    A = rng.standard_normal((128, N)).astype(np.float32)
    fp = C.POINTER(C.c_float)
    D = np.zeros((128, N), np.float32)
    assert lib.gbnde_tc_selftest(G.ctypes.data_as(fp), A.ctypes.data_as(fp), N, 128, 2, D.ctypes.data_as(fp)) == 0
    Gh = _bf16(G); Gl = _bf16(G - Gh)
    Ah = _bf16(A); Al = _bf16(A - Ah)
    emul = Gh.T @ Ah + Gh.T @ Al + Gl.T @ Ah
    ref = G.astype(np.float64).T @ A.astype(np.float64)
    scale = np.abs(ref).max()
    assert np.abs(D - emul).max() / scale < 1e-5
    assert np.abs(D - ref).max() / scale < 3e-5


def test_epilogue_tanh_against_library_tanhf(lib):
    """The tensor-core epilogue's tanh (the exponential identity on the
    ex2/rcp instructions) stays within a few 2^-24 of the library tanhf,
    absolutely, and keeps NaN, signs, odd symmetry and the saturation."""
    fp = C.POINTER(C.c_float)
    x = np.concatenate([np.linspace(-12.0, 12.0, 1 << 21), np.linspace(-0.7, 0.7, 1 << 20),
                        np.array([0.0, -0.0, 1e-30, -1e-30, 0.6, -0.6, np.nextafter(0.6, 0),
                                  20.0, -20.0, 1e30, -1e30, np.inf, -np.inf])]).astype(np.float32)
    ytc = np.empty_like(x)
    ylib = np.empty_like(x)
    assert lib.gbnde_act_selftest(x.ctypes.data_as(fp), x.size, 1, ytc.ctypes.data_as(fp),
                                  ylib.ctypes.data_as(fp)) == 0
    err = np.abs(ytc.astype(np.float64) - ylib.astype(np.float64))
    # bound: half the ex2.approx relative error (2^-22) at e = 1, the refined
    # reciprocal (2^-23) and the final rounding: below 8 units of 2^-24
    assert err.max() <= 8.0 * 2.0 ** -24, err.max()
    # signs agree except where the identity rounds a tiny |x| to 0
    assert np.all((np.sign(ytc) == np.sign(ylib)) | ((ytc == 0) & (np.abs(x) < 1e-6)))
    ylin = ytc[: 1 << 21]
    assert np.array_equal(ylin, -ylin[::-1])  # odd: the grid is symmetric about 0
    assert np.all(np.abs(ytc) <= 1.0)
    xn = np.array([np.nan], np.float32)
    yn, yl = np.empty_like(xn), np.empty_like(xn)
    assert lib.gbnde_act_selftest(xn.ctypes.data_as(fp), 1, 1, yn.ctypes.data_as(fp), yl.ctypes.data_as(fp)) == 0
    assert np.isnan(yn[0])
