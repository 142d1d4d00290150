"""The FP32 arithmetic of the dense zeta kernel (k_sweep_dense), restated in
numpy and measured against the FP64 product of the same operator (CPU).

The kernel rounds the operator to FP32 once, takes each line less its first
value (g = f - f0 in FP32), and forms every output as four partial sums
(columns 4k, 4k+1, 4k+2, 4k+3 in packed pairs of FMAs) added as
(ea.x + ea.y) + (eb.x + eb.y).  Here each FMA is a product exact in FP64
plus the partial sum, rounded to FP32 (a double rounding the device does not
have, rare enough not to show in these bounds).  On lines that are nearly
uniform (a large constant part, as density or energy carry) the error of the
derivative is that of the FP32 input itself: the kernel adds nothing visible
to it, while a product without the first value taken out is several times
worse.
"""
import numpy as np
import pytest

from tandemproject_gb300.solver import dense_zeta_operator


def _fma32(a, b, c):
    return (np.float64(a) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def kernel_fp32(m32, f32, take_first=True):
    """k_sweep_dense's operation order on FP32 lines (columns of f32)."""
    L = m32.shape[0]
    lm = (L + 3) // 4 * 4
    g = np.zeros((lm, f32.shape[1]), np.float32)
    g[:L] = f32 - f32[0:1] if take_first else f32
    m = np.zeros((L, lm), np.float32)
    m[:, :L] = m32
    out = np.zeros((L, f32.shape[1]), np.float32)
    z = np.zeros(f32.shape[1], np.float32)
    for i in range(L):
        ax, ay, bx, by = z, z, z, z
        for k in range(lm // 4):
            ax = _fma32(m[i, 4 * k], g[4 * k], ax)
            ay = _fma32(m[i, 4 * k + 1], g[4 * k + 1], ay)
            bx = _fma32(m[i, 4 * k + 2], g[4 * k + 2], bx)
            by = _fma32(m[i, 4 * k + 3], g[4 * k + 3], by)
        out[i] = (ax + ay) + (bx + by)
    return out


@pytest.fixture(scope="module")
def operator(ati_lib):
    from tandemproject_gb300.config import small_case
    return dense_zeta_operator(small_case(lxibk=(16, 40, 16), letbk=(12, 12), lzebk=(31,)), 0)


def _lines(L, c, a, n=2048, seed=0):
    rng = np.random.default_rng(seed)
    k = np.arange(L)[:, None]
    wave = np.sin(2 * np.pi * rng.integers(1, 6, n)[None, :] * k / (L - 1) + rng.uniform(0, 2 * np.pi, n)[None, :])
    return c + a * (wave + 0.1 * rng.standard_normal((L, n)))


def _err(d, ref):
    return float(np.max(np.abs(d - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("c,a", [(1.0, 1e-3), (1.0 / 1.4, 1e-4), (1.0, 1e-5)])
def test_nearly_uniform_lines_keep_the_input_rounding(operator, c, a):
    f = _lines(operator.shape[0], c, a)
    ref = operator @ f
    f32 = f.astype(np.float32)
    e_input = _err(operator @ f32.astype(np.float64), ref)  # the FP32 input alone, exact product
    e_kernel = _err(kernel_fp32(operator.astype(np.float32), f32), ref)
    e_plain = _err(kernel_fp32(operator.astype(np.float32), f32, take_first=False), ref)
    # measured: kernel = input to three digits (1.16e-4, 5.8e-4, 1.1e-2); without f0 taken out 3.0-3.3x worse
    assert e_kernel <= 1.05 * e_input, (e_kernel, e_input)
    assert e_plain >= 2.0 * e_kernel, (e_plain, e_kernel)


def test_lines_of_order_one(operator):
    f = _lines(operator.shape[0], 0.0, 1.0)
    ref = operator @ f
    e = _err(kernel_fp32(operator.astype(np.float32), f.astype(np.float32)), ref)
    assert e < 1e-6, e  # measured 4.4e-7: a few FP32 roundings of the largest derivative


def test_constant_lines_have_zero_derivative(operator):
    f = np.full((operator.shape[0], 64), 0.7142857, np.float32)
    assert not np.any(kernel_fp32(operator.astype(np.float32), f))
