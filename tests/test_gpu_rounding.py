"""The FP64 -> FP32 rounding of FP32 tableaux (blpg_round_f32 mode 0: the
loaders' integer-operation rounding) against CUDA's conversion instruction
(__double2float_rn, mode 1) on the edge cases of round-to-nearest-even.

Expected: the same bits everywhere except below FP32's normal range
(|x| < 2^-126), where the tableau rounding gives a zero of the input's sign
by design, and NaN, which stays NaN."""
import ctypes as C

import numpy as np
import pytest

from simplexprojects_gb300 import _native as N

pytestmark = pytest.mark.gpu

FLT_MIN = np.float64(np.finfo(np.float32).tiny)   # 2^-126
FLT_MAX = np.float64(np.finfo(np.float32).max)


def _round(x: np.ndarray, mode: int) -> np.ndarray:
    import torch
    d_in = torch.from_numpy(np.ascontiguousarray(x, np.float64)).cuda()
    d_out = torch.empty(x.size, dtype=torch.float32, device="cuda")
    N.check(N.lib().blpg_round_f32(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                   x.size, mode, None), "blpg_round_f32")
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _edge_cases() -> np.ndarray:
    one_ulp32 = 2.0 ** -23
    vals = [0.0, -0.0, 1.0, -1.0, 0.1, 1 / 3, np.pi, 1e-30, 1e30, 123456.789,
            # exact ties between two FP32 values: even stays, odd rounds up
            1.0 + 0.5 * one_ulp32, 1.0 + 1.5 * one_ulp32, -(1.0 + 2.5 * one_ulp32),
            # one FP64 ulp either side of a tie
            np.nextafter(1.0 + 0.5 * one_ulp32, 2.0), np.nextafter(1.0 + 0.5 * one_ulp32, 0.0),
            # carry into the exponent: just below 2, rounding up to 2
            2.0 - 0.25 * one_ulp32, np.nextafter(2.0, 0.0), 2.0 ** 100 * (2.0 - 0.4 * one_ulp32),
            # around FLT_MAX: stays, rounds down to it, ties up to infinity, beyond
            FLT_MAX, np.nextafter(FLT_MAX, np.inf), FLT_MAX * (1 + 2.0 ** -25),
            FLT_MAX * (1 + 2.0 ** -24), -FLT_MAX * (1 + 2.0 ** -24), 1e39, -1e300, np.inf, -np.inf,
            # around FLT_MIN (2^-126): the smallest normal, just above, just below
            FLT_MIN, -FLT_MIN, np.nextafter(FLT_MIN, 1.0), np.nextafter(FLT_MIN, 0.0),
            FLT_MIN * (1 - 2.0 ** -30), FLT_MIN * 0.5, 1e-40, -1e-44, 5e-324,
            np.nan]
    rng = np.random.default_rng(1)
    rand = np.concatenate([rng.standard_normal(4000) * 10.0 ** rng.integers(-30, 30, 4000),
                           rng.uniform(0, 1, 4000)])
    return np.concatenate([np.array(vals, dtype=np.float64), rand])


def test_tableau_rounding_matches_cuda_conversion(built):
    x = _edge_cases()
    mine = _round(x, 0)
    cuda = _round(x, 1)
    nan = np.isnan(x)
    assert np.isnan(mine[nan]).all() and np.isnan(cuda[nan]).all()
    low = ~nan & (np.abs(x) < FLT_MIN)
    assert (mine[low] == 0).all()
    assert np.array_equal(np.signbit(mine[low]), np.signbit(x[low]))
    rest = ~nan & ~low
    assert rest.sum() > 8000
    assert np.array_equal(mine[rest].view(np.uint32), cuda[rest].view(np.uint32))
    # and both are IEEE round-to-nearest-even, as the host's conversion
    assert np.array_equal(mine[rest].view(np.uint32), x[rest].astype(np.float32).view(np.uint32))
