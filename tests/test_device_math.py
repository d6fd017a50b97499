"""The FP64 elementary functions of the generated device models
(csrc/vgb_math.cuh): table-driven exp and log after Tang, Newton-Raphson
division, pow through exp and log.

GPU: accuracy against the host's libm (numpy) over the argument ranges the
models reach, and IEEE results for every special case (which go to CUDA's
own functions).  CPU: the build-time tables against independent values.
"""

import ctypes as C
import math
import re

import numpy as np
import pytest

from vajax_gb300 import _lib

ULP = 2.0 ** -52


def _device_eval(fn, a, b=None):
    import torch
    lib = _lib.load()
    ad = torch.as_tensor(np.ascontiguousarray(a, np.float64), device="cuda")
    bd = torch.as_tensor(np.ascontiguousarray(b, np.float64), device="cuda") if b is not None else None
    out = torch.empty_like(ad)
    code = lib.vgb_math_eval(fn, len(a), C.c_void_p(ad.data_ptr()), C.c_void_p(bd.data_ptr()) if bd is not None
                             else None, C.c_void_p(out.data_ptr()), None)
    _lib.check(code)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(got, ref):
    ok = np.isfinite(ref) & (ref != 0)
    return float(np.max(np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])))


def _same_special(got, ref):
    both_nan = np.isnan(got) & np.isnan(ref)
    return bool(np.all(both_nan | (got == ref)))


@pytest.mark.gpu
def test_division_within_one_ulp(cuda):
    rng = np.random.default_rng(1)
    n = 1 << 18
    a = np.exp(rng.uniform(-690, 690, n)) * rng.choice([-1, 1], n)
    b = np.exp(rng.uniform(-690, 690, n)) * rng.choice([-1, 1], n)
    with np.errstate(all="ignore"):
        ref = a / b
    got = _device_eval(0, a, b)
    fin = np.isfinite(ref) & (np.abs(ref) > 1e-300)
    assert _rel(got[fin], ref[fin]) <= ULP
    special_a = np.array([1.0, -1.0, 0.0, 1.0, np.inf, np.nan, 1e300, 1e-300, 3.0, 5e-324])
    special_b = np.array([0.0, 0.0, 0.0, np.inf, 2.0, 1.0, 1e-300, 1e300, 5e-324, 3.0])
    with np.errstate(all="ignore"):
        assert _same_special(_device_eval(0, special_a, special_b), special_a / special_b)
        safe = np.where(special_b == 0.0, 0.0, special_a / np.where(special_b == 0.0, 1.0, special_b))
    assert _same_special(_device_eval(4, special_a, special_b), safe)


@pytest.mark.gpu
def test_reciprocal_within_one_ulp(cuda):
    rng = np.random.default_rng(6)
    x = np.exp(rng.uniform(-700, 700, 1 << 18)) * rng.choice([-1, 1], 1 << 18)
    with np.errstate(all="ignore"):
        ref = 1.0 / x
        assert _rel(_device_eval(5, x), ref) <= ULP
        special = np.array([0.0, -0.0, np.inf, np.nan, 5e-324, 1e-310, 1e300])
        assert _same_special(_device_eval(5, special), 1.0 / special)


@pytest.mark.gpu
def test_exp_within_two_ulp(cuda):
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-706, 706, 1 << 18), rng.uniform(-1, 1, 1 << 16),
                        rng.uniform(-1e-6, 1e-6, 1 << 12)])
    assert _rel(_device_eval(1, x), np.exp(x)) <= 2 * ULP
    special = np.array([0.0, -0.0, 710.0, -746.0, np.inf, -np.inf, np.nan])
    with np.errstate(all="ignore"):
        assert _same_special(_device_eval(1, special), np.exp(special))
    # beyond +-707 the library function takes over (results near overflow and subnormal)
    edge = np.array([707.0, 707.5, 709.7, -707.0, -708.0, -720.0])
    assert _rel(_device_eval(1, edge), np.exp(edge)) <= 2 * ULP


@pytest.mark.gpu
def test_log_within_two_ulp(cuda):
    rng = np.random.default_rng(3)
    x = np.concatenate([np.exp(rng.uniform(-690, 690, 1 << 18)), 1.0 + rng.uniform(-1e-3, 1e-3, 1 << 16),
                        np.nextafter(1.0, [0.0, 2.0]), 2.0 - rng.uniform(0, 1e-3, 1 << 12)])
    ref = np.log(x)
    got = _device_eval(2, x)
    assert _rel(got, ref) <= 2 * ULP
    special = np.array([1.0, 0.0, -0.0, -1.0, np.inf, np.nan])
    with np.errstate(all="ignore"):
        assert _same_special(_device_eval(2, special), np.log(special))
    sub = np.array([5e-324, 1e-310, 2.2e-308])  # subnormals: the library function
    assert _rel(_device_eval(2, sub), np.log(sub)) <= 2 * ULP


@pytest.mark.gpu
def test_pow_relative_error(cuda):
    rng = np.random.default_rng(4)
    n = 1 << 16
    x = np.exp(rng.uniform(-7, 7, n))
    y = rng.uniform(-6, 6, n)
    ref = np.power(x, y)
    # exp(y ln x) carries the rounding of y ln x into the result: |y ln x| ulps
    bound = (2 + np.abs(y * np.log(x))) * 2 * ULP
    got = _device_eval(3, x, y)
    assert np.all(np.abs(got - ref) / np.abs(ref) <= bound)
    sx = np.array([0.0, -2.0, -2.0, 2.0, np.inf, np.nan, 1.0, 1e300])
    sy = np.array([2.0, 3.0, 0.5, np.inf, 2.0, 1.0, np.nan, 10.0])
    with np.errstate(all="ignore"):
        assert _same_special(_device_eval(3, sx, sy), np.power(sx, sy))


def _tables():
    from vajax_gb300.build import math_tables
    text = math_tables()
    consts = {m.group(1): float.fromhex(m.group(2)) for m in re.finditer(r"#define (\w+) \((\S+)\)", text)}
    arrays = {}
    for m in re.finditer(r"double (\w+)\[(\d+)\] = \{([^}]*)\}", text):
        arrays[m.group(1)] = np.array([float.fromhex(v) for v in m.group(3).replace("\n", "").split(",")])
        assert len(arrays[m.group(1)]) == int(m.group(2))
    return consts, arrays


def test_math_tables_against_libm():
    consts, t = _tables()
    j = np.arange(64)
    assert np.max(np.abs(t["VGB_EXP2_TAB"] / np.exp2(j / 64.0) - 1)) <= ULP
    F = 1 + np.arange(129) / 128.0
    assert np.max(np.abs(t["VGB_LOG_INVF"] * F - 1)) <= ULP
    lnf = t["VGB_LOG_LNF_HI"] + t["VGB_LOG_LNF_LO"]
    assert np.max(np.abs(lnf[1:] / np.log(F[1:]) - 1)) <= ULP
    assert t["VGB_LOG_LNF_HI"][0] == 0.0
    assert t["VGB_LOG_LNF_HI"][128] == consts["VGB_LN2_HI"]  # exact cancellation just below 1


def test_math_split_constants():
    consts, _ = _tables()
    # heads with few enough significant bits that the reduction products are exact
    m, _ = math.frexp(consts["VGB_LN2_64_HI"])
    assert (m * 2 ** 36).is_integer()
    m, _ = math.frexp(consts["VGB_LN2_HI"])
    assert (m * 2 ** 42).is_integer()
    assert abs(consts["VGB_LN2_HI"] + consts["VGB_LN2_LO"] - math.log(2)) <= 1e-16
    assert abs((consts["VGB_LN2_64_HI"] + consts["VGB_LN2_64_LO"]) * 64 - math.log(2)) <= 1e-16
    assert abs(consts["VGB_INV_LN2_64"] * math.log(2) / 64 - 1) <= ULP
