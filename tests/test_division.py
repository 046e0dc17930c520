"""The plain path's shared-divisor division must return the IEEE quotient bit
for bit: random operands over the whole proven exponent window, operands
outside it (fallback), special significands, quotients next to powers of
two and next to rounding midpoints, signed zeros, infinities and NaNs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MANT = np.uint64((1 << 52) - 1)


def _compose(rng, n, elo, ehi, mant=None):
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    exp = rng.integers(elo, ehi + 1, n, dtype=np.uint64) << np.uint64(52)
    if mant is None:
        mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    return (sign | exp | (np.asarray(mant, dtype=np.uint64) & MANT)).view(np.float64)


def _operands():
    rng = np.random.default_rng(7)
    A, B = [], []
    n = 4_000_000
    # 1. random operands across the window [2^-250, 2^251)
    A.append(_compose(rng, n, 1023 - 250, 1023 + 250))
    B.append(_compose(rng, n, 1023 - 250, 1023 + 250))
    # 2. the whole exponent range, subnormals, inf and NaN included (fallback)
    A.append(_compose(rng, n // 4, 0, 2047))
    B.append(_compose(rng, n // 4, 0, 2047))
    # 3. special significands: 1.0, 1+ulp, all ones, all ones - 1
    specials = np.array([0, 1, (1 << 52) - 1, (1 << 52) - 2, 1 << 51, (1 << 51) - 1], dtype=np.uint64)
    m = 1_000_000
    A.append(_compose(rng, m, 1023 - 60, 1023 + 60, specials[rng.integers(0, len(specials), m)]))
    B.append(_compose(rng, m, 1023 - 60, 1023 + 60, specials[rng.integers(0, len(specials), m)]))
    A.append(_compose(rng, m, 1023 - 60, 1023 + 60))
    B.append(_compose(rng, m, 1023 - 60, 1023 + 60, specials[rng.integers(0, len(specials), m)]))
    # 4. quotients next to powers of two: a = b * (1 - k 2^-53) and b * (1 + k 2^-52)
    b = _compose(rng, m, 1023 - 100, 1023 + 100)
    k = rng.integers(1, 8, m).astype(np.float64)
    A.append(b * (1.0 - k * 2.0 ** -53))
    B.append(b)
    A.append(b * (1.0 + k * 2.0 ** -52) * 4.0)
    B.append(b)
    # 5. quotients next to rounding midpoints: a = RN(b * (q + ulp(q)/2 (1 + small)))
    q = _compose(rng, m, 1023 - 30, 1023 + 30)
    mid = q.astype(np.longdouble) + np.spacing(np.abs(q)).astype(np.longdouble) / 2 * np.sign(q)
    jitter = 1 + rng.integers(-4, 5, m).astype(np.longdouble) * np.longdouble(2.0) ** -62
    A.append((b.astype(np.longdouble) * mid * jitter).astype(np.float64))
    B.append(b)
    # 6. exact quotients and integer-valued operands
    A.append(b * rng.integers(1, 1 << 20, m).astype(np.float64))
    B.append(b)
    ints = rng.integers(1, 1 << 30, (2, m)).astype(np.float64)
    A.append(ints[0])
    B.append(ints[1])
    # 7. signed zeros, infinities, NaN, zero divisors
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.0, 1e-300, 5e-324, 1e300], dtype=np.float64)
    aa, bb = np.meshgrid(sp, sp)
    A.append(aa.ravel())
    B.append(bb.ravel())
    return np.concatenate(A), np.concatenate(B)


def test_shared_divisor_division_is_the_ieee_quotient():
    import torch
    from microfc_gb300 import _lib
    a, b = _operands()
    L = _lib.load()
    dev = torch.device("cuda", 0)
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    qf, qi = torch.empty_like(ta), torch.empty_like(ta)
    s = torch.cuda.current_stream(dev)
    _lib.check(L.mfc_gpu_selftest_div(ctypes.c_void_p(ta.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
                                      ctypes.c_void_p(qf.data_ptr()), ctypes.c_void_p(qi.data_ptr()), len(a),
                                      ctypes.c_void_p(s.cuda_stream)))
    qf, qi = qf.cpu().numpy(), qi.cpu().numpy()
    bad = np.flatnonzero(qf.view(np.uint64) != qi.view(np.uint64))
    assert bad.size == 0, [(a[i].hex(), b[i].hex(), qf[i].hex(), qi[i].hex()) for i in bad[:5]]
    # the device's IEEE quotient is the host's
    with np.errstate(all="ignore"):
        host = a / b
    fin = ~np.isnan(host)
    assert np.array_equal(qi[fin].view(np.uint64), host[fin].view(np.uint64))
    assert np.isnan(qi[~fin]).all()
