"""The erosion kernels' division where a divisor repeats (Markstein's correction of a reciprocal
product, IEEE-division fallback outside its safe range) is bit-identical to IEEE division: checked
against numpy's correctly rounded float32 quotient on 16M random pairs spanning every exponent,
plus zeros, subnormals, infinities and NaNs."""
from __future__ import annotations

import numpy as np
import pytest

import master_thesis_gb300 as T

pytestmark = pytest.mark.gpu


def random_floats(rng, n, exp_lo, exp_hi, signed=True):
    mant = rng.integers(0, 1 << 23, n, dtype=np.uint32)
    exp = rng.integers(exp_lo + 127, exp_hi + 127 + 1, n).astype(np.uint32)
    sign = (rng.integers(0, 2, n).astype(np.uint32) << 31) if signed else np.zeros(n, np.uint32)
    return (sign | (exp << 23) | mant).view(np.float32)


def test_div_rn_matches_ieee_division():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    n = 1 << 24
    a = random_floats(rng, n, -126, 127)
    b = random_floats(rng, n, -40, 40, signed=False)
    # the kernels' operand ranges: height / flux differences over pipe length 1000, flux over
    # water depth >= 0.01, talus differences over their sum
    k = n // 4
    a[:k] = (rng.normal(0, 1, k) * 10.0 ** rng.uniform(-12, 3, k)).astype(np.float32)
    b[:k] = np.where(rng.uniform(size=k) < 0.5, np.float32(1000.0),
                     (0.01 + rng.exponential(1.0, k)).astype(np.float32))
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1.17549435e-38, 3.4028235e38,
                         2.0 ** -64, -(2.0 ** -64), 2.0 ** 64, np.nextafter(np.float32(2.0 ** -64), 0)],
                        np.float32)
    a[k:k + specials.size] = specials
    b[k:k + specials.size] = np.float32(1000.0)
    b[k + specials.size:k + 2 * specials.size] = np.float32(0.37)
    a[k + specials.size:k + 2 * specials.size] = specials
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty_like(da)
    T.check(T.lib().tecto_selftest_div(da.data_ptr(), db.data_ptr(), out.data_ptr(), n, None), "selftest_div")
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        want = a / b
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    bad = np.flatnonzero(~same)
    assert bad.size == 0, f"{bad.size} mismatches, e.g. a={a[bad[:4]]} b={b[bad[:4]]} got={got[bad[:4]]} want={want[bad[:4]]}"


def test_div_var_matches_ieee_division():
    """The per-lane form (a correctly rounded reciprocal of each divisor, then Markstein's
    correction) on the same pairs."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    n = 1 << 24
    a = random_floats(rng, n, -126, 127)
    b = random_floats(rng, n, -40, 40, signed=False)
    # the kernels' per-cell divisors: water depth >= 0.01, flux total x dt + 1e-6
    k = n // 2
    a[:k] = (rng.normal(0, 1, k) * 10.0 ** rng.uniform(-12, 3, k)).astype(np.float32)
    b[:k] = np.where(rng.uniform(size=k) < 0.5, (0.01 + rng.exponential(1.0, k)),
                     1e-6 + rng.exponential(1e-3, k) * 10.0 ** rng.uniform(-3, 3, k)).astype(np.float32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, 1.17549435e-38, 3.4028235e38,
                         2.0 ** -64, 2.0 ** 64, 2.0 ** -32, 2.0 ** 32], np.float32)
    b[k:k + specials.size] = specials
    a[k:k + specials.size] = np.float32(0.37)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty_like(da)
    T.check(T.lib().tecto_selftest_div_var(da.data_ptr(), db.data_ptr(), out.data_ptr(), n, None),
            "selftest_div_var")
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        want = a / b
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    bad = np.flatnonzero(~same)
    assert bad.size == 0, f"{bad.size} mismatches, e.g. a={a[bad[:4]]} b={b[bad[:4]]} got={got[bad[:4]]} want={want[bad[:4]]}"


def test_rcp_and_sqrt_exhaustive():
    """Every positive normal float: the kernels' reciprocal equals the correctly rounded one on
    [2^-32, 2^32] and their square root on [2^-100, 2^100], the ranges the kernels test before
    using them."""
    torch = pytest.importorskip("torch")
    bad = torch.zeros(512, dtype=torch.int64, device="cuda")
    T.check(T.lib().tecto_selftest_rcp_sqrt(bad.data_ptr(), None), "selftest_rcp_sqrt")
    torch.cuda.synchronize()
    h = bad.cpu().numpy()
    rcp, sq = h[:256], h[256:]
    hist = {"rcp": {e - 127: int(c) for e, c in enumerate(rcp) if c},
            "sqrt": {e - 127: int(c) for e, c in enumerate(sq) if c}}
    print("mismatches per binary exponent:", hist)
    assert rcp[127 - 32:127 + 33].sum() == 0, hist
    assert sq[127 - 100:127 + 101].sum() == 0, hist
