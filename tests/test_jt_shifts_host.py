"""The warp-parallel shift attempts of the root solver's finish
(csrc/ccd_jt_shifts.h), resolved on the CPU with the same device code: each
stage's remaining shifts started from the stage's state and the first one in
order that finds a zero taken.  Against the sequential solver (the
reference's rpoly order, src/rpoly.h:211-249) on polynomials with clustered
and multiple roots, whose stages fail shift after shift: zeros, root counts
and status bit for bit.  CPU only."""
import ctypes

import numpy as np

from hostcheck.build import core_lib

P = ctypes.c_void_p


def _polys(rng, n):
    """Degree 3..6: a fifth with normal coefficients, the rest with a root of
    multiplicity 2..deg whose copies are spread by 0, 1e-9, 1e-6 or 1e-3."""
    coef = np.zeros((n, 7))
    deg = rng.integers(3, 7, n).astype(np.int32)
    for i in range(n):
        d = int(deg[i])
        kind = i % 5
        if kind == 0:
            c = rng.normal(size=d + 1)
        else:
            spread = (0.0, 1e-9, 1e-6, 1e-3)[kind - 1]
            r = rng.uniform(-1, 2)
            roots = [r + spread * rng.normal() for _ in range(int(rng.integers(2, d + 1)))]
            roots += list(rng.uniform(-2, 2, d - len(roots)))
            c = np.poly(roots) * rng.uniform(0.5, 2)
        coef[i, :d + 1] = c
    return coef, deg


def test_parallel_shifts_equal_sequential_solve():
    lib = core_lib()
    n = 200_000
    coef, deg = _polys(np.random.default_rng(1), n)
    zs, zp = np.zeros((n, 6)), np.zeros((n, 6))
    rs, rp = np.zeros(n, np.int32), np.zeros(n, np.int32)
    status, ahead = np.zeros(2 * n, np.int32), np.zeros(n, np.int32)
    lib.hc_shift_check(ctypes.c_int64(n), coef.ctypes.data_as(P), deg.ctypes.data_as(P), zs.ctypes.data_as(P),
                       rs.ctypes.data_as(P), zp.ctypes.data_as(P), rp.ctypes.data_as(P), status.ctypes.data_as(P),
                       ahead.ctypes.data_as(P))
    np.testing.assert_array_equal(rp, rs)
    np.testing.assert_array_equal(zp.view(np.uint64), zs.view(np.uint64))
    np.testing.assert_array_equal(status[1::2], status[0::2])
    # the set exercises the parallel path: solves whose stages needed later
    # shifts, and solves whose 20 shifts all failed
    assert (ahead > 0).sum() > 500 and (ahead >= 19).any() and (rp < deg).any()
