"""Shared helpers for the parity tests: tolerance rules and device setup.

Tolerances (stated before any run, not tuned):
  * integers, Min/Max/Loc values and locs, scans of integers, histograms,
    sort keys and permutations: bit-exact;
  * double Sum: |gpu - S| <= 1e-12 * |S|, S the compensated FP64 sum; for
    ill-conditioned data the check also passes when |gpu - S| <= 1e-12 *
    ||x||_2 (both bounds must fail to fail);
  * float Sum (accumulated in FP32): the same two-sided rule with 1e-5;
  * Prod: relative n * eps(type) (the worst-case bound of n-1 roundings).
"""
import numpy as np

REL_F64 = 1e-12
REL_F32 = 1e-5


def sum_ok(got, x, rel):
    import oracle
    s, a, q = oracle.sum_compensated(x)
    err = abs(float(got) - s)
    return err <= rel * abs(s) or err <= rel * np.sqrt(q), (float(got), s, err, np.sqrt(q))


def sum_tol(dtype):
    return REL_F64 if np.dtype(dtype) == np.float64 else REL_F32


def prod_ok(got, x):
    exact = float(np.prod(x.astype(np.float64)))
    eps = np.finfo(x.dtype).eps
    tol = max(x.size, 1) * eps
    return abs(float(got) - exact) <= tol * abs(exact) + 1e-300, (float(got), exact)
