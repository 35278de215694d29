"""The exact fixed-point accumulator behind the split double Sum
(kokkos_gb300/csrc/gbk_fixsum.cuh), compiled for the host with g++ and
checked against exact rational sums (fractions.Fraction): one accumulator
over a whole input is correctly rounded up to its periodic folds into FP64;
per-thread runs stay within FP64 rounding of the exact sum; integers and
subnormals are exact; exponent spreads far beyond 53 bits, exact cancellation
of values near the overflow threshold, overflow to infinity, and Inf/NaN keep
their FP64 meaning."""
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "fixsum_check.cpp")
BIN = os.path.join(ROOT, "kokkos_gb300", "_build", "fixsum_check")


@pytest.fixture(scope="module")
def driver():
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    hdr = os.path.join(ROOT, "kokkos_gb300", "csrc", "gbk_fixsum.cuh")
    if not os.path.exists(BIN) or os.path.getmtime(BIN) < max(os.path.getmtime(SRC), os.path.getmtime(hdr)):
        subprocess.run([cxx, "-O2", "-std=c++17", "-x", "c++", SRC, "-o", BIN], check=True)
    return BIN


def run(driver, x, per=1 << 40):
    out = subprocess.run([driver, str(per)], input=np.ascontiguousarray(x, dtype=np.float64).tobytes(),
                         stdout=subprocess.PIPE, check=True).stdout
    return float(out)


def exact(x):
    s = sum((Fraction(v) for v in x.tolist()), Fraction(0))
    try:
        return float(s), s
    except OverflowError:
        return (np.inf if s > 0 else -np.inf), s


def cases():
    rng = np.random.default_rng(11)
    return {
        "uniform": rng.random(50001),
        "normal": rng.standard_normal(50000),
        "wide": rng.standard_normal(20000) * 10.0 ** rng.integers(-300, 300, 20000),
        "cancel": np.concatenate([rng.standard_normal(2000) * 1e25, -rng.standard_normal(2000) * 1e25,
                                  rng.random(7)]),
        "subnormal": rng.random(5000) * 1e-312,  # every partial sum stays below 2^-1021: exact in FP64
        "ints": rng.integers(-(1 << 40), 1 << 40, 40001).astype(np.float64),
        "negative": -rng.random(30000),
    }


@pytest.mark.parametrize("name", list(cases()))
def test_fixsum_matches_exact(driver, name):
    x = cases()[name]
    want, q = exact(x)
    absum = float(np.sum(np.abs(x)))
    for per in (1 << 40, 1000, 37, 2):
        got = run(driver, x, per)
        if name in ("ints", "subnormal"):
            assert got == want, (name, per, got, want)
        elif per == 1 << 40 and len(x) <= (1 << 14):
            assert got == want, (name, got, want)  # one accumulator, no fold: correctly rounded
        else:
            # per-run results and folds are FP64 values added in FP64
            n_terms = len(x) // min(per, 1 << 14) + 2
            assert abs(got - want) <= 2 * n_terms * np.finfo(np.float64).eps * absum, (name, per, got, want)


def test_fixsum_single_fold_is_correctly_rounded(driver):
    """Up to 2^14 values fold once: the result is the exact sum rounded."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        x = rng.standard_normal(1 << 14) * 10.0 ** rng.integers(-20, 20, 1 << 14)
        want, _ = exact(x)
        assert run(driver, x) == want


def test_fixsum_special_values(driver):
    big = np.full(64, 1.5e308)
    big[1::2] = -1.5e308
    assert run(driver, big) == 0.0  # exact cancellation, no intermediate overflow
    assert run(driver, np.full(64, 1.5e308)) == np.inf
    assert run(driver, np.array([1.0, np.inf, 2.0, 3.0])) == np.inf
    assert np.isnan(run(driver, np.array([1.0, np.inf, 2.0, -np.inf])))
    assert np.isnan(run(driver, np.array([np.nan, 1.0, 2.0])))
    assert run(driver, np.zeros(9)) == 0.0
    assert run(driver, np.array([5e-324, 5e-324, -5e-324])) == 5e-324
