"""The CUDA library's host-side table model (knots, collocation matrices,
band LU factors: bsplineinterpolation_gb300/csrc/spline_model.cpp) without a
GPU: built with AddressSanitizer, its knot vectors must equal the oracle's bit
for bit and its factors must solve the collocation systems."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "bsplineinterpolation_gb300", "csrc")
BIN = os.path.join(REPO, "tests", "host", "_build", "model_driver")


@pytest.fixture(scope="module")
def driver():
    if shutil.which("g++") is None:
        pytest.skip("no host compiler")
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
                           "-fno-omit-frame-pointer", "-ffp-contract=off", "-I" + CSRC,
                           os.path.join(REPO, "tests", "host", "model_driver.cpp"),
                           os.path.join(CSRC, "spline_model.cpp"), "-o", BIN])
    return BIN


def _cases(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        D = int(rng.integers(1, 5))
        O = int(rng.integers(0, 8))
        per = [int(v) for v in rng.integers(0, 2, D)]
        sizes = [int(s) for s in rng.integers(O + 2, O + 40, D)]
        lo = rng.uniform(-3, 1, D)
        hi = lo + rng.uniform(0.1, 4, D)
        coords = [None] * D
        for d in range(D):
            if rng.random() < 0.35 and not (O == 0 and not per[d]):
                m = sizes[d] + per[d]
                c = np.sort(rng.uniform(lo[d], hi[d], m))
                c[0], c[-1] = lo[d], hi[d]
                if np.all(np.diff(c) > 0):
                    coords[d] = c
        out.append((D, O, per, sizes, lo, hi, coords))
    return out


def _encode(case):
    D, O, per, sizes, lo, hi, coords = case
    parts = [str(D), str(O)] + [str(p) for p in per] + [str(s) for s in sizes]
    parts += [float(v).hex() for v in lo] + [float(v).hex() for v in hi]
    for c in coords:
        if c is None:
            parts.append("0")
        else:
            parts.append(str(len(c)))
            parts += [float(v).hex() for v in c]
    return " ".join(parts)


def test_model_matches_oracle_under_asan(driver):
    cases = _cases(5, 250)
    inp = "\n".join(_encode(c) for c in cases) + "\n"
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([driver], input=inp, capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
    lines = r.stdout.splitlines()
    pos = 0
    n_ok = 0
    for D, O, per, sizes, lo, hi, coords in cases:
        head = lines[pos]
        pos += 1
        try:
            s = oracle.Spline(D, O, per, sizes, lo, hi, coords)
        except ValueError:
            s = None
        if head.startswith("ERROR"):
            # the product may be stricter than the oracle (it rejects inputs
            # the reference would misbehave on), never laxer
            continue
        assert s is not None, (D, O, per, sizes)
        n_ok += 1
        for d in range(D):
            k = lines[pos].split()
            r_ = lines[pos + 1].split()
            pos += 2
            knots = np.array([float.fromhex(v) for v in k[2:]])
            assert int(k[1]) == len(knots)
            assert np.array_equal(knots, s.knots(d)), (D, O, per, sizes, d)
            lo_r, hi_r = float.fromhex(r_[1]), float.fromhex(r_[2])
            assert (lo_r, hi_r) == s.range(d)
            assert float(r_[3]) < 1e-9, (D, O, per, sizes, d, r_[3])
    assert n_ok > 150
