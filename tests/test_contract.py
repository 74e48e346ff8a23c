"""Arithmetic contract: accuracy of the shared transcendental functions against double
precision, and the PCG4D sequence against an independent implementation."""
import numpy as np
import pytest

import oracle


def ulp(x):
    x = np.abs(x.astype(np.float32))
    return np.spacing(np.maximum(x, np.float32(1.17549435e-38)))


@pytest.mark.parametrize("fn,lo,hi,ref", [
    ("sin", -8.0, 8.0, np.sin), ("cos", -8.0, 8.0, np.cos), ("tan", -1.4, 1.4, np.tan),
    ("acos", -1.0, 1.0, np.arccos), ("exp", -30.0, 30.0, np.exp), ("log", 1e-6, 1e6, np.log)])
def test_unary_accuracy(fn, lo, hi, ref):
    rng = np.random.default_rng(7)
    if fn == "log":
        x = np.exp(rng.uniform(np.log(lo), np.log(hi), 200000)).astype(np.float32)
    else:
        x = rng.uniform(lo, hi, 200000).astype(np.float32)
    got = oracle.contract(fn, x).astype(np.float64)
    want = ref(x.astype(np.float64))
    err = np.abs(got - want)
    # at most 4 ulp of the result, or 2^-24 absolute around zeros of the function
    tol = 4 * ulp(want) + (2.0 ** -24 if fn in ("sin", "cos", "tan", "log") else 0.0) + \
        (4e-7 if fn == "acos" else 0.0)
    assert np.all(err <= tol), (fn, float((err / ulp(want)).max()))


def test_atan2_accuracy_and_quadrants():
    rng = np.random.default_rng(8)
    y = rng.normal(size=200000).astype(np.float32)
    x = rng.normal(size=200000).astype(np.float32)
    got = oracle.contract("atan2", y, x).astype(np.float64)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.all(np.abs(got - want) <= 4 * ulp(want) + 2.0 ** -24)
    sp = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0], np.float32)
    sx = np.array([1.0, 1.0, -1.0, -1.0, 0.0, 0.0], np.float32)
    np.testing.assert_allclose(oracle.contract("atan2", sp, sx), np.arctan2(sp, sx), atol=1e-7)


def test_pow_accuracy():
    rng = np.random.default_rng(9)
    x = rng.uniform(1e-3, 4.0, 100000).astype(np.float32)
    y = rng.uniform(-3.0, 3.0, 100000).astype(np.float32)
    got = oracle.contract("pow", x, y).astype(np.float64)
    want = np.power(x.astype(np.float64), y.astype(np.float64))
    assert np.all(np.abs(got - want) <= 16 * ulp(want))
    special = oracle.contract("pow", np.array([0, 0, 1, 2, -1], np.float32), np.array([2, 0, 5, 0, 2], np.float32))
    assert special[0] == 0 and special[1] == 1 and special[2] == 1 and special[3] == 1 and np.isnan(special[4])


def pcg4d_python(px, py, frame, n):
    M = 0xFFFFFFFF
    v = [int(px) & M, int(py) & M, frame & M, (int(px) + int(py)) & M]
    out = []
    for _ in range(n):
        v = [(a * 1664525 + 1013904223) & M for a in v]
        v[0] = (v[0] + v[1] * v[3]) & M; v[1] = (v[1] + v[2] * v[0]) & M
        v[2] = (v[2] + v[0] * v[1]) & M; v[3] = (v[3] + v[1] * v[2]) & M
        v = [a ^ (a >> 16) for a in v]
        v[0] = (v[0] + v[1] * v[3]) & M; v[1] = (v[1] + v[2] * v[0]) & M
        v[2] = (v[2] + v[0] * v[1]) & M; v[3] = (v[3] + v[1] * v[2]) & M
        out.append(np.float32(np.float32(v[0]) / np.float32(4294967295.0)))
    return np.array(out, np.float32)


def test_pcg4d_sequence():
    for px, py, frame in [(0.5, 0.5, 1), (17.5, 3.5, 2), (255.5, 255.5, 64)]:
        got = oracle.rand_sequence(px, py, frame, 32)
        want = pcg4d_python(px, py, frame, 32)
        assert got.tobytes() == want.tobytes()
        assert np.all((got >= 0) & (got <= 1))
