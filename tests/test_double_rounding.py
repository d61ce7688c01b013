"""The FP32 double-float evaluation of the reference's double-precision
expressions (csrc/double_rounding.cuh): on the host over seeded arguments, and
on the device through bepugpu_probe_double_rounding, every result equals the
float the double expression rounds to, and the FP32 path decides nearly all."""
import ctypes
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from bepuphysics1_gb300 import native as N

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "bepuphysics1_gb300" / "csrc" / "double_rounding.cuh"


def test_host_routines_match_the_double_expressions(tmp_path):
    exe = tmp_path / "double_rounding_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", str(ROOT / "tests" / "double_rounding_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "400000"], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = {line.split()[0]: [int(v) for v in line.split()[1:]] for line in out if line.strip()}
    for name in ("invsqrt", "sqrtquotient"):
        n, fast, bad = rows[name]
        assert bad == 0, name
        assert fast > 0.995 * n, (name, fast, n)
    n, fast, bad, typical, typical_fast = rows["pow"]
    assert bad == 0
    # results below 2^-100 and dt ln c below -80 always take the double path
    assert fast > 0.9 * n and typical_fast > 0.999 * typical, rows["pow"]


def _table(name):
    import re
    text = HEADER.read_text()
    body = text[text.index("#define BEPU_POW_TABLES"):text.index("struct PowTables")]
    vals = [float.fromhex(v.rstrip("f")) for v in re.findall(r"-?0x[0-9a-fp.+-]+f", body)]
    assert len(vals) == 2 + 22 + 28
    return {"ln2": vals[:2], "odd": vals[2:24], "fact": vals[24:]}


def _split(x: Fraction):
    hi = np.float32(float(x))
    lo = np.float32(float(x - Fraction(float(hi))))
    return float(hi), float(lo)


def test_series_constants_are_the_nearest_float_pairs():
    t = _table(None)
    for k in range(11):
        assert tuple(t["odd"][2 * k:2 * k + 2]) == _split(Fraction(1, 2 * k + 1)), k
    f = Fraction(1)
    for n in range(14):
        if n:
            f /= n
        assert tuple(t["fact"][2 * n:2 * n + 2]) == _split(f), n
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 120
    ln2 = Fraction(mp.nstr(mp.log(2), 40))
    assert tuple(t["ln2"]) == _split(ln2)


def _cases(rng, n):
    x = np.concatenate([rng.uniform(0, 4, n // 2),
                        np.ldexp(rng.uniform(0.5, 1.5, n // 2), rng.integers(-95, 95, n // 2))]).astype(np.float32)
    e = np.concatenate([rng.uniform(0, 0.0676, n // 2),
                        np.ldexp(rng.uniform(0.5, 1.5, n // 2), rng.integers(-95, 95, n // 2))]).astype(np.float32)
    y = np.where(rng.random(n) < 0.7, np.float32(0.52),
                 np.ldexp(rng.uniform(0.5, 1.5, n), rng.integers(-50, 50, n))).astype(np.float32)
    c = np.concatenate([rng.uniform(0, 1, n // 2), rng.uniform(0, 1, n // 2) ** 20]).astype(np.float32)
    c[:64] = 0
    c[64:128] = 1
    dt = np.where(rng.random(n) < 0.75, np.float32(1 / 60), rng.uniform(0, 16, n)).astype(np.float32)
    return x, e, y, c, dt


@pytest.mark.gpu
def test_device_routines_match_the_double_expressions(gpu_context):
    rng = np.random.default_rng(11)
    n = 1 << 21
    x, e, y, c, dt = _cases(rng, n)
    want = {
        0: (1.0 / np.sqrt(x.astype(np.float64))).astype(np.float32),
        1: (np.sqrt(e.astype(np.float64)) / y.astype(np.float64)).astype(np.float32),
        2: np.power(c.astype(np.float64), dt.astype(np.float64)).astype(np.float32),
    }
    args = {0: (x, None), 1: (e, y), 2: (c, dt)}
    lib = gpu_context.lib
    for kind, (a, b) in args.items():
        out = np.zeros(n, np.float32)
        fast = ctypes.c_uint32()
        gpu_context.check(lib.bepugpu_probe_double_rounding(gpu_context.handle, kind, N.ptr(a),
                                                            N.ptr(b) if b is not None else None, n, N.ptr(out),
                                                            ctypes.byref(fast)))
        np.testing.assert_array_equal(out.view(np.uint32), want[kind].view(np.uint32), err_msg=f"kind {kind}")
        assert fast.value > (0.9 if kind == 2 else 0.995) * n, (kind, fast.value)
