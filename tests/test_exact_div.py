"""exact_div.cuh: division of a double by 1..9, division by sqrt(2) through
its reciprocal with Markstein's correction, and <=, >, > 0 on the integer
pipe must return exactly the IEEE results (the SCIDDICA-T and SCIARA-fv2
kernels rely on them for bit-exactness)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exact_div_host(tmp_path):
    exe = str(tmp_path / "exact_div_check")
    subprocess.run(["g++", "-O2", "-o", exe, os.path.join(ROOT, "tests", "native", "exact_div_check.cpp")],
                   check=True)
    out = subprocess.run([exe, "20000000", "3"], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip().splitlines()[-1] == "0", out.stdout


def _inputs(n, seed):
    from opencal_gb300.workloads import splitmix64_array
    r = splitmix64_array(seed, 3 * n)
    raw = r[:n].view(np.float64).copy()
    model = (r[n:2 * n] >> np.uint64(11)).astype(np.float64) / 2.0 ** 53 * 4000.0 - 200.0
    x = np.where(np.arange(n) % 2 == 0, raw, model)
    c = (r[2 * n:] % np.uint64(9)).astype(np.int32) + 1
    y = np.where(np.arange(n) % 3 == 0, x * (1 + 1e-16), np.roll(x, 1))
    specials = np.array([0.0, -0.0, 1e-310, -1e-310, np.inf, -np.inf, np.nan, 1e308, 2.2250738585072014e-308, 0.1])
    x[: len(specials)] = specials
    return np.ascontiguousarray(x), np.ascontiguousarray(c), np.ascontiguousarray(y)


@pytest.mark.gpu
def test_exact_div_device():
    import opencal_gb300 as cal
    import probes
    cal.build()
    x, c, y = _inputs(1 << 22, 11)
    assert probes.exact_div_mismatches(x, c, y) == 0
