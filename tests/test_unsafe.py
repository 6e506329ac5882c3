"""Unsafe operations on the GPU (cal2DUnsafe.h) against the oracle, which
is pinned to the reference library (tests/test_oracle_pins.py):

* the probe's integer and byte spreads through calAddNext2Di/b and
  calAddNextX2Di/b (device atomics; integer sums do not depend on their
  order) and its single-writer neighbour stores through calSetX2Dr,
  calGetNextX2Dr, calSetCurrentX2Dr and calInitX2Dr: bit for bit, on every
  neighbourhood and both boundaries, launched per step or replayed as a
  recorded step;
* SCIDDICA-T in the reference's unsafe form (outflows moved at once with
  calAddNext2Dr / calAddNextX2Dr): real sums in atomic order, so the
  comparison is to a relative tolerance (stated below) plus mass
  conservation."""
import numpy as np
import pytest

from opencal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# relative tolerance per cell for SCIDDICA-T in unsafe form after 50 steps:
# each next(h) receives up to five real contributions in an unspecified
# order (the reference's serial order versus the GPU's atomics)
RTOL = 1e-12


@pytest.fixture(scope="module")
def libs():
    import opencal_gb300 as cal
    import oracle
    cal.build()
    oracle.build()
    return cal, oracle


def _inputs(rows, cols, seed):
    u = W.uniform_array(seed, (rows, cols))
    v0 = np.where(u < 0.3, 1 + (W.uniform_array(seed + 1, (rows, cols)) * 19).astype(np.int32), 0).astype(np.int32)
    b0 = (W.uniform_array(seed + 2, (rows, cols)) < 0.2).astype(np.int8)
    w0 = W.quantise(W.uniform_array(seed + 3, (rows, cols)))
    return v0, b0, w0


@pytest.mark.parametrize("nb", [1, 2, 3, 4])
@pytest.mark.parametrize("tor", [0, 1])
@pytest.mark.parametrize("graph", [False, True])
def test_unsafe_probe_bit_exact(libs, nb, tor, graph):
    cal, oracle = libs
    v0, b0, w0 = _inputs(41, 54, 70 + nb)
    ref = oracle.unsafe2d(v0, b0, w0, 12, nbhd=nb, toroidal=tor)
    import probes
    got = probes.unsafe2d(v0, b0, w0, 12, nbhd=nb, toroidal=tor, graph=graph)
    for name, a, b in zip(("v", "b", "w", "u", "x"), got, ref):
        assert a.tobytes() == b.tobytes(), name


def test_sciddicaT_unsafe_close_to_reference(libs):
    cal, oracle = libs
    z, h = W.sciddicaT_inputs(96, 112, seed=5)
    rz, rh = oracle.sciddicaT_unsafe(z, h, 50, toroidal=True)
    gz, gh = cal.sciddicaT_unsafe(z, h, 50, toroidal=True)
    assert gz.tobytes() == rz.tobytes()
    scale = np.abs(rh).max()
    mask = np.abs(rh) > 1e-9 * scale
    rel = np.abs(gh - rh)[mask] / np.abs(rh)[mask]
    assert rel.max() <= RTOL, rel.max()
    assert abs(gh.sum() - rh.sum()) <= 1e-12 * abs(rh.sum())
