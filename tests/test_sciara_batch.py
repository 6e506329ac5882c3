"""SCIARA-fv2 split step (csrc/models/sciara_batch.cu): one scenario
reproduces the device-process program (csrc/models/sciara.cu, the
reference's elementary processes behind the C API) bit for bit -- both use
the transcendental forms of csrc/models/sciara_math.cuh and the reference's
operation order -- and a batch
of scenarios with uneven grids reproduces each scenario run alone.  Against
the oracle (the C library's transcendental functions) the tolerance of
test_sciara.py applies.  A lava list too small for the flow is reported as
an error, not overrun."""
import numpy as np
import pytest

from opencal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # as tests/test_sciara.py: the GPU's transcendental forms vs the C library


@pytest.fixture(scope="module")
def cal():
    import opencal_gb300 as cal
    cal.build()
    return cal


def _scenario(rows, cols, seed, et):
    z, vents, rates = W.sciara_inputs(rows, cols, seed=seed)
    return (z, vents, rates, et)


def _same(a, b, what):
    for k in ("z", "slt", "st", "msl"):
        assert a[k].tobytes() == b[k].tobytes(), f"{what}: {k} max diff {np.abs(a[k] - b[k]).max()}"


@pytest.mark.parametrize("rows,cols,seed", [(64, 80, 5), (96, 128, 6), (77, 101, 7)])
def test_split_step_equals_device_processes(cal, rows, cols, seed):
    sc = _scenario(rows, cols, seed, 600)
    ref = cal.sciara(sc[0], sc[1], sc[2], 600, 0, ac=False)
    (got,), steps = cal.sciara_batch([sc])
    assert steps == ref["steps"]
    _same(got, ref, f"{rows}x{cols}")


def test_batch_equals_scenarios_alone(cal):
    scs = [_scenario(64, 80, 11, 900), _scenario(120, 90, 12, 900), _scenario(97, 130, 13, 900)]
    got, steps = cal.sciara_batch(scs)
    for k, sc in enumerate(scs):
        ref = cal.sciara(sc[0], sc[1], sc[2], 900, 0, ac=True)
        assert steps == ref["steps"]
        _same(got[k], ref, f"scenario {k}")


def test_batch_close_to_oracle(cal):
    import oracle
    oracle.build()
    sc = _scenario(96, 112, 21, 1200)
    ref = oracle.sciara(sc[0], sc[1], sc[2], 1200, 0, ac=False)
    (got,), steps = cal.sciara_batch([sc])
    assert steps == ref["steps"]
    for k in ("slt", "st", "z", "msl"):
        r, g = ref[k], got[k]
        scale = max(np.abs(r).max(), 1e-300)
        mask = (np.abs(r) > 1e-9 * scale) | (np.abs(g) > 1e-9 * scale)
        rel = np.abs(g - r)[mask] / np.maximum(np.abs(r)[mask], 1e-300)
        assert (rel.max() if rel.size else 0.0) <= RTOL, k


def test_list_overflow_is_an_error(cal):
    sc = _scenario(160, 160, 31, 3600)
    with pytest.raises(cal.CALError):
        cal.sciara_batch([sc], 200, list_fraction=1e-9)


def test_undo_tape_grows_to_the_run(cal):
    """Four small grids (6 tiles each) over the whole emission (360 steps)
    flag more tiles than the default tape holds (2 x 24 + 4096): the call
    reruns the forward with the size it counted and matches a generous
    explicit tape; an explicit tape that is too small is an error."""
    scs = [_scenario(48, 64, 41 + k, 3600) for k in range(4)]
    targets = [np.zeros((48, 64)) for _ in scs]
    loss_d, g_d = cal.sciara_loss_grad(scs, targets)
    loss_e, g_e = cal.sciara_loss_grad(scs, targets, tape_slots=200000)
    # loss and gradients are sums by double atomics: equal up to their order
    np.testing.assert_allclose(loss_d, loss_e, rtol=1e-12)
    for a, b in zip(g_d, g_e):
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-14)
    with pytest.raises(cal.CALError):
        cal.sciara_loss_grad(scs, targets, tape_slots=16)


def _loss(cal, sc, target):
    (out,), _ = cal.sciara_batch([sc])
    d = out["slt"] - target
    return float((d * d).sum())


def test_emission_rate_gradient_matches_finite_differences(cal):
    """dL/drate of the adjoint (decisions frozen) against central finite
    differences of the forward, at a point where no decision flips within
    the step (relative step 1e-7)"""
    z, vents, rates = W.sciara_inputs(56, 64, seed=41, nvents=2, phases=3)
    et = 300
    true = [[r * 0.9 for r in rr] for rr in rates]
    (tgt_run,), _ = cal.sciara_batch([(z, vents, true, et)])
    target = tgt_run["slt"]
    sc = (z, vents, rates, et)
    loss, (g,) = cal.sciara_loss_grad([sc], [target])
    assert loss[0] == pytest.approx(_loss(cal, sc, target), rel=1e-12)
    checked = 0
    for v in range(len(vents)):
        for p in range(3):
            d = rates[v][p] * 1e-7
            up = [list(rr) for rr in rates]
            dn = [list(rr) for rr in rates]
            up[v][p] += d
            dn[v][p] -= d
            fd = (_loss(cal, (z, vents, up, et), target) - _loss(cal, (z, vents, dn, et), target)) / (2 * d)
            assert g[v, p] == pytest.approx(fd, rel=2e-4, abs=1e-9 * max(1.0, abs(fd))), (v, p)
            checked += 1
    assert checked == 6 and np.abs(g).max() > 0


def test_gradient_batch_equals_scenarios_alone(cal):
    scs, tgts = [], []
    for k, (r, c) in enumerate([(48, 60), (64, 52)]):
        z, vents, rates = W.sciara_inputs(r, c, seed=50 + k, phases=3)
        sc = (z, vents, rates, 300)
        (t,), _ = cal.sciara_batch([(z, vents, [[x * 1.1 for x in rr] for rr in rates], 300)])
        scs.append(sc)
        tgts.append(t["slt"])
    loss, grads = cal.sciara_loss_grad(scs, tgts)
    for k in range(2):
        l1, (g1,) = cal.sciara_loss_grad([scs[k]], [tgts[k]])
        assert loss[k] == pytest.approx(l1[0], rel=1e-13)
        np.testing.assert_allclose(grads[k], g1, rtol=1e-10, atol=1e-14)
