"""Batched SCIDDICA-T ensembles (opencal_gb300.ensemble): every instance of a
packed ensemble with uneven grid sizes and its own parameters advances
bit-exactly like the oracle run of that instance alone; every tile shape
gives the same result; the sparse work-lists stay below the full tile count;
the ensemble adjoint's loss and gradients match the single-model adjoint of
each instance; the FD comparison arm agrees with the adjoint; a small
calibration recovers the parameters."""
import numpy as np
import pytest

from opencal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# uneven sizes: odd column counts (no 16-byte rows), thin grids, several tile rows
DIMS = [(40, 52), (33, 47), (64, 64), (97, 130), (70, 35), (129, 66)]
STEPS = 60


@pytest.fixture(scope="module")
def env():
    import torch

    import opencal_gb300 as cal
    import oracle
    from opencal_gb300 import ensemble as E
    cal.build()
    oracle.build()
    rng = W.SplitMix64(77)
    params = [(rng.uniform(0.3, 0.7), rng.uniform(5e-4, 5e-3)) for _ in DIMS]
    zs, hs = W.ensemble_inputs(DIMS, first_seed=500)
    return torch, oracle, E, params, zs, hs


def _refs(oracle, params, zs, hs, steps):
    return [oracle.sciddicaT(z, h, steps, toroidal=False, p_r=p[0], p_eps=p[1])[1] for p, z, h in zip(params, zs, hs)]


def test_forward_bit_exact(env):
    torch, oracle, E, params, zs, hs = env
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    got = ens.unpack(ens.forward())
    for b, (g, r) in enumerate(zip(got, _refs(oracle, params, zs, hs, STEPS))):
        assert g.tobytes() == r.tobytes(), f"instance {b} {DIMS[b]}"


@pytest.mark.parametrize("shape", ["32x16", "64x16", "64x32", "16x8", "32x8"])
def test_every_tile_shape_bit_exact(env, shape):
    torch, oracle, E, params, zs, hs = env
    ens = E.Ensemble(DIMS, params, zs, hs, 25)
    ens.set_shape(shape)
    got = ens.unpack(ens.forward())
    for b, (g, r) in enumerate(zip(got, _refs(oracle, params, zs, hs, 25))):
        assert g.tobytes() == r.tobytes(), f"instance {b} {DIMS[b]} shape {shape}"


def test_zero_steps_is_canonical_h0(env):
    torch, oracle, E, params, zs, hs = env
    hs2 = [h.copy() for h in hs]
    hs2[0][0, 0] = -0.0
    ens = E.Ensemble(DIMS, params, zs, hs2, 0)
    got = ens.unpack(ens.forward())
    for g, h in zip(got, hs2):
        assert g.tobytes() == (h + 0.0).tobytes()


def test_work_lists_are_sparse(env):
    torch, oracle, E, params, zs, hs = env
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    ens.set_shape("32x16")
    ens.forward()
    counts = ens.active_tiles()
    total = sum(((c + 31) // 32) * ((r + 15) // 16) for r, c in DIMS)
    assert counts.max() <= total
    assert counts[0] > 0 and counts.min() < total


def test_autotune_picks_a_shape(env):
    torch, oracle, E, params, zs, hs = env
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    name, ms = ens.autotune(10)
    assert name in E.SHAPES and all(v > 0 for v in ms.values())
    got = ens.unpack(ens.forward())
    for g, r in zip(got, _refs(oracle, params, zs, hs, STEPS)):
        assert g.tobytes() == r.tobytes()


def test_gradients_match_single_model_adjoint(env):
    """loss, dL/dp_r, dL/dp_eps and dL/dh0 of every instance against the
    single-model adjoint (cal.adjoint.rollout) of that instance"""
    torch, oracle, E, params, zs, hs = env
    import opencal_gb300 as cal
    dev = torch.device("cuda")
    true = [(p[0] * 0.9, p[1] * 1.2) for p in params]
    tgts = _refs(oracle, true, zs, hs, STEPS)
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    loss, grad, gh0 = ens.loss_grad(ens.pack(tgts), want_h0_grad=True)
    gh0 = ens.unpack(gh0)
    for b in range(len(DIMS)):
        z = torch.from_numpy(zs[b]).to(dev)
        h0 = torch.from_numpy(hs[b]).to(dev).requires_grad_(True)
        pr = torch.tensor(params[b][0], dtype=torch.float64, device=dev, requires_grad=True)
        pe = torch.tensor(params[b][1], dtype=torch.float64, device=dev, requires_grad=True)
        hT = cal.adjoint.rollout(z, h0, pr, pe, STEPS)
        L = ((hT - torch.from_numpy(tgts[b]).to(dev)) ** 2).sum()
        L.backward()
        assert loss[b] == pytest.approx(L.item(), rel=1e-12, abs=1e-300)
        assert grad[b, 0] == pytest.approx(pr.grad.item(), rel=1e-9, abs=1e-12)
        assert grad[b, 1] == pytest.approx(pe.grad.item(), rel=1e-9, abs=1e-9)
        np.testing.assert_allclose(gh0[b], h0.grad.cpu().numpy(), rtol=1e-9, atol=1e-12)


def test_recorded_evaluation_equals_launch_by_launch(env):
    """loss_grad as one graph launch (tape layout on the device) against the
    launch-by-launch evaluation: losses and gradients equal up to the
    summation order of their atomics; a second call replays the same graph."""
    torch, oracle, E, params, zs, hs = env
    true = [(p[0] * 0.9, p[1] * 1.2) for p in params]
    tgts = _refs(oracle, true, zs, hs, STEPS)
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    tgt = ens.pack(tgts)
    ens.set_graph(False)
    l0, g0, h0 = ens.loss_grad(tgt, want_h0_grad=True)
    ens.set_graph(True)
    l1, g1, h1 = ens.loss_grad(tgt, want_h0_grad=True)
    launches, nodes = ens.graph_stats()
    assert launches >= 1 and nodes > 4 * STEPS
    l2, g2, _ = ens.loss_grad(tgt, want_h0_grad=True)
    assert ens.graph_stats()[0] == launches + 1  # replayed: one launch, tape already large enough
    np.testing.assert_allclose(l1, l0, rtol=1e-12, atol=0)
    np.testing.assert_allclose(l2, l0, rtol=1e-12, atol=0)
    np.testing.assert_allclose(g1, g0, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(g2, g0, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(h1.cpu().numpy(), h0.cpu().numpy(), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("graph", [True, False])
def test_whole_rollout_tape_equals_segments(env, graph):
    """the adjoint with the whole rollout on the tape (no recomputation)
    against sqrt(T) segments recomputed from checkpoints: same losses, same
    dL/dh0, gradients equal up to the summation order of their atomics"""
    torch, oracle, E, params, zs, hs = env
    true = [(p[0] * 0.9, p[1] * 1.2) for p in params]
    tgts = _refs(oracle, true, zs, hs, STEPS)
    ens = E.Ensemble(DIMS, params, zs, hs, STEPS)
    ens.set_graph(graph)
    tgt = ens.pack(tgts)
    assert ens.tape_info()["full"]  # the default chooses by memory: this small ensemble fits
    ens.set_tape("segments")
    l0, g0, h0 = ens.loss_grad(tgt, want_h0_grad=True)
    seg = ens.tape_info()
    ens.set_tape("full")
    l1, g1, h1 = ens.loss_grad(tgt, want_h0_grad=True)
    full = ens.tape_info()
    assert not seg["full"] and full["full"]
    assert full["need_bytes"] > seg["need_bytes"] > 0
    assert full["capacity_bytes"] >= full["need_bytes"]
    np.testing.assert_allclose(l1, l0, rtol=1e-12, atol=0)  # per-block sums added by atomics
    np.testing.assert_allclose(g1, g0, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(h1.cpu().numpy(), h0.cpu().numpy(), rtol=1e-12, atol=1e-15)


def test_long_rollout_segments_laid_out_on_host(env):
    """1100 steps: segments of 34 steps are laid out on the host and run
    launch by launch; the whole-rollout tape (offsets chained on the device)
    gives the same losses and gradients"""
    torch, oracle, E, params, zs, hs = env
    steps = 1100
    dims, ps = DIMS[:2], params[:2]
    true = [(p[0] * 0.9, p[1] * 1.2) for p in ps]
    tgts = _refs(oracle, true, zs[:2], hs[:2], steps)
    ens = E.Ensemble(dims, ps, zs[:2], hs[:2], steps)
    tgt = ens.pack(tgts)
    ens.set_tape("segments")
    l0, g0, h0 = ens.loss_grad(tgt, want_h0_grad=True)
    assert ens.graph_stats()[0] == 0  # not run as a graph
    ens.set_tape("full")
    l1, g1, h1 = ens.loss_grad(tgt, want_h0_grad=True)
    assert ens.graph_stats()[0] >= 1
    np.testing.assert_allclose(l1, l0, rtol=1e-12, atol=0)
    np.testing.assert_allclose(g1, g0, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(h1.cpu().numpy(), h0.cpu().numpy(), rtol=1e-12, atol=1e-15)


def test_fd_arm_agrees_with_adjoint(env):
    """central FD of the plain drop-in (the comparison arm) against the
    ensemble adjoint on one instance, at a point where no decision flips"""
    torch, oracle, E, params, zs, hs = env
    b = 3
    true = (params[b][0] * 0.95, params[b][1] * 1.1)
    tgt = _refs(oracle, [true], [zs[b]], [hs[b]], STEPS)[0]
    ens = E.Ensemble([DIMS[b]], [params[b]], [zs[b]], [hs[b]], STEPS)
    loss, grad = ens.loss_grad(ens.pack([tgt]))
    s = E.FDSession(zs[b], hs[b], params[b][0], params[b][1], STEPS, tgt)
    try:
        f0, g = s.fd_grad(params[b][0], params[b][1], rel_step=1e-7)
    finally:
        s.close()
    assert f0 == pytest.approx(loss[0], rel=1e-12)
    assert g[0] == pytest.approx(grad[0, 0], rel=2e-4)
    assert g[1] == pytest.approx(grad[0, 1], rel=2e-3)


def test_calibration_recovers_parameters(env):
    torch, oracle, E, params, zs, hs = env
    true = params[:4]
    dims = DIMS[:4]
    steps = 80
    tgts = _refs(oracle, true, zs[:4], hs[:4], steps)
    p0 = [(p[0] * 1.08, p[1] * 0.92) for p in true]
    ens = E.Ensemble(dims, p0, zs[:4], hs[:4], steps)
    out = E.calibrate(ens, ens.pack(tgts), p0, iters=60, p_true=true, tol=1e-3)
    assert out["converged_at"] is not None, out["rel_err"]
    assert np.all(out["rel_err"] < 1e-3)
