"""SCIDDICA-T adjoint (opencal_gb300.adjoint): forward bit-exact with the
oracle; gradients w.r.t. p_r, p_eps and h0 against central finite
differences -- of the GPU forward and of the CPU oracle (serial OpenCAL's
arithmetic) -- at a point away from switching points (the FD step is far
smaller than any decision margin it would have to cross)."""
import numpy as np
import pytest

from opencal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROWS, COLS, STEPS, SEED = 96, 88, 40, 23
P_R, P_EPS = 0.5, 0.001
TARGET = (0.42, 0.0015)


@pytest.fixture(scope="module")
def setup():
    import torch

    import opencal_gb300 as cal
    import oracle
    cal.build()
    oracle.build()
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    _, tgt, _ = oracle.sciddicaT(z, h, STEPS, toroidal=False, p_r=TARGET[0], p_eps=TARGET[1])
    dev = torch.device("cuda")
    return cal, oracle, torch, z, h, tgt, dev


def _loss_np(hT, tgt):
    return float(((hT - tgt) ** 2).sum())


def test_forward_matches_oracle(setup):
    cal, oracle, torch, z, h, tgt, dev = setup
    hT = cal.adjoint.rollout(torch.from_numpy(z).to(dev), torch.from_numpy(h).to(dev), P_R, P_EPS, STEPS)
    _, ref, _ = oracle.sciddicaT(z, h, STEPS, toroidal=False, p_r=P_R, p_eps=P_EPS)
    assert hT.cpu().numpy().tobytes() == ref.tobytes()


def _grads(setup):
    cal, oracle, torch, z, h, tgt, dev = setup
    zt = torch.from_numpy(z).to(dev)
    h0 = torch.from_numpy(h).to(dev).requires_grad_(True)
    pr = torch.tensor(P_R, dtype=torch.float64, device=dev, requires_grad=True)
    pe = torch.tensor(P_EPS, dtype=torch.float64, device=dev, requires_grad=True)
    hT = cal.adjoint.rollout(zt, h0, pr, pe, STEPS)
    L = ((hT - torch.from_numpy(tgt).to(dev)) ** 2).sum()
    L.backward()
    return float(L), float(pr.grad), float(pe.grad), h0.grad.cpu().numpy()


def _fd(f, x, d):
    return (f(x + d) - f(x - d)) / (2 * d)


def test_gradients_vs_gpu_finite_differences(setup):
    cal, oracle, torch, z, h, tgt, dev = setup
    L, gr, ge, gh = _grads(setup)
    zt = torch.from_numpy(z).to(dev)

    def L_gpu(pr=P_R, pe=P_EPS, h0=h):
        with torch.no_grad():
            hT = cal.adjoint.rollout(zt, torch.from_numpy(h0).to(dev), pr, pe, STEPS)
        return _loss_np(hT.cpu().numpy(), tgt)

    fd_r = _fd(lambda x: L_gpu(pr=x), P_R, 1e-7)
    fd_e = _fd(lambda x: L_gpu(pe=x), P_EPS, 1e-10)
    assert gr != 0 and abs(gr - fd_r) <= 1e-5 * abs(fd_r), (gr, fd_r)
    assert ge != 0 and abs(ge - fd_e) <= 1e-4 * abs(fd_e), (ge, fd_e)
    # directional derivative along v, supported on cells well inside the source
    rng = np.random.default_rng(5)
    v = np.where(h > 0.05, rng.standard_normal(h.shape), 0.0)
    fd_v = _fd(lambda s: L_gpu(h0=h + s * v), 0.0, 1e-8)
    an_v = float((gh * v).sum())
    assert abs(an_v - fd_v) <= 1e-5 * abs(fd_v), (an_v, fd_v)


def test_gradients_vs_oracle_finite_differences(setup):
    """Finite differences of serial OpenCAL's arithmetic (the CPU oracle)."""
    cal, oracle, torch, z, h, tgt, dev = setup
    L, gr, ge, gh = _grads(setup)

    def L_cpu(pr):
        _, hT, _ = oracle.sciddicaT(z, h, STEPS, toroidal=False, p_r=pr, p_eps=P_EPS)
        return _loss_np(hT, tgt)

    assert abs(L - L_cpu(P_R)) <= 1e-12 * L
    fd_r = _fd(L_cpu, P_R, 1e-7)
    assert abs(gr - fd_r) <= 1e-5 * abs(fd_r), (gr, fd_r)


def test_config_size_gradients_vs_gpu_finite_differences():
    """The calibration configuration itself: 1024 x 1024, T = 2000 steps,
    DEM and source from seed 3, target from a forward run at p_r = 0.42,
    p_eps = 0.0015, gradient at (0.5, 0.001) with sqrt(T) checkpoints.  The
    forward gives the split step's bits (the oracle-pinned plain step); the
    gradients agree with central differences of the GPU forward to 1e-4
    relative (the differences' own truncation and rounding at this size)."""
    import torch

    import opencal_gb300 as cal
    cal.build()
    rows = cols = 1024
    steps = 2000
    z, h = W.sciddicaT_inputs(rows, cols, seed=3)
    dev = torch.device("cuda")
    zt = torch.from_numpy(z).to(dev)
    with torch.no_grad():
        tgt = cal.adjoint.rollout(zt, torch.from_numpy(h).to(dev), 0.42, 0.0015, steps)
    _, ref, _ = cal.sciddicaT(z, h, steps, toroidal=False, p_r=0.42, p_eps=0.0015, mode=cal.MODE_FUSED)
    assert tgt.cpu().numpy().tobytes() == ref.tobytes()
    h0 = torch.from_numpy(h).to(dev).requires_grad_(True)
    pr = torch.tensor(P_R, dtype=torch.float64, device=dev, requires_grad=True)
    pe = torch.tensor(P_EPS, dtype=torch.float64, device=dev, requires_grad=True)
    L = ((cal.adjoint.rollout(zt, h0, pr, pe, steps) - tgt) ** 2).sum()
    L.backward()

    def L_gpu(p_r=P_R, p_eps=P_EPS, hh=h):
        with torch.no_grad():
            hT = cal.adjoint.rollout(zt, torch.from_numpy(hh).to(dev), p_r, p_eps, steps)
            return float(((hT - tgt) ** 2).sum())

    fd_r = _fd(lambda x: L_gpu(p_r=x), P_R, 1e-7)
    fd_e = _fd(lambda x: L_gpu(p_eps=x), P_EPS, 1e-10)
    assert float(pr.grad) != 0 and abs(float(pr.grad) - fd_r) <= 1e-4 * abs(fd_r), (float(pr.grad), fd_r)
    assert float(pe.grad) != 0 and abs(float(pe.grad) - fd_e) <= 1e-4 * abs(fd_e), (float(pe.grad), fd_e)
    rng = np.random.default_rng(7)
    v = np.where(h > 0.05, rng.standard_normal(h.shape), 0.0)
    fd_v = _fd(lambda s: L_gpu(hh=h + s * v), 0.0, 1e-8)
    an_v = float((h0.grad.cpu().numpy() * v).sum())
    assert abs(an_v - fd_v) <= 1e-4 * abs(fd_v), (an_v, fd_v)
