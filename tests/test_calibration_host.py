"""Host-side logic of the batched calibration (opencal_gb300.ensemble), no GPU:
the per-instance BFGS with Armijo backtracking, vectorised over instances,
reaches the minimum of known quadratics in log-parameter space (each
instance its own curvature and optimum, one started at its optimum); and the
recovery fraction counts only the identifiable parameters of each instance."""
import numpy as np

from opencal_gb300 import ensemble as E


def _quadratics(B, seed=3):
    rng = np.random.default_rng(seed)
    x_star = rng.uniform(-3.0, 0.0, size=(B, 2))
    A = np.empty((B, 2, 2))
    for b in range(B):
        q, _ = np.linalg.qr(rng.normal(size=(2, 2)))
        A[b] = q @ np.diag(rng.uniform(0.5, 50.0, size=2)) @ q.T
    return x_star, A


def _f_g(x, x_star, A):
    d = x - x_star
    Ad = np.einsum("bij,bj->bi", A, d)
    return np.einsum("bi,bi->b", d, Ad), 2.0 * Ad


def test_bfgs_reaches_every_instance_minimum():
    B = 6
    x_star, A = _quadratics(B)
    x0 = x_star + np.random.default_rng(5).uniform(-0.5, 0.5, size=(B, 2))
    x0[2] = x_star[2]  # already at its optimum: must stay there
    opt = E._BFGS(x0)
    f, g = _f_g(x0, x_star, A)
    opt.first(f, g)
    for _ in range(60):
        f, g = _f_g(opt.trial, x_star, A)
        opt.accept(f, g)
    np.testing.assert_allclose(opt.x, x_star, rtol=0, atol=1e-6)
    # accepted points never increase the loss of an instance
    assert np.all(opt.f <= _f_g(x0, x_star, A)[0] + 1e-300)


def test_bfgs_rejected_step_is_halved_and_state_kept():
    x_star, A = _quadratics(2, seed=11)
    x0 = x_star + 0.3
    opt = E._BFGS(x0, step0=50.0)  # a first step far too long
    f0, g0 = _f_g(x0, x_star, A)
    opt.first(f0, g0)
    x_before, trial = opt.x.copy(), opt.trial.copy()
    f, g = _f_g(trial, x_star, A)
    armijo = f <= f0 + 1e-4 * np.einsum("bi,bi->b", g0, trial - x0)
    opt.accept(f, g)
    for b in range(2):
        if armijo[b]:
            np.testing.assert_array_equal(opt.x[b], trial[b])
        else:
            np.testing.assert_array_equal(opt.x[b], x_before[b])
            assert opt.alpha[b] == 0.5
            np.testing.assert_allclose(opt.trial[b], x_before[b] + 0.5 * (trial[b] - x_before[b]), rtol=1e-15)


def test_recovered_fraction_counts_identifiable_parameters_only():
    p_true = np.array([[0.5, 1e-3], [0.4, 2e-3], [0.3, 3e-3], [0.6, 4e-3]])
    params = p_true.copy()
    params[0, 0] *= 1 + 5e-4   # within 1e-3
    params[1, 1] *= 1 + 2e-3   # off, but p_eps of instance 1 is not identifiable
    params[2, 0] *= 1 - 2e-3   # off and identifiable
    params[3, :] *= 1 + 2e-3   # both off, neither identifiable
    mask = np.ones((4, 2), dtype=bool)
    mask[1, 1] = False
    mask[3, :] = False
    assert E.recovered_fraction(params, p_true, mask) == 0.75
    assert E.recovered_fraction(params, p_true, np.ones((4, 2), dtype=bool)) == 0.25
    assert E.recovered_fraction(params, p_true, mask, tol=3e-3) == 1.0
