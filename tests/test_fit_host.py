"""The detach M-step's bounded least squares (wp_fit_offset_exponential),
host code of the library: runs without a GPU.

It restates least_squares_fit_of_offset_exponential
(util/levmar-helper.cc:44-85: weights by sqrt(w), bounds [0, 1], holds as
lb = ub, 10 iterations) with its own projected Levenberg-Marquardt, so it is
compared with the reference's levmar on the problems the EM loop poses
(starts near the optimum), not bit for bit."""
import numpy as np
import pytest

from whatprot_gb300 import capi


def model(p, n):
    t = np.arange(n)
    return p[0] + p[1] * np.exp(-p[2] * t)


def cost(p, y, w):
    return float(np.sum(w * (y - model(p, len(y))) ** 2))


def test_recovers_exact_curve():
    truth = np.array([0.04, 0.12, 0.35])
    for n in (6, 15, 30):
        y = model(truth, n)
        w = np.linspace(1e3, 2e2, n)
        p = capi.fit_offset_exponential(y, w, truth * np.array([1.1, 0.9, 1.05]))
        assert np.allclose(p, truth, atol=1e-6), (n, p)


def test_bounds_and_holds():
    rng = np.random.default_rng(3)
    for _ in range(50):
        n = int(rng.integers(2, 20))
        y = rng.uniform(-0.5, 1.5, n)
        w = rng.uniform(1, 100, n)
        p0 = rng.uniform(0, 1, 3)
        held = [bool(rng.random() < 0.4) for _ in range(3)]
        p = capi.fit_offset_exponential(y, w, p0, held)
        assert np.all(p >= 0.0) and np.all(p <= 1.0)
        for k in range(3):
            if held[k]:
                assert p[k] == p0[k]
        assert cost(p, y, w) <= cost(np.clip(p0, 0, 1), y, w) * (1 + 1e-12)


def test_empty_and_zero_weight_points():
    p = capi.fit_offset_exponential([], [], [0.1, 0.2, 0.3])
    assert np.array_equal(p, [0.1, 0.2, 0.3])
    # A timestep with no expected detach mass (n = 0, y = 0/0) is ignored.
    y = np.array([0.05, np.nan, 0.05, 0.05])
    w = np.array([100.0, 0.0, 100.0, 100.0])
    p = capi.fit_offset_exponential(y, w, [0.01, 0.0, 0.0], (False, True, True))
    assert abs(p[0] - 0.05) < 1e-9


def test_matches_reference_levmar_fixed_point(reference):
    """Called repeatedly from its own output, as the EM loop does (each
    M-step starts from the last estimate), each method settles on a fixed
    point.  Where the reference's levmar settles, both agree; ours never
    ends at a higher cost."""
    rng = np.random.default_rng(7)
    settled = 0
    for trial in range(60):
        n = int(rng.integers(5, 30))
        truth = np.array([rng.uniform(0.01, 0.1), rng.uniform(0.02, 0.3), rng.uniform(0.05, 0.8)])
        w = rng.uniform(1e3, 1e5, n)
        y = model(truth, n) + rng.normal(0, 1, n) / np.sqrt(w)
        a = truth.copy()
        b = truth.copy()
        for _ in range(40):
            a2 = reference.offset_exponential(y, w, a)
            b2 = capi.fit_offset_exponential(y, w, b)
            da, db = np.max(np.abs(a2 - a)), np.max(np.abs(b2 - b))
            a, b = a2, b2
            if da < 1e-12 and db < 1e-12:
                break
        assert cost(b, y, w) <= cost(a, y, w) * (1 + 1e-9), (trial, a, b)
        if da < 1e-12:
            settled += 1
            assert np.max(np.abs(a - b)) < 1e-6, (trial, a, b)
    assert settled >= 50


def test_emission_mstep_matches_scipy():
    """wp_fit_emission_mstep reaches the maximum of the expected
    log-likelihood that an independent optimiser (scipy Nelder-Mead on the
    same objective) finds, from a far start; a channel with weight at n = 0
    only fits bg_sig and keeps mu and sig."""
    from scipy.optimize import minimize
    rng = np.random.default_rng(1)
    C, N = 3, 16
    mu_t, sig_t, bg_t = np.array([1.1, 0.9, 1.0]), np.array([0.15, 0.2, 0.1]), np.array([0.01, 0.02, 0.03])
    w = np.zeros((C, N))
    x = np.zeros((C, N))
    xx = np.zeros((C, N))
    for c in range(C):
        for n in range(5 if c < 2 else 1):
            v = bg_t[c] ** 2 + mu_t[c] * n * sig_t[c] ** 2
            s = rng.normal(mu_t[c] * n, np.sqrt(v), 4000)
            w[c, n], x[c, n], xx[c, n] = len(s), s.sum(), (s * s).sum()
    mu0, sig0, bg0 = [1.5, 0.6, 1.2], [0.1, 0.3, 0.2], [0.03, 0.01, 0.05]
    mu, sig, bg, step = capi.emission_mstep(w, x, xx, mu0, sig0, bg0)

    def negq(th, c):
        m_, s_, b_ = np.exp(th)
        q = 0.0
        for n in range(N):
            if w[c, n] <= 0:
                continue
            mm, v = m_ * n, b_ ** 2 + m_ * n * s_ ** 2
            q += -0.5 * w[c, n] * np.log(v) - (xx[c, n] - 2 * mm * x[c, n] + mm * mm * w[c, n]) / (2 * v)
        return -q

    for c in range(2):
        res = minimize(negq, np.log([1.0, 0.1, 0.01]), args=(c,), method="Nelder-Mead",
                       options={"xatol": 1e-12, "fatol": 1e-12, "maxiter": 20000, "maxfev": 40000})
        assert -negq(np.log([mu[c], sig[c], bg[c]]), c) >= -res.fun - 1e-6
        assert np.allclose([mu[c], sig[c], bg[c]], np.exp(res.x), rtol=1e-5)
    assert mu[2] == mu0[2] and sig[2] == sig0[2]
    assert abs(bg[2] - np.sqrt(xx[2, 0] / w[2, 0])) <= 1e-8
    assert step >= abs(mu[0] - mu0[0])
