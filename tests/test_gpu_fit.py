"""Parity of the GPU Baum-Welch fit (wp_fit_estep, wp_hmm_fit) with the
oracle's improve_fit and with fits recorded from the reference.

Tolerances.  E-step: each expected count is a sum over reads of FP32
state-vector products with exact power-of-two frames, accumulated in FP64;
it must match the oracle's FP64 sum to a relative 1e-5 of the sum of the
magnitudes involved (the denominator of the same parameter).  Sum of log P:
|delta| <= 1e-5 per read.  Full fit: the reference stops when the largest
parameter change falls below 1e-6, so fitted parameters are compared to
1e-4 absolute, and the detach rate curve base + initial * exp(-decay * t)
(identifiable even where base and initial trade off at decay = 0) to 1e-4.
"""
import math

import numpy as np
import pytest

from whatprot_gb300 import capi
from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
from whatprot_gb300.simulate import paper_model, simulate_radiometries

from conftest import GOLDEN  # noqa: F401

pytestmark = pytest.mark.gpu


def _model(C, block=False):
    sm = paper_model(C)
    if block:
        sm.p_initial_block, sm.p_cyclic_block = 0.07, 0.025
        sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    return sm


def _reads(sm, seq, T, n, seed):
    ds = DyeSeqSet(sm.num_channels, [seq], np.array([0], np.int32), np.array([1], np.int32))
    rads, _ = simulate_radiometries(sm, ds, T, n, seed=seed)
    return rads


def _oracle_sums(oracle, sm, T, seq, rads):
    from oracle_lib import WpoFitSums
    dmax = max(int(np.sum(seq == c)) for c in range(sm.num_channels))
    s = WpoFitSums()
    lps = []
    for r in rads:
        _, lp, _ = oracle.improve_fit(sm, T, seq, r, dmax, sums=s)
        lps.append(lp)
    return s.as_dict(T, sm.num_channels), np.array(lps)


def _close(g, o, scale, what):
    g, o = np.asarray(g, float), np.asarray(o, float)
    if g.size == 0:
        assert o.size == 0, what
        return
    err = np.max(np.abs(g - o))
    assert err <= 1e-5 * max(float(np.max(np.abs(scale))), 1e-300), (what, g, o)


ESTEP_CASES = [
    # C, T, dye-seq, reads, block
    (2, 8, "..0.1.0..1", 64, False),
    (2, 6, "0.1.01", 48, True),
    (3, 10, "0.1.2.0.1.2", 40, False),
    (1, 5, "..000", 30, True),
    (3, 16, "0.1.2.0..1.2.0..1.2.0", 24, False),   # 4/3/3 dyes, T=16
    (4, 6, "0123.0", 20, False),
    (2, 1, "01", 16, True),
]


@pytest.mark.parametrize("kernel", [0, 1], ids=["cta", "thread"])
@pytest.mark.parametrize("case", ESTEP_CASES, ids=[f"C{c[0]}T{c[1]}{'B' if c[4] else ''}" for c in ESTEP_CASES])
def test_estep_vs_oracle(gpu_ctx, oracle, case, kernel):
    C, T, seq_str, n, block = case
    gpu_ctx.fit_set_kernel(kernel)
    sm = _model(C, block)
    seq = parse_dye_seq(seq_str)
    rads = _reads(sm, seq, T, n, seed=7 * len(seq_str) + C)
    # start the E-step away from the generating model
    sm.p_edman_failure *= 1.3
    for cm in sm.channel_models:
        cm.p_bleach *= 0.8
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.fit_begin(seq, rads)
    s, sl, nz = gpu_ctx.fit_estep()
    gpu_ctx.fit_set_kernel(0)
    g = s.as_dict(T, C)
    o, lps = _oracle_sums(oracle, sm, T, seq, rads)
    assert nz == int(np.sum(~np.isfinite(lps)))
    assert abs(sl - float(np.sum(lps[np.isfinite(lps)]))) <= 1e-5 * len(rads)
    _close(g["edman_num"], o["edman"][0], o["edman"][1], "edman num")
    _close(g["edman_den"], o["edman"][1], o["edman"][1], "edman den")
    _close(g["detach_x"], o["detach_x"], o["detach_n"], "detach x")
    _close(g["detach_n"], o["detach_n"], o["detach_n"], "detach n")
    _close(g["init_block_num"], o["init_block"][0], o["init_block"][1], "initial block num")
    _close(g["init_block_den"], o["init_block"][1], o["init_block"][1], "initial block den")
    _close(g["cyc_block_num"], o["cyc_block"][0], o["cyc_block"][1], "cyclic block num")
    _close(g["cyc_block_den"], o["cyc_block"][1], o["cyc_block"][1], "cyclic block den")
    for c in range(C):
        _close(g["bleach_num"][c], o["bleach"][0][c], o["bleach"][1][c], f"bleach num {c}")
        _close(g["bleach_den"][c], o["bleach"][1][c], o["bleach"][1][c], f"bleach den {c}")
        _close(g["dud_num"][c], o["dud"][0][c], o["dud"][1][c], f"dud num {c}")
        _close(g["dud_den"][c], o["dud"][1][c], o["dud"][1][c], f"dud den {c}")


def test_estep_zero_probability_read(gpu_ctx, oracle):
    """A read no state can emit (P == 0 in FP64) adds nothing and is counted."""
    C, T = 2, 6
    sm = _model(C)
    seq = parse_dye_seq("0.1.01")
    rads = _reads(sm, seq, T, 10, seed=9)
    rads[3, 0, 0] = 1e4
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.fit_begin(seq, rads)
    s, sl, nz = gpu_ctx.fit_estep()
    o, lps = _oracle_sums(oracle, sm, T, seq, rads)
    assert not np.isfinite(lps[3])
    assert nz == 1
    _close(s.as_dict(T, C)["edman_den"], o["edman"][1], o["edman"][1], "edman den")


def test_estep_errors(gpu_ctx):
    C, T = 2, 6
    sm = _model(C)
    gpu_ctx.upload_model(sm, T)
    with pytest.raises(capi.WpError):
        gpu_ctx.fit_begin(np.array([0, 2], np.int16), np.zeros((1, T, C)))  # channel 2 of 2
    with pytest.raises(capi.WpError):
        gpu_ctx.fit_begin(np.zeros(16, np.int16), np.zeros((1, T, C)))  # 16 dyes on a channel
    inter = _model(C)
    inter.channel_models[0].interactions[1] = 0.9
    gpu_ctx.fit_begin(parse_dye_seq("01"), np.zeros((2, T, C)))
    gpu_ctx.upload_model(inter, T)
    with pytest.raises(capi.WpError) as e:
        gpu_ctx.fit_estep()
    assert e.value.status == 5
    gpu_ctx.upload_model(sm, T + 1)
    with pytest.raises(capi.WpError) as e:
        gpu_ctx.fit_estep()  # model timesteps differ from the staged reads
    assert e.value.status == 6
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.fit_begin(parse_dye_seq("01"), np.zeros((0, T, C)))
    s, sl, nz = gpu_ctx.fit_estep()
    assert s.p_edman_failure_den == 0.0 and sl == 0.0 and nz == 0


def _params(m):
    return np.array([m.p_edman_failure, m.p_detach, m.p_initial_detach, m.p_initial_detach_decay,
                     m.p_initial_block, m.p_cyclic_block]
                    + [c.p_bleach for c in m.channel_models] + [c.p_dud for c in m.channel_models])


def _detach_curve(p, T):
    t = np.arange(T - 1)
    return p[1] + p[2] * np.exp(-p[3] * t)


@pytest.mark.parametrize("name", ["fit_c2_t8.npz", "fit_c2_t6_block.npz"])
def test_fit_vs_reference(name):
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, name))
    C, T = int(z["C"]), int(z["T"])
    st = z["start"]
    sm = paper_model(C)
    (sm.p_edman_failure, sm.p_detach, sm.p_initial_detach, sm.p_initial_detach_decay,
     sm.p_initial_block, sm.p_cyclic_block) = st[:6]
    for c in range(C):
        sm.channel_models[c].p_bleach = st[6 + c]
        sm.channel_models[c].p_dud = st[6 + C + c]
    fitter = capi.HMMFitter(T, C, float(z["threshold"]), 1e9, sm, None, z["seq"])
    fitted, log_l = fitter.fit(z["rads"])
    got, ref = _params(fitted), z["ref_params"]
    assert fitter.step_size < float(z["threshold"])
    # everything but the detach triple directly; the detach rate as a curve
    keep = [0, 4, 5] + list(range(6, 6 + 2 * C))
    assert np.max(np.abs(got[keep] - ref[keep])) <= 1e-4, (got, ref)
    assert np.max(np.abs(_detach_curve(got, T) - _detach_curve(ref, T))) <= 1e-4, (got, ref)
    assert math.isfinite(log_l)
    assert abs(log_l - float(z["ref_log_l"])) <= 1e-6 * abs(float(z["ref_log_l"])) + 1e-3
    # log_likelihood of the mirror agrees with the fit's own final value
    assert abs(fitter.log_likelihood(z["rads"], fitted) - log_l) <= 1e-9 * abs(log_l)


def test_bootstrap_fit(tmp_path):
    """bootstrap_fit: the fit on all reads equals wp_hmm_fit's, rounds are
    reproducible from the seed and scatter around it, the bounds bracket the
    rounds, and the params CSV has the reference's layout."""
    import os
    from conftest import GOLDEN
    from whatprot_gb300.io import write_params
    z = np.load(os.path.join(GOLDEN, "fit_c2_t8.npz"))
    C, T = int(z["C"]), int(z["T"])
    st = z["start"]
    sm = paper_model(C)
    (sm.p_edman_failure, sm.p_detach, sm.p_initial_detach, sm.p_initial_detach_decay,
     sm.p_initial_block, sm.p_cyclic_block) = st[:6]
    for c in range(C):
        sm.channel_models[c].p_bleach = st[6 + c]
        sm.channel_models[c].p_dud = st[6 + C + c]
    ctx = capi.Context(0)
    try:
        res = ctx.bootstrap_fit(sm, T, z["seq"], z["rads"], 1e-5, 6, 0.9, seed=5)
        fitted, step, ll, _ = ctx.hmm_fit(sm, T, z["seq"], z["rads"], 1e-5)
        assert np.allclose(_params(res["best"]), _params(fitted), atol=1e-12)
        assert res["log_l"] == ll
        again = ctx.bootstrap_fit(sm, T, z["seq"], z["rads"], 1e-5, 6, 0.9, seed=5)
        assert all(np.array_equal(_params(a), _params(b)) for a, b in zip(res["models"], again["models"]))
        other = ctx.bootstrap_fit(sm, T, z["seq"], z["rads"], 1e-5, 6, 0.9, seed=6)
        assert not np.array_equal(_params(res["models"][0]), _params(other["models"][0]))
        P = np.array([_params(m) for m in res["models"]])
        lo, hi = _params(res["ci_min"]), _params(res["ci_max"])
        assert np.all(lo <= hi)
        assert np.all(P.min(axis=0) <= lo + 1e-15) and np.all(hi <= P.max(axis=0) + 1e-15)
        # rounds scatter around the full fit by a few percent of the rates
        assert np.all(np.abs(P[:, [0, 6, 7, 8, 9]] - _params(fitted)[[0, 6, 7, 8, 9]]) < 0.05)
        path = tmp_path / "params.csv"
        write_params(path, C, res["models"], res["log_ls"])
        lines = open(path).read().splitlines()
        assert lines[0] == ("p_edman_failure,p_detach,p_initial_detach,p_initial_detach_decay,p_initial_block,"
                            "p_cyclic_block,ch0:p_bleach,ch0:p_dud,ch1:p_bleach,ch1:p_dud,log(L)")
        assert len(lines) == 7 and len(lines[1].split(",")) == 11
    finally:
        ctx.close()


# ---- emission statistics and the mu / sig / bg_sig fit (no reference
# counterpart: the reference never fits them; the oracle's FP64 E-step and
# the generating model are the checks).
EMIS_CASES = [
    (2, 8, "..0.1.0..1", 48, False),
    (2, 6, "0.1.01", 40, True),
    (3, 16, "0.1.2.0..1.2.0..1.2.0", 16, False),
]


@pytest.mark.parametrize("kernel", [0, 1], ids=["cta", "thread"])
@pytest.mark.parametrize("case", EMIS_CASES, ids=[f"C{c[0]}T{c[1]}{'B' if c[4] else ''}" for c in EMIS_CASES])
def test_emission_statistics_vs_oracle(gpu_ctx, oracle, case, kernel):
    """Posterior weight per (channel, dye count) at the emissions and its
    intensity moments: within 1e-5 of the total weight (reads x timesteps)
    of the oracle's FP64 sums; the weights of each channel sum to it."""
    C, T, seq_str, n, block = case
    gpu_ctx.fit_set_kernel(kernel)
    gpu_ctx.fit_set_emission(True)
    sm = _model(C, block)
    seq = parse_dye_seq(seq_str)
    rads = _reads(sm, seq, T, n, seed=11 * len(seq_str) + C)
    sm.channel_models[0].sig *= 1.2
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.fit_begin(seq, rads)
    gpu_ctx.fit_estep()
    w, x, xx = gpu_ctx.fit_emission_sums().arrays(C)
    gpu_ctx.fit_set_emission(False)
    gpu_ctx.fit_set_kernel(0)
    o, lps = _oracle_sums(oracle, sm, T, seq, rads)
    live = int(np.sum(np.isfinite(lps)))
    total = float(live * T)
    assert np.allclose(w.sum(axis=1), total, rtol=1e-5, atol=0)
    xs = float(np.max(np.abs(rads))) + 1.0
    _close(w, o["emis_w"][:, :w.shape[1]], total, "emission weight")
    _close(x, o["emis_x"][:, :w.shape[1]], total * xs, "emission x")
    _close(xx, o["emis_xx"][:, :w.shape[1]], total * xs * xs, "emission xx")


def test_fit_emission_recovers_generating_model(gpu_ctx):
    """fit_emission on reads of a known model from a +-30 % start: every rate
    and each channel's mu, sig and bg_sig back to the generating values
    within the statistical error of 20,000 reads."""
    C, T = 2, 8
    truth = _model(C)
    truth.channel_models[0].mu, truth.channel_models[1].mu = 1.0, 0.8
    truth.channel_models[0].sig, truth.channel_models[1].sig = 0.16, 0.12
    truth.channel_models[0].bg_sig, truth.channel_models[1].bg_sig = 0.05, 0.04
    seq = parse_dye_seq("..0.1.0..1.1")
    rads = _reads(truth, seq, T, 20000, seed=5)
    start = _model(C)
    for cm, f in zip(start.channel_models, (1.3, 0.7)):
        cm.mu, cm.sig, cm.bg_sig = 0.9 * f, 0.14 * f, 0.06 / f
    fitted, step, ll, iters = gpu_ctx.hmm_fit(start, T, seq, rads, 1e-6, 600.0, fit_emission=True)
    assert step < 1e-6 and math.isfinite(ll) and iters > 2
    for c, (cf, ct) in enumerate(zip(fitted.channel_models, truth.channel_models)):
        assert abs(cf.mu - ct.mu) <= 0.01 * ct.mu, (c, cf.mu, ct.mu)
        assert abs(cf.sig - ct.sig) <= 0.05 * ct.sig, (c, cf.sig, ct.sig)
        assert abs(cf.bg_sig - ct.bg_sig) <= 0.08 * ct.bg_sig, (c, cf.bg_sig, ct.bg_sig)
        assert abs(cf.p_bleach - ct.p_bleach) <= 0.01
        assert abs(cf.p_dud - ct.p_dud) <= 0.02
    assert abs(fitted.p_edman_failure - truth.p_edman_failure) <= 0.01
    # without fit_emission the emission parameters stay the start's
    held, _, _, _ = gpu_ctx.hmm_fit(start, T, seq, rads[:2000], 1e-4, 600.0)
    assert all(h.mu == s.mu and h.sig == s.sig and h.bg_sig == s.bg_sig
               for h, s in zip(held.channel_models, start.channel_models))


# ---- batched EM instances (bootstrap rounds at once)
def _fixture_start():
    import os
    z = np.load(os.path.join(GOLDEN, "fit_c2_t8.npz"))
    C, T = int(z["C"]), int(z["T"])
    st = z["start"]
    sm = paper_model(C)
    (sm.p_edman_failure, sm.p_detach, sm.p_initial_detach, sm.p_initial_detach_decay,
     sm.p_initial_block, sm.p_cyclic_block) = st[:6]
    for c in range(C):
        sm.channel_models[c].p_bleach = st[6 + c]
        sm.channel_models[c].p_dud = st[6 + C + c]
    return z, sm, C, T


SUM_FIELDS = ["p_edman_failure_num", "p_edman_failure_den", "p_initial_block_num", "p_initial_block_den",
              "p_cyclic_block_num", "p_cyclic_block_den"]


def _sum_vec(s, T, C):
    v = [getattr(s, f) for f in SUM_FIELDS]
    v += list(s.p_detach_x[:T - 1]) + list(s.p_detach_n[:T - 1])
    v += list(s.p_bleach_num[:C]) + list(s.p_bleach_den[:C]) + list(s.p_dud_num[:C]) + list(s.p_dud_den[:C])
    return np.array(v, np.float64)


def test_estep_batch_matches_single_esteps(gpu_ctx):
    """wp_fit_estep_batch: each instance's expected counts and log P equal a
    single E-step with that model over that read list (FP64 sums formed in
    another order: 1e-10 relative)."""
    import copy
    z, sm, C, T = _fixture_start()
    rads, seq = z["rads"], z["seq"]
    rng = np.random.default_rng(3)
    models = []
    for b in range(3):
        m = copy.deepcopy(sm)
        m.p_edman_failure *= 1.0 + 0.2 * b
        m.p_detach *= 1.0 + 0.1 * b
        for cm in m.channel_models:
            cm.p_bleach *= 1.0 + 0.15 * b
        models.append(m)
    idx = rng.integers(0, len(rads), (3, 150)).astype(np.int32)
    single = []
    gpu_ctx.fit_set_emission(False)
    for b in range(3):
        gpu_ctx.upload_model(models[b], T)
        gpu_ctx.fit_begin(seq, rads[idx[b]])
        single.append(gpu_ctx.fit_estep())
    gpu_ctx.upload_model(models[0], T)
    gpu_ctx.fit_begin(seq, rads)
    gpu_ctx.fit_set_emission(False)
    out, sl, nz = gpu_ctx.fit_estep_batch(models, idx)
    for b in range(3):
        a, e = _sum_vec(out[b], T, C), _sum_vec(single[b][0], T, C)
        assert np.allclose(a, e, rtol=1e-10, atol=1e-12), (b, np.max(np.abs(a - e) / np.maximum(np.abs(e), 1e-300)))
        assert abs(sl[b] - single[b][1]) <= 1e-10 * abs(single[b][1]) and nz[b] == single[b][2]


def test_fit_batch_matches_sequential_fits(gpu_ctx):
    """wp_hmm_fit_batch: every instance converges to the fit wp_hmm_fit
    reaches on the same reads (FP64 sums formed in another order)."""
    z, sm, C, T = _fixture_start()
    rads, seq = z["rads"], z["seq"]
    idx = np.random.default_rng(4).integers(0, len(rads), (4, len(rads))).astype(np.int32)
    fits, lls, steps = gpu_ctx.hmm_fit_batch(sm, T, seq, rads, idx, 1e-5)
    for b in range(4):
        f, step, ll, _ = gpu_ctx.hmm_fit(sm, T, seq, rads[idx[b]], 1e-5)
        assert np.allclose(_params(fits[b]), _params(f), rtol=1e-7, atol=1e-10), b
        assert abs(lls[b] - ll) <= 1e-9 * abs(ll)
        # the step is a difference of nearly equal parameter sets, and the
        # detach M-step is a least-squares fit stopped after 10 iterations,
        # so the sums' rounding shows in it far more than in the parameters
        # (same iteration count: same size)
        assert abs(steps[b] - step) <= 5e-2 * max(step, 1e-12)


@pytest.mark.parametrize("kernel", [0, 1], ids=["cta", "thread"])
def test_fit_vs_fp64_oracle_em(gpu_ctx, kernel):
    """A full fit (HMMFitter::fit to a 1e-6 step from a perturbed start) with
    the GPU's FP32 E-step against the same EM with the oracle's FP64 E-step
    and the same host M-step (tests/oracle_lib.py oracle_em): every fitted
    rate, the detach curve included, within 1e-5 absolute."""
    from oracle_lib import oracle_em
    sm = paper_model(3)
    seq = parse_dye_seq("..0.1.2..0.1..2.0")
    one = DyeSeqSet(3, [seq], np.array([0], np.int32), np.array([1], np.int32))
    rads, _ = simulate_radiometries(sm, one, 10, 1500, seed=31)
    start = paper_model(3)
    start.p_edman_failure *= 1.4
    start.p_detach *= 0.6
    for c, cm in enumerate(start.channel_models):
        cm.p_bleach *= (1.3, 0.7, 1.2)[c]
        cm.p_dud *= (0.6, 1.4, 1.1)[c]
    ctx = capi.Context(0)
    try:
        ctx.upload_model(start, 10)
        ctx.fit_set_kernel(kernel)
        g, _, _, g_it = ctx.hmm_fit(start, 10, seq, rads, 1e-6)
    finally:
        ctx.close()
    o, _, o_it = oracle_em(start, 10, seq, rads, 1e-6, threads=8)
    curve = lambda m: np.array([m.p_detach_at(t) for t in range(9)])
    assert abs(g.p_edman_failure - o.p_edman_failure) <= 1e-5
    assert np.max(np.abs(curve(g) - curve(o))) <= 1e-5
    for a, b in zip(g.channel_models, o.channel_models):
        assert abs(a.p_bleach - b.p_bleach) <= 1e-5
        assert abs(a.p_dud - b.p_dud) <= 1e-5
    assert abs(g_it - o_it) <= 2
