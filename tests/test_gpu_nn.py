"""Parity of the GPU kNN stage (wp_nn_classify) and hybrid classifier
(wp_hybrid_classify) with the oracle and with the reference.

Tolerances.  Distances are FP32 on the GPU and FP64 in the oracle, so the
entry at the k-hit boundary can differ when two distances agree to about
1e-6: a read's candidate set must match the oracle's exactly for at least
98 % of reads, and where it matches, scores and totals must agree to a
relative 2e-5 (FP32 distances inside exp(-d^2 / 2 sig^2)).  Against the
reference the k-hit set is allowed to differ (its kd-tree search can keep a
few more far tracks), so the check there is on decisions: the hybrid's top-1
id and the kNN best id agree for at least 95 % of reads, and the hybrid's
scores agree to 1e-5 relative wherever the reference's kNN candidate set
and total equal ours."""
import numpy as np
import pytest

from conftest import GOLDEN, load_fixture  # noqa: F401
from whatprot_gb300 import capi
from whatprot_gb300.io import DyeTrackSet
from whatprot_gb300.model import DyeSeqSet
from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_dye_track_set, simulate_radiometries

pytestmark = pytest.mark.gpu
REL = 2e-5


def _data(C, T, P, per, nreads, seed, inter=False, lmin=6, lmax=16):
    sm = paper_model(C)
    if inter and C > 1:
        sm.channel_models[0].interactions[1] = 0.9
        sm.channel_models[1].flat_interactions[0] = 0.95
    ds = random_dye_seqs(P, C, lmin, lmax, max_per_channel=5, min_total=1, seed=seed)
    dts = simulate_dye_track_set(sm, ds, T, per, seed=seed + 1)
    rads, ids = simulate_radiometries(sm, ds, T, nreads, seed=seed + 2)
    return sm, ds, dts, rads, ids


def _compare(gpu, ora, what, min_frac=0.98):
    gnc, gid, gsc, gtot = gpu
    onc, oid, osc, otot = ora
    R = len(gnc)
    same = 0
    for r in range(R):
        a = list(gid[r, :gnc[r]])
        b = list(oid[r, :onc[r]])
        if gnc[r] == onc[r] and a == b:
            same += 1
            assert abs(gtot[r] - otot[r]) <= REL * abs(otot[r]) + 1e-300, (what, r, gtot[r], otot[r])
            np.testing.assert_allclose(gsc[r, :gnc[r]], osc[r, :onc[r]], rtol=REL, atol=1e-300,
                                       err_msg=f"{what} read {r}")
    assert same >= min_frac * R, f"{what}: candidate lists equal for {same}/{R} reads"


NN_CASES = [
    # C, T, P, per, reads, k, sig, h, interactions
    (2, 8, 50, 60, 150, 200, 0.5, 20, False),
    (3, 16, 60, 40, 100, 150, 0.5, 30, False),
    (1, 6, 30, 50, 80, 100, 0.7, 10, False),     # DP 16
    (4, 16, 40, 30, 60, 120, 0.5, 40, False),    # DP 64
    (2, 10, 40, 50, 80, 150, 0.5, 25, True),
    (2, 8, 10, 20, 60, 100000, 0.5, 1024, False),  # k above every hit: all tracks kept
]


@pytest.mark.parametrize("case", NN_CASES, ids=[f"C{c[0]}T{c[1]}k{c[5]}h{c[7]}{'I' if c[8] else ''}"
                                                 for c in NN_CASES])
def test_nn_vs_oracle(gpu_ctx, oracle, case):
    C, T, P, per, nreads, k, sig, h, inter = case
    sm, ds, dts, rads, _ = _data(C, T, P, per, nreads, seed=100 + C * 7 + T, inter=inter)
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_tracks(dts)
    g = gpu_ctx.nn_classify(rads, k, sig, h)
    o = oracle.nn_classify(sm, T, dts, rads, k, sig, h)
    _compare(g, o, f"kNN {case}")


def test_hybrid_vs_oracle(gpu_ctx, oracle):
    """Same k-hit semantics on both sides: top-1 ids equal where the kNN
    candidate lists are equal (>= 98 % of reads), scores to 2e-5."""
    sm, ds, dts, rads, _ = _data(3, 16, 60, 40, 100, seed=44)
    k, sig, h, cut = 150, 0.5, 30, 5.0
    gpu_ctx.upload_model(sm, 16)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gnc, gid, gsc, gtot = gpu_ctx.nn_classify(rads, k, sig, h)
    onc, oid, osc, otot = oracle.nn_classify(sm, 16, dts, rads, k, sig, h)
    hid, hsc, htot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    oh_id, oh_sc, oh_tot = oracle.hybrid_classify(sm, 16, dts, ds, rads, k, sig, h, cut)
    same = 0
    for r in range(len(gnc)):
        if gnc[r] == onc[r] and np.array_equal(gid[r, :gnc[r]], oid[r, :onc[r]]):
            same += 1
            assert hid[r] == oh_id[r], r
            assert abs(hsc[r] / htot[r] - oh_sc[r] / oh_tot[r]) <= REL * abs(oh_sc[r] / oh_tot[r]) + 1e-300
    assert same >= 0.98 * len(gnc)


def test_nn_deterministic(gpu_ctx):
    sm, ds, dts, rads, _ = _data(3, 16, 60, 40, 100, seed=5)
    gpu_ctx.upload_model(sm, 16)
    gpu_ctx.upload_tracks(dts)
    a = gpu_ctx.nn_classify(rads, 150, 0.5, 30)
    b = gpu_ctx.nn_classify(rads, 150, 0.5, 30)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def _fixture(name):
    z, ds = load_fixture(name)
    dts = DyeTrackSet(z["tracks"], z["src_off"], z["src_id"], z["src_count"], z["src_hits"])
    return z, ds, dts


@pytest.mark.parametrize("name", ["nn_c2_t8.npz", "nn_c3_t16.npz"])
def test_nn_and_hybrid_vs_reference(gpu_ctx, name):
    z, ds, dts = _fixture(name)
    C, T = int(z["C"]), int(z["T"])
    k, sig, h, cut = int(z["k"]), float(z["sig"]), int(z["h"]), float(z["cutoff"])
    sm = paper_model(C)
    rads = z["rads"]
    R = rads.shape[0]
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gnc, gid, gsc, gtot = gpu_ctx.nn_classify(rads, k, sig, h)
    best = np.array([gid[r, gnc[r] - 1] for r in range(R)])
    assert np.mean(best == z["nn_best_id"]) >= 0.95
    hid, hsc, htot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    assert np.mean(hid == z["hy_id"]) >= 0.95, np.mean(hid == z["hy_id"])
    same_set = 0
    for r in range(R):
        # the same k-hit set shows as the same candidates with the same total
        if (gnc[r] == z["nn_ncand"][r] and set(gid[r, :gnc[r]]) == set(z["nn_ids"][r, :gnc[r]])
                and abs(gtot[r] - z["nn_total"][r]) <= REL * z["nn_total"][r]):
            same_set += 1
            if hid[r] == z["hy_id"][r]:
                adj_g = hsc[r] / htot[r]
                adj_r = z["hy_score"][r] / z["hy_total"][r]
                assert abs(adj_g - adj_r) <= 1e-5 * abs(adj_r) + 1e-300, (r, adj_g, adj_r)
    assert same_set >= 0.3 * R


def test_hybrid_is_knn_then_hmm(gpu_ctx):
    """The hybrid's result equals the HMM over the kNN candidates (in
    ascending kNN score) times the candidates' subfraction."""
    sm, ds, dts, rads, _ = _data(2, 8, 50, 60, 80, seed=21)
    k, sig, h, cut = 200, 0.5, 15, 5.0
    gpu_ctx.upload_model(sm, 8)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    hid, hsc, htot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    nc, ids, sc, tot = gpu_ctx.nn_classify(rads, k, sig, h)
    index = {int(i): n for n, i in enumerate(ds.ids)}
    cand = np.concatenate([[index[int(i)] for i in ids[r, :nc[r]]] for r in range(len(nc))]).astype(np.int32)
    off = np.concatenate([[0], np.cumsum(nc)]).astype(np.int32)
    cid, csc, ctot, _ = gpu_ctx.classify(rads, cut, cand, off)
    for r in range(len(nc)):
        sub = 0.0
        for i in range(nc[r]):
            sub += (sc[r, i] / tot[r]) * float(ds.counts[index[int(ids[r, i])]])
        assert hid[r] == cid[r]
        assert hsc[r] == csc[r] * sub or (hsc[r] == 0.0 and htot[r] == 1.0)
        assert htot[r] == ctot[r] or htot[r] == 1.0


def test_nn_errors(gpu_ctx):
    sm, ds, dts, rads, _ = _data(2, 8, 10, 10, 10, seed=3)
    ctx = capi.Context(0)
    try:
        ctx.upload_model(sm, 8)
        with pytest.raises(capi.WpError) as e:
            ctx.nn_classify(rads, 10, 0.5, 5)  # no tracks yet
        assert e.value.status == 6
        ctx.upload_tracks(dts)
        with pytest.raises(capi.WpError) as e:
            ctx.nn_classify(rads, 10, 0.5, 2000)
        assert e.value.status == 5
        with pytest.raises(capi.WpError) as e:
            ctx.nn_classify(rads, 0, 0.5, 5)
        assert e.value.status == 1
        bad = DyeTrackSet(dts.tracks, dts.src_off, dts.src_id, dts.src_count, np.zeros_like(dts.src_hits))
        with pytest.raises(capi.WpError) as e:
            ctx.upload_tracks(bad)
        assert e.value.status == 1
        ctx.upload_model(sm, 9)
        with pytest.raises(capi.WpError) as e:
            ctx.nn_classify(np.zeros((2, 9, 2)), 10, 0.5, 5)  # tracks have 8 timesteps
        assert e.value.status == 6
        ctx.upload_model(sm, 8)
        empty = DyeTrackSet(np.zeros((0, 8, 2), np.int16), np.zeros(1, np.int32), np.zeros(0, np.int32),
                            np.zeros(0, np.int32), np.zeros(0, np.int32))
        ctx.upload_tracks(empty)
        nc, ids, sc, tot = ctx.nn_classify(rads, 10, 0.5, 5)
        assert np.all(nc == 0) and np.all(tot == 0.0)
    finally:
        ctx.close()


@pytest.mark.parametrize("which", ["k1", "k_all_but_one"])
def test_nn_threshold_extremes(gpu_ctx, oracle, which):
    """k = 1 (the k-hit radius is the nearest entry's) and k one below every
    hit (the radius is the farthest entry's): the reads' distance bins sit
    at the edges of their estimated windows, the selection stays exact."""
    sm, ds, dts, rads, _ = _data(2, 8, 40, 30, 80, seed=444)
    gpu_ctx.upload_model(sm, 8)
    gpu_ctx.upload_tracks(dts)
    k = 1 if which == "k1" else int(dts.src_hits.sum()) - 1
    g = gpu_ctx.nn_classify(rads, k, 0.5, 10)
    o = oracle.nn_classify(sm, 8, dts, rads, k, 0.5, 10)
    _compare(g, o, f"kNN k={k}")
