"""Parity of the GPU kNN stage (wp_nn_classify) and hybrid classifier
(wp_hybrid_classify) with the oracle and with the reference.

Two k-hit selections (wp_nn_set_selection): "kdtree", the reference's
(its kd-tree built over the tracks in upload order, searched with KBest;
the default), and "prefix", the shortest distance-ordered prefix reaching k
hits.  Each is compared with the oracle's restatement of the same selection.

Tolerances.  The kd-tree replay decides every push with FP64 distances
summed as the reference sums them, so its kept set is the reference's; the
brute-force collect keeps the same set (FP32 screening, FP64 at the
boundary).  Near entries' weights are FP64 as in the reference, far ones
FP32 (below 1e-8 of the largest weight).  So candidate lists must match the
oracle's / reference's for every read except where the reference's heap
picks among equal scores at the h-th place (named per read, at most a
fifth of the reads), with scores within 1e-5 of the list's largest and the
best score and total within 1e-5 relative.  The prefix selection's boundary
entry is decided by FP32 distances: its lists must match the oracle's for
>= 98 % of reads, scores within 2e-5."""
import numpy as np
import pytest

from conftest import GOLDEN, load_fixture  # noqa: F401
from whatprot_gb300 import capi
from whatprot_gb300.io import DyeTrackSet
from whatprot_gb300.model import DyeSeqSet
from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_dye_track_set, simulate_radiometries

pytestmark = pytest.mark.gpu
REL = 2e-5     # prefix selection (FP32 boundary)
REL_KD = 1e-5  # kd-tree selection
SELECTIONS = ["kdtree", "prefix"]


def _data(C, T, P, per, nreads, seed, inter=False, lmin=6, lmax=16):
    sm = paper_model(C)
    if inter and C > 1:
        sm.channel_models[0].interactions[1] = 0.9
        sm.channel_models[1].flat_interactions[0] = 0.95
    ds = random_dye_seqs(P, C, lmin, lmax, max_per_channel=5, min_total=1, seed=seed)
    dts = simulate_dye_track_set(sm, ds, T, per, seed=seed + 1)
    rads, ids = simulate_radiometries(sm, ds, T, nreads, seed=seed + 2)
    return sm, ds, dts, rads, ids


def _compare(gpu, ora, what, selection):
    """Candidate lists (ids, scores), totals and best scores of two kNN
    results; returns the reads whose lists differ only by a tie at the h-th
    place."""
    from conftest import nn_lists_match
    gnc, gid, gsc, gtot = gpu
    onc, oid, osc, otot = ora
    R = len(gnc)
    rel = REL_KD if selection == "kdtree" else REL
    same, ties = 0, []
    for r in range(R):
        ok, tie = nn_lists_match(gid[r], gsc[r], gnc[r], oid[r], osc[r], onc[r], rel)
        if not ok:
            continue
        same += 1
        if tie:
            ties.append(r)
        assert abs(gtot[r] - otot[r]) <= rel * abs(otot[r]) + 1e-300, (what, r, gtot[r], otot[r])
        if gnc[r] > 0:
            gb, ob = np.max(gsc[r, :gnc[r]]), np.max(osc[r, :onc[r]])
            assert abs(gb - ob) <= rel * abs(ob) + 1e-300, (what, r, gb, ob)
    need = R if selection == "kdtree" else 0.98 * R
    assert same >= need, f"{what}: candidate lists equal for {same}/{R} reads"
    assert len(ties) <= 0.2 * R, f"{what}: {len(ties)} reads tied at the h-th place"
    return ties


NN_CASES = [
    # C, T, P, per, reads, k, sig, h, interactions
    (2, 8, 50, 60, 150, 200, 0.5, 20, False),
    (3, 16, 60, 40, 100, 150, 0.5, 30, False),
    (1, 6, 30, 50, 80, 100, 0.7, 10, False),     # DP 16
    (4, 16, 40, 30, 60, 120, 0.5, 40, False),    # DP 64
    (2, 10, 40, 50, 80, 150, 0.5, 25, True),
    (2, 8, 10, 20, 60, 100000, 0.5, 1024, False),  # k above every hit: all tracks kept
]


@pytest.mark.parametrize("selection", SELECTIONS)
@pytest.mark.parametrize("case", NN_CASES, ids=[f"C{c[0]}T{c[1]}k{c[5]}h{c[7]}{'I' if c[8] else ''}"
                                                 for c in NN_CASES])
def test_nn_vs_oracle(gpu_ctx, oracle, case, selection):
    C, T, P, per, nreads, k, sig, h, inter = case
    sm, ds, dts, rads, _ = _data(C, T, P, per, nreads, seed=100 + C * 7 + T, inter=inter)
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_tracks(dts)
    gpu_ctx.set_nn_selection(selection)
    try:
        g = gpu_ctx.nn_classify(rads, k, sig, h)
    finally:
        gpu_ctx.set_nn_selection("kdtree")
    o = oracle.nn_classify(sm, T, dts, rads, k, sig, h, selection=selection)
    _compare(g, o, f"kNN {case} {selection}", selection)


@pytest.mark.parametrize("selection", SELECTIONS)
def test_hybrid_vs_oracle(gpu_ctx, oracle, selection):
    """The same selection on both sides: top-1 ids equal and adjusted scores
    to 1e-5 (2e-5 prefix) wherever the kNN candidate lists are equal."""
    from conftest import nn_lists_match
    sm, ds, dts, rads, _ = _data(3, 16, 60, 40, 100, seed=44)
    k, sig, h, cut = 150, 0.5, 30, 5.0
    gpu_ctx.upload_model(sm, 16)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gpu_ctx.set_nn_selection(selection)
    try:
        gnc, gid, gsc, gtot = gpu_ctx.nn_classify(rads, k, sig, h)
        hid, hsc, htot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    finally:
        gpu_ctx.set_nn_selection("kdtree")
    onc, oid, osc, otot = oracle.nn_classify(sm, 16, dts, rads, k, sig, h, selection=selection)
    oh_id, oh_sc, oh_tot = oracle.hybrid_classify(sm, 16, dts, ds, rads, k, sig, h, cut, selection=selection)
    rel = REL_KD if selection == "kdtree" else REL
    same = 0
    for r in range(len(gnc)):
        ok, tie = nn_lists_match(gid[r], gsc[r], gnc[r], oid[r], osc[r], onc[r], rel)
        if ok and not tie:
            same += 1
            assert hid[r] == oh_id[r], r
            assert abs(hsc[r] / htot[r] - oh_sc[r] / oh_tot[r]) <= rel * abs(oh_sc[r] / oh_tot[r]) + 1e-300
    assert same >= (0.8 if selection == "kdtree" else 0.98) * len(gnc)


def test_nn_deterministic(gpu_ctx):
    sm, ds, dts, rads, _ = _data(3, 16, 60, 40, 100, seed=5)
    gpu_ctx.upload_model(sm, 16)
    gpu_ctx.upload_tracks(dts)
    a = gpu_ctx.nn_classify(rads, 150, 0.5, 30)
    b = gpu_ctx.nn_classify(rads, 150, 0.5, 30)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["nn_c2_t8.npz", "nn_c3_t16.npz", "nn_c3_t16_2k.npz"])
def test_nn_and_hybrid_vs_reference(gpu_ctx, oracle, name):
    """The default (kd-tree) selection against the reference's recorded
    NNClassifier and HybridClassifier results: candidate lists equal on
    every read up to ties at the h-th place, best scores and totals within
    1e-5; hybrid top-1 ids equal and adjusted scores within 1e-5 on every
    read without such a tie.  nn_c3_t16_2k is the benchmark's k = 10,000
    on 118,488 tracks (regenerated by the oracle's seeded generator)."""
    from test_oracle import nn_fixture_inputs
    z, ds, dts, sm = nn_fixture_inputs(oracle, name)
    T = int(z["T"])
    k, sig, h, cut = int(z["k"]), float(z["sig"]), int(z["h"]), float(z["cutoff"])
    rads = z["rads"]
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gpu_ctx.set_nn_selection("kdtree")
    g = gpu_ctx.nn_classify(rads, k, sig, h)
    ties = _compare(g, (z["nn_ncand"], z["nn_ids"], z["nn_scores"], z["nn_total"]), f"reference {name}", "kdtree")
    hid, hsc, htot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    index = {int(i): n for n, i in enumerate(ds.ids)}
    hmm_ties = []
    for r in range(len(hid)):
        if r in ties:
            continue
        if hid[r] != z["hy_id"][r]:
            # the HMM over the same candidates: accepted where the two
            # peptides' probabilities agree to 1e-5 (the FP32 engine's
            # tolerance), checked with the oracle's FP64 log P
            ll = oracle.loglik_all(sm, T, ds, rads[r:r + 1], cut)[0]
            a, b = index[int(hid[r])], index[int(z["hy_id"][r])]
            assert abs(ll[a] - ll[b]) <= 1e-5, (name, r, hid[r], z["hy_id"][r], ll[a], ll[b])
            hmm_ties.append(r)
        adj_g = hsc[r] / htot[r]
        adj_r = z["hy_score"][r] / z["hy_total"][r]
        assert abs(adj_g - adj_r) <= REL_KD * abs(adj_r) + 1e-300, (name, r, adj_g, adj_r)
    assert len(hmm_ties) <= 0.05 * len(hid), (name, hmm_ties)


def test_prefix_selection_vs_reference(gpu_ctx, oracle):
    """The prefix selection keeps fewer far tracks than the reference: its
    totals never exceed the reference's, and its hybrid top-1 still agrees
    for >= 95 % of reads."""
    from test_oracle import nn_fixture_inputs
    z, ds, dts, sm = nn_fixture_inputs(oracle, "nn_c2_t8.npz")
    T = int(z["T"])
    k, sig, h, cut = int(z["k"]), float(z["sig"]), int(z["h"]), float(z["cutoff"])
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gpu_ctx.set_nn_selection("prefix")
    try:
        gnc, gid, gsc, gtot = gpu_ctx.nn_classify(z["rads"], k, sig, h)
        hid, _, _ = gpu_ctx.hybrid_classify(z["rads"], k, sig, h, cut)
    finally:
        gpu_ctx.set_nn_selection("kdtree")
    assert np.all(gtot <= z["nn_total"] * (1 + REL))
    assert np.mean(hid == z["hy_id"]) >= 0.95


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


@pytest.mark.parametrize("selection", SELECTIONS)
@pytest.mark.parametrize("which", ["k1", "k_all_but_one"])
def test_nn_threshold_extremes(gpu_ctx, oracle, which, selection):
    """k = 1 (the k-hit radius is the nearest entry's) and k one below every
    hit (the radius is the farthest entry's): the reads' distance bins sit
    at the edges of their estimated windows, the selection stays exact."""
    sm, ds, dts, rads, _ = _data(2, 8, 40, 30, 80, seed=444)
    gpu_ctx.upload_model(sm, 8)
    gpu_ctx.upload_tracks(dts)
    k = 1 if which == "k1" else int(dts.src_hits.sum()) - 1
    gpu_ctx.set_nn_selection(selection)
    try:
        g = gpu_ctx.nn_classify(rads, k, 0.5, 10)
    finally:
        gpu_ctx.set_nn_selection("kdtree")
    o = oracle.nn_classify(sm, 8, dts, rads, k, 0.5, 10, selection=selection)
    _compare(g, o, f"kNN k={k}", selection)
