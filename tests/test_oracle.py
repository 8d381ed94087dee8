"""The oracle (CPU FP64 restatement) against the reference's own goldens,
against fixtures recorded from the reference, and (where the reference build
is present) against the reference live.  Also checks the closed-form pruning
boxes the CUDA kernels rely on against the oracle's literal prune passes."""
import numpy as np
import pytest

from conftest import load_fixture
from oracle_lib import DBL_MAX
from whatprot_gb300.model import SequencingModel, dye_seq_string, parse_dye_seq
from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_radiometries


def test_peptide_hmm_goldens(oracle, goldens):
    sm = SequencingModel.from_json(goldens["model"])
    seq = parse_dye_seq(goldens["dye_seq"])
    for case in goldens["cases"]:
        cut = DBL_MAX if case["dist_cutoff"] is None else case["dist_cutoff"]
        p, logp, _ = oracle.probability(sm, goldens["num_timesteps"], seq,
                                        np.array(case["rad"]), goldens["max_num_dyes"], cut)
        exp = case["expected"]
        if exp == 0.0:
            assert p == 0.0 and logp == -np.inf, case["name"]
        else:
            assert abs(p - exp) <= 1e-9 * abs(exp), (case["name"], p, exp)
            assert abs(logp - np.log(exp)) <= 1e-9 * abs(np.log(exp)) + 1e-12, case["name"]


@pytest.mark.parametrize("name", ["classify_c2_t8.npz", "classify_c3_t16.npz",
                                  "classify_c2_t6_block_nocut.npz"])
def test_classify_fixture(oracle, name):
    z, ds = load_fixture(name)
    sm = paper_model(int(z["C"]))
    if bool(z["block"]):
        sm.p_initial_block, sm.p_cyclic_block = 0.07, 0.025
        sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    cut = DBL_MAX if np.isnan(z["cutoff"]) else float(z["cutoff"])
    oid, osc, otot = oracle.classify(sm, int(z["T"]), ds, z["rads"], cut, threads=4)
    assert np.array_equal(oid, z["ref_id"])
    np.testing.assert_allclose(osc, z["ref_score"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(otot, z["ref_total"], rtol=1e-12, atol=0)


def test_pair_fixture(oracle):
    z, ds = load_fixture("pairs_c3_t6_block.npz")
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block = 0.07, 0.025
    sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    T, dmax = int(z["T"]), int(z["dmax"])
    for i in range(z["rads"].shape[0]):
        for j in range(len(ds)):
            for key, cut in (("prob_cut5", 5.0), ("prob_nocut", DBL_MAX)):
                p, _, _ = oracle.probability(sm, T, ds.seqs[j], z["rads"][i], dmax, cut)
                exp = z[key][i, j]
                assert abs(p - exp) <= 1e-12 * abs(exp), (i, j, key, p, exp)


def closed_form_boxes(oracle, sm, T, seq, rad, dmax, cut):
    """The boxes the kernels use: L_t = suffix max of cmin, U_t = min(D+1,
    prefix min of cmax); empty iff some L_t >= U_t."""
    C = sm.num_channels
    lo = np.zeros((T, C), int)
    hi = np.zeros((T, C), int)
    for t in range(T):
        a, b = oracle.emission_range(sm, rad, t, dmax, cut)
        lo[t], hi[t] = a, b
    D = np.array([np.sum(np.asarray(seq) == c) for c in range(C)])
    L = np.maximum.accumulate(lo[::-1], axis=0)[::-1]
    U = np.minimum(np.minimum.accumulate(hi, axis=0), D[None, :] + 1)
    return bool(np.any(L >= U)), L, U


@pytest.mark.parametrize("C,T,cut", [(2, 8, 5.0), (3, 10, 5.0), (3, 10, 2.5), (1, 6, 3.0), (4, 5, 5.0)])
def test_closed_form_pruning_boxes(oracle, C, T, cut):
    sm = paper_model(C)
    ds = random_dye_seqs(25, C, 3, 14, max_per_channel=4, seed=C * 100 + T)
    rads, _ = simulate_radiometries(sm, ds, T, 40, seed=C * 7 + T)
    # perturb some reads to exercise empty and odd boxes
    rng = np.random.default_rng(5)
    rads[::5] += rng.normal(0, 0.8, rads[::5].shape)
    dmax = ds.max_num_dyes(T)
    n_empty = n_full = 0
    for i in range(rads.shape[0]):
        for j in range(len(ds)):
            empty, lo, hi = oracle.pruned_boxes(sm, T, ds.seqs[j], rads[i], dmax, cut)
            e2, L, U = closed_form_boxes(oracle, sm, T, ds.seqs[j], rads[i], dmax, cut)
            assert empty == e2, (i, j)
            if not empty:
                n_full += 1
                np.testing.assert_array_equal(lo, L)
                np.testing.assert_array_equal(hi, U)
            else:
                n_empty += 1
    assert n_empty > 0 and n_full > 0


def test_oracle_matches_reference_live(oracle, reference):
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block = 0.05, 0.02
    sm.channel_models[0].interactions[1] = 0.9
    sm.channel_models[2].flat_interactions[2] = 0.95
    ds = random_dye_seqs(15, 3, 5, 16, max_per_channel=4, min_total=1, seed=77)
    rads, _ = simulate_radiometries(sm, ds, 7, 12, seed=78)
    dmax = ds.max_num_dyes(7)
    for i in range(rads.shape[0]):
        for j in range(len(ds)):
            for cut in (5.0, DBL_MAX):
                p, _, _ = oracle.probability(sm, 7, ds.seqs[j], rads[i], dmax, cut)
                r = reference.probability(sm, 7, dye_seq_string(ds.seqs[j]), rads[i], dmax, cut)
                assert p == r or abs(p - r) <= 1e-12 * abs(r)


def test_improve_fit_matches_reference_live(oracle, reference):
    sm = paper_model(2)
    sm.p_initial_block, sm.p_cyclic_block = 0.05, 0.02
    sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    ds = random_dye_seqs(3, 2, 6, 10, max_per_channel=3, min_total=1, seed=9)
    rads, _ = simulate_radiometries(sm, ds, 6, 8, seed=10)
    dmax = ds.max_num_dyes(6)
    for i in range(rads.shape[0]):
        s = ds.seqs[i % 3]
        _, _, so = oracle.improve_fit(sm, 6, s, rads[i], dmax)
        _, sr = reference.improve_fit(sm, 6, dye_seq_string(s), rads[i], dmax)
        a, b = so.as_dict(6, 2), sr.as_dict(6, 2)
        for k in a:
            if k.startswith("emis"):  # emission statistics: no reference counterpart
                continue
            x = np.concatenate([np.ravel(v) for v in a[k]])
            y = np.concatenate([np.ravel(v) for v in b[k]])
            np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-300)


def nn_fixture_inputs(oracle, name):
    """A kNN fixture's inputs: the stored dye-track set, or for the larger
    fixture the set regenerated from its dye-seqs by the oracle's seeded
    simulate dt (the set the reference was run on)."""
    from whatprot_gb300.io import DyeTrackSet
    z, ds = load_fixture(name)
    sm = paper_model(int(z["C"]))
    if "tracks" in z.files:
        dts = DyeTrackSet(z["tracks"], z["src_off"], z["src_id"], z["src_count"], z["src_hits"])
    else:
        dts, _ = oracle.simulate_dt(sm, int(z["T"]), ds, int(z["per_peptide"]), int(z["track_seed"]))
        assert len(dts) == int(z["num_tracks"])
    return z, ds, dts, sm


NN_FIXTURES = ["nn_c2_t8.npz", "nn_c3_t16.npz", "nn_c3_t16_2k.npz"]


@pytest.mark.parametrize("name", NN_FIXTURES)
def test_nn_oracle_vs_reference_fixture(oracle, name):
    """The oracle's kd-tree selection (the reference's tree and KBest,
    restated) reproduces the reference's kNN and hybrid results: totals and
    score vectors to 1e-12, the same candidate ids except where the
    reference's heap picks among equal scores at the h-th place, the same
    hybrid top-1 ids and adjusted scores to 1e-12 on every other read."""
    from conftest import nn_lists_match
    z, ds, dts, sm = nn_fixture_inputs(oracle, name)
    T = int(z["T"])
    k, sig, h, cut = int(z["k"]), float(z["sig"]), int(z["h"]), float(z["cutoff"])
    rads = z["rads"]
    nc, ids, sc, tot = oracle.nn_classify(sm, T, dts, rads, k, sig, h)
    np.testing.assert_allclose(tot, z["nn_total"], rtol=1e-12, atol=0)
    ties = []
    for r in range(len(nc)):
        ok, tie = nn_lists_match(ids[r], sc[r], nc[r], z["nn_ids"][r], z["nn_scores"][r], z["nn_ncand"][r], 1e-12)
        assert ok, r
        if tie:
            ties.append(r)
    hid, hsc, htot = oracle.hybrid_classify(sm, T, dts, ds, rads, k, sig, h, cut)
    for r in range(len(nc)):
        if r in ties:  # another subset of the tied candidates reached the HMM
            continue
        assert hid[r] == z["hy_id"][r], r
        adj, radj = hsc[r] / htot[r], z["hy_score"][r] / z["hy_total"][r]
        assert abs(adj - radj) <= 1e-12 * abs(radj), (r, adj, radj)
    assert len(ties) <= 0.2 * len(nc)


def test_nn_prefix_selection_differs_from_the_reference(oracle):
    """The shortest-prefix selection (WP_NN_PREFIX) keeps fewer far tracks
    than the reference's kd-tree search: its totals are never above the
    reference's, and below it on some reads."""
    z, ds, dts, sm = nn_fixture_inputs(oracle, "nn_c2_t8.npz")
    nc, ids, sc, tot = oracle.nn_classify(sm, int(z["T"]), dts, z["rads"], int(z["k"]), float(z["sig"]),
                                          int(z["h"]), selection="prefix")
    assert np.all(tot <= z["nn_total"] * (1 + 1e-12))
    assert np.any(tot < z["nn_total"] * (1 - 1e-9))


def test_oracle_emission_posteriors_sum_to_timesteps():
    """The oracle's emission statistics: at every emission the posterior over
    each channel's dye count (detached state at 0) sums to 1, so each
    channel's weights sum to reads x timesteps, and the weighted mean
    intensity of count n is near n mu for the generating model."""
    from oracle_lib import Oracle, WpoFitSums
    from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
    from whatprot_gb300.simulate import paper_model, simulate_radiometries
    sm = paper_model(2)
    seq = parse_dye_seq("..0.1.0..1")
    one = DyeSeqSet(2, [seq], np.array([0], np.int32), np.array([1], np.int32))
    rads, _ = simulate_radiometries(sm, one, 8, 300, seed=13)
    s = WpoFitSums()
    for r in rads:
        Oracle().improve_fit(sm, 8, seq, r, 2, sums=s)
    d = s.as_dict(8, 2)
    assert np.allclose(d["emis_w"].sum(axis=1), 300 * 8, rtol=1e-12)
    for c in range(2):
        for n in (1, 2):
            assert abs(d["emis_x"][c, n] / d["emis_w"][c, n] - n) < 0.05
