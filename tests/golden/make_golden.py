"""Regenerate the reference fixtures in this directory.

Runs the reference's own classes, compiled from its sources into
oracle/_ref/libwpref.so by ``make -C oracle ref`` (only possible where the
reference checkout is present), on seeded synthetic inputs, and stores inputs
and outputs as small .npz files.  The GPU tests compare against these
fixtures and against the oracle; they never need the reference itself.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

from oracle_lib import DBL_MAX, Reference  # noqa: E402
from whatprot_gb300.model import dye_seq_string  # noqa: E402
from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_radiometries  # noqa: E402


def ragged(ds):
    flat, off = ds.ragged()
    return flat, off


def classify_fixture(name, C, T, P, lmin, lmax, nreads, cutoff, seed, block=False, maxc=None, mint=0):
    sm = paper_model(C)
    if block:
        sm.p_initial_block, sm.p_cyclic_block = 0.07, 0.025
        sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    ds = random_dye_seqs(P, C, lmin, lmax, max_per_channel=maxc, min_total=mint, seed=seed)
    rads, true_ids = simulate_radiometries(sm, ds, T, nreads, seed=seed + 1)
    ref = Reference()
    rid, rsc, rtot, _ = ref.classify(sm, T, ds, rads, cutoff if cutoff is not None else DBL_MAX, threads=8)
    flat, off = ragged(ds)
    np.savez_compressed(os.path.join(HERE, name), C=C, T=T, cutoff=np.nan if cutoff is None else cutoff,
                        block=block, seqs=flat, offsets=off, ids=ds.ids, counts=ds.counts, rads=rads,
                        true_ids=true_ids, ref_id=rid, ref_score=rsc, ref_total=rtot)
    print(name, rads.shape, "top-1 vs truth", float(np.mean(rid == true_ids)))


def pair_fixture(name, C, T, P, nreads, seed):
    """Per-pair reference probabilities (pruned and unpruned) with blocks."""
    sm = paper_model(C)
    sm.p_initial_block, sm.p_cyclic_block = 0.07, 0.025
    sm.p_initial_detach, sm.p_initial_detach_decay = 0.03, 0.04
    ds = random_dye_seqs(P, C, 4, 14, max_per_channel=4, min_total=1, seed=seed)
    rads, _ = simulate_radiometries(sm, ds, T, nreads, seed=seed + 1)
    ref = Reference()
    dmax = ds.max_num_dyes(T)
    probs = np.zeros((2, rads.shape[0], P))
    for i in range(rads.shape[0]):
        for j in range(P):
            s = dye_seq_string(ds.seqs[j])
            probs[0, i, j] = ref.probability(sm, T, s, rads[i], dmax, 5.0)
            probs[1, i, j] = ref.probability(sm, T, s, rads[i], dmax, DBL_MAX)
    flat, off = ragged(ds)
    np.savez_compressed(os.path.join(HERE, name), C=C, T=T, seqs=flat, offsets=off, ids=ds.ids,
                        counts=ds.counts, rads=rads, dmax=dmax, prob_cut5=probs[0], prob_nocut=probs[1])
    print(name, probs.shape, "nonzero pruned", int(np.sum(probs[0] > 0)))


def fit_fixture(name, C, T, seq_str, nreads, threshold, seed, block=False):
    """HMMFitter::fit of the reference on simulated reads of one dye-seq,
    from a seeded perturbation (x0.5..x1.5) of the generating model."""
    import copy
    from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
    true = paper_model(C)
    if block:
        true.p_initial_block, true.p_cyclic_block = 0.07, 0.025
        true.p_initial_detach, true.p_initial_detach_decay = 0.03, 0.04
    seq = parse_dye_seq(seq_str)
    ds = DyeSeqSet(num_channels=C, seqs=[seq], counts=np.array([1], np.int32), ids=np.array([0], np.int32))
    rads, _ = simulate_radiometries(true, ds, T, nreads, seed=seed)
    rng = np.random.default_rng(seed + 1)
    start = copy.deepcopy(true)
    f = lambda: rng.uniform(0.5, 1.5)
    start.p_edman_failure *= f()
    start.p_detach *= f()
    start.p_initial_detach *= f()
    start.p_initial_detach_decay *= f()
    start.p_initial_block *= f()
    start.p_cyclic_block *= f()
    for cm in start.channel_models:
        cm.p_bleach *= f()
        cm.p_dud *= f()
    out, ll, step, secs = Reference().fit(start, T, seq_str, rads, threshold)
    def params(m):
        get = (lambda c, k: getattr(m.channel_models[c], k)) if hasattr(m, "channel_models") else (
            lambda c, k: getattr(m, k)[c])
        return np.array([m.p_edman_failure, m.p_detach, m.p_initial_detach, m.p_initial_detach_decay,
                         m.p_initial_block, m.p_cyclic_block]
                        + [get(c, "p_bleach") for c in range(C)] + [get(c, "p_dud") for c in range(C)])
    np.savez_compressed(os.path.join(HERE, name), C=C, T=T, seq=seq, seq_str=seq_str, rads=rads,
                        threshold=threshold, start=params(start), bg_sig=[cm.bg_sig for cm in true.channel_models],
                        sig=[cm.sig for cm in true.channel_models], ref_params=params(out), ref_log_l=ll,
                        ref_step=step)
    print(name, rads.shape, "ref fit", params(out), ll, step, f"{secs:.1f}s")


def nn_fixture(name, C, T, P, lmin, lmax, per_peptide, nreads, k, sig, h, cutoff, seed):
    """NNClassifier and HybridClassifier of the reference on a simulated
    dye-track training set."""
    from whatprot_gb300.simulate import simulate_dye_track_set
    sm = paper_model(C)
    ds = random_dye_seqs(P, C, lmin, lmax, max_per_channel=5, min_total=1, seed=seed)
    dts = simulate_dye_track_set(sm, ds, T, per_peptide, seed=seed + 1)
    rads, true_ids = simulate_radiometries(sm, ds, T, nreads, seed=seed + 2)
    ref = Reference()
    nc, ids, sc, tot, bid, bsc, btot, _ = ref.nn_classify(sm, T, dts, rads, k, sig, h)
    hid, hsc, htot, _ = ref.hybrid_classify(sm, T, dts, ds, rads, k, sig, h, cutoff)
    flat, off = ragged(ds)
    np.savez_compressed(os.path.join(HERE, name), C=C, T=T, k=k, sig=sig, h=h, cutoff=cutoff, seqs=flat,
                        offsets=off, ids=ds.ids, counts=ds.counts, tracks=dts.tracks, src_off=dts.src_off,
                        src_id=dts.src_id, src_count=dts.src_count, src_hits=dts.src_hits, rads=rads,
                        true_ids=true_ids, nn_ncand=nc, nn_ids=ids, nn_scores=sc, nn_total=tot, nn_best_id=bid,
                        nn_best_score=bsc, nn_best_total=btot, hy_id=hid, hy_score=hsc, hy_total=htot)
    print(name, len(dts), "tracks,", rads.shape[0], "reads; hybrid top-1 vs truth",
          float(np.mean(hid == true_ids)), "nn best vs truth", float(np.mean(bid == true_ids)))


def nn_wide_fixture(name, C, T, P, lmin, lmax, per_peptide, nreads, k, sig, h, cutoff, seed):
    """The same at the benchmark's k on a larger training set, too large to
    store: the dye-tracks are regenerated from the stored dye-seqs by the
    oracle's seeded, single-threaded simulate dt (wpo_simulate_dt), so the
    fixture holds the dye-seqs, the seed, the reads and the reference's
    outputs."""
    from oracle_lib import Oracle
    sm = paper_model(C)
    ds = random_dye_seqs(P, C, lmin, lmax, max_per_channel=5, min_total=1, seed=seed)
    dts, _ = Oracle().simulate_dt(sm, T, ds, per_peptide, seed + 1)
    rads, true_ids = simulate_radiometries(sm, ds, T, nreads, seed=seed + 2)
    ref = Reference()
    nc, ids, sc, tot, bid, bsc, btot, secs = ref.nn_classify(sm, T, dts, rads, k, sig, h)
    hid, hsc, htot, hsecs = ref.hybrid_classify(sm, T, dts, ds, rads, k, sig, h, cutoff)
    flat, off = ragged(ds)
    np.savez_compressed(os.path.join(HERE, name), C=C, T=T, k=k, sig=sig, h=h, cutoff=cutoff, seqs=flat,
                        offsets=off, ids=ds.ids, counts=ds.counts, per_peptide=per_peptide, track_seed=seed + 1,
                        num_tracks=len(dts), rads=rads, true_ids=true_ids, nn_ncand=nc, nn_ids=ids, nn_scores=sc,
                        nn_total=tot, nn_best_id=bid, nn_best_score=bsc, nn_best_total=btot, hy_id=hid,
                        hy_score=hsc, hy_total=htot)
    print(name, len(dts), "tracks,", rads.shape[0], "reads; hybrid top-1 vs truth",
          float(np.mean(hid == true_ids)), f"nn {secs:.1f}s hybrid {hsecs:.1f}s")


def sim_fixture(name, seed):
    """Statistics of the reference's generate_dye_track: per dye-seq the mean
    live dye count per (t, c) and the fraction of undetectable tracks over
    200,000 draws, for a model with blocks and initial detach."""
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block = 0.05, 0.02
    sm.p_initial_detach, sm.p_initial_detach_decay = 0.04, 0.3
    T = 12
    seqs = ["0.1.2.0.1", ".00..1.22.0.1.2", "2..1..0"]
    ref = Reference()
    means, sq, trivial = [], [], []
    n = 200000
    for i, s in enumerate(seqs):
        tr = ref.generate_dye_tracks(sm, T, s, n, seed + i).astype(np.float64)
        means.append(tr.mean(axis=0))
        sq.append((tr ** 2).mean(axis=0))
        trivial.append(float(np.mean(np.all(tr[:, 0, :] == 0, axis=1))))
    np.savez_compressed(os.path.join(HERE, name), T=T, seqs=np.array(seqs), n=n, mean=np.array(means),
                        meansq=np.array(sq), trivial=np.array(trivial),
                        model=np.array([sm.p_initial_block, sm.p_cyclic_block, sm.p_initial_detach,
                                        sm.p_initial_detach_decay]))
    print(name, "trivial fractions", trivial)


def dedup_fixture(name, seed):
    """The reference's dedup_dye_tracks (on its vendored MapReduce-MPI) over
    dye-tracks from its own generate_dye_track: six dye-seqs, ids repeated
    across dye-seqs and counts that differ between instances of one id (the
    reduce keeps the first instance's count), plus a few all-zero tracks
    (dedup keeps them; only generate_dye_tracks drops them).  Output in
    canonical order (tracks lexicographic, sources by id)."""
    sm = paper_model(3)
    T = 10
    seqs = ["0.1.2.0.1", ".00..1.22.0.1.2", "2..1..0", "0..1", "22.1", "1.1.1..0"]
    seq_ids = [5, 9, 5, -3, 7, 9]
    ref = Reference()
    rng = np.random.default_rng(seed)
    tracks, ids, cnts = [], [], []
    for i, s in enumerate(seqs):
        tr = ref.generate_dye_tracks(sm, T, s, 500, seed + i)
        tracks.append(tr)
        ids += [seq_ids[i]] * len(tr)
        cnts += list(rng.integers(1, 4, len(tr)))
    tracks = np.concatenate(tracks)
    perm = rng.permutation(len(tracks))
    tracks, ids, cnts = tracks[perm], np.array(ids, np.int32)[perm], np.array(cnts, np.int32)[perm]
    out = ref.dedup_dye_tracks(tracks, ids, cnts)
    np.savez_compressed(os.path.join(HERE, name), T=T, C=3, tracks=tracks, ids=ids, cnts=cnts,
                        out_tracks=out.tracks, out_src_off=out.src_off, out_src_id=out.src_id,
                        out_src_count=out.src_count, out_src_hits=out.src_hits)
    print(name, len(tracks), "instances ->", len(out), "tracks,", len(out.src_id), "sources")


if __name__ == "__main__":
    if not Reference.available():
        sys.exit("oracle/_ref/libwpref.so missing: run `make -C oracle ref` where the reference is present")
    which = sys.argv[1:] or ["classify", "pairs", "fit", "nn", "sim", "dedup"]
    if "classify" in which:
        classify_fixture("classify_c2_t8.npz", 2, 8, 100, 6, 12, 300, 5.0, seed=101)
        classify_fixture("classify_c3_t16.npz", 3, 16, 60, 8, 30, 60, 5.0, seed=202, maxc=5, mint=1)
        classify_fixture("classify_c2_t6_block_nocut.npz", 2, 6, 30, 4, 10, 40, None, seed=303, block=True)
    if "pairs" in which:
        pair_fixture("pairs_c3_t6_block.npz", 3, 6, 12, 10, seed=404)
    if "fit" in which:
        fit_fixture("fit_c2_t8.npz", 2, 8, "..0.1.0..1", 400, 1e-6, seed=505)
        fit_fixture("fit_c2_t6_block.npz", 2, 6, "0.1.01", 300, 1e-6, seed=606, block=True)
    if "nn" in which:
        nn_fixture("nn_c2_t8.npz", 2, 8, 60, 6, 12, 100, 200, 300, 0.5, 20, 5.0, seed=707)
        nn_fixture("nn_c3_t16.npz", 3, 16, 80, 8, 24, 60, 120, 200, 0.5, 30, 5.0, seed=808)
    if "nn" in which or "nnwide" in which:
        nn_wide_fixture("nn_c3_t16_2k.npz", 3, 16, 2000, 8, 30, 100, 100, 10000, 0.5, 200, 5.0, seed=1111)
    if "sim" in which:
        sim_fixture("sim_tracks_c3_t12.npz", seed=909)
    if "dedup" in which:
        dedup_fixture("dedup_c3_t10.npz", seed=1010)
