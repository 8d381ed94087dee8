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


if __name__ == "__main__":
    if not Reference.available():
        sys.exit("oracle/_ref/libwpref.so missing: run `make -C oracle ref` where the reference is present")
    classify_fixture("classify_c2_t8.npz", 2, 8, 100, 6, 12, 300, 5.0, seed=101)
    classify_fixture("classify_c3_t16.npz", 3, 16, 60, 8, 30, 60, 5.0, seed=202, maxc=5, mint=1)
    classify_fixture("classify_c2_t6_block_nocut.npz", 2, 6, 30, 4, 10, 40, None, seed=303, block=True)
    pair_fixture("pairs_c3_t6_block.npz", 3, 6, 12, 10, seed=404)
