"""The learned proposal network on the GPU (wp_mlp_*): logits and gradients
against the CPU oracle (oracle/mlp_oracle.py, FP64 with BF16 rounding at the
GPU's rounding points), and what training gains.

Tolerance: the oracle rounds to BF16 where the GPU does, so only the
tensor cores' FP32 summation order differs (and the BF16 roundings it can
tip): loss within 1e-4 relative, logits within 3e-4 of the largest logit
magnitude, each gradient within 1e-3 relative Frobenius error and a cosine
similarity above 0.99999 (measured on three seeds: loss 2e-6, logits up to
9e-5, gradients up to 1e-4, cosines 1 - 1e-8)."""
import os
import sys

import numpy as np
import pytest

from whatprot_gb300 import capi
from whatprot_gb300.simulate import paper_model, random_dye_seqs

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


def _ctx(P, C=2, T=8, seed=5):
    sm = paper_model(C)
    ds = random_dye_seqs(P, C, 6, 14, max_per_channel=4, min_total=1, seed=seed)
    ctx = capi.Context(0)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    return ctx, sm, ds


def test_gradients_match_oracle():
    import torch
    import mlp_oracle
    ctx, sm, ds = _ctx(100)
    try:
        net = capi.ProposalNet(ctx, hidden=256, seed=3)
        B = 128
        rads, pep, _ = ctx.simulate_reads(B, seed=11)
        x = rads.reshape(B, -1).astype(np.float32)
        params = {n: net.get(i).astype(np.float64) for i, n in enumerate(capi.ProposalNet.PARAMS)}
        d_x = torch.from_numpy(x).cuda()
        d_y = torch.from_numpy(pep.astype(np.int32)).cuda()
        loss = net.train_step(d_x.data_ptr(), d_y.data_ptr(), B, 0.0)
        ora_loss, g, L = mlp_oracle.gradients(params, x.astype(np.float64), pep, len(ds))
        assert abs(loss - ora_loss) <= 1e-4 * max(1.0, abs(ora_loss))
        logits = net.logits(rads)
        assert np.max(np.abs(logits - L[:, :len(ds)])) <= 3e-4 * np.max(np.abs(L))
        for i, n in enumerate(capi.ProposalNet.PARAMS):
            gg = net.get(i, grad=True).astype(np.float64).reshape(g[n].shape)
            rel = np.linalg.norm(gg - g[n]) / max(np.linalg.norm(g[n]), 1e-30)
            cos = float(np.sum(gg * g[n]) / max(np.linalg.norm(gg) * np.linalg.norm(g[n]), 1e-30))
            assert rel <= 1e-3 and cos >= 0.99999, (n, rel, cos)
        net.close()
    finally:
        ctx.close()


def test_training_gains_recall_and_feeds_the_hmm():
    """What the trained network gains: recall@h of the true peptide far
    above the untrained network's, and the HMM over its proposals finds the
    full HMM's best probability for almost every read (many peptides share
    a dye-seq prefix and so tie exactly; which of the tied ids is reported is
    not compared) at the full HMM's top-1 accuracy."""
    P, T = 150, 8
    ctx, sm, ds = _ctx(P, T=T, seed=9)
    try:
        net = capi.ProposalNet(ctx, hidden=512, seed=4)
        rads, pep, _ = ctx.simulate_reads(3000, seed=99)
        ok = pep >= 0
        rads, pep = rads[ok], pep[ok]
        h = 40

        def recall():
            idx, prob, mass = net.propose(rads, h)
            return float(np.mean([pep[r] in idx[r] for r in range(len(pep))]))

        r0 = recall()
        first = net.train(16384, batch=1024, lr=1e-3, seed=1)
        last = net.train(400000, batch=1024, lr=1e-3, seed=2)
        r1 = recall()
        assert last < first - 0.5, (first, last)
        assert r0 <= 0.5 and r1 >= 0.95, (r0, r1)
        logp = ctx.loglik_all(rads, 5.0)
        full_id, _, _, _ = ctx.classify(rads, 5.0)
        mid, msc, mtot = net.hybrid_classify(rads, h, 5.0)
        index = {int(i): n for n, i in enumerate(ds.ids)}
        best = logp.max(axis=1)
        got = np.array([logp[r, index[int(mid[r])]] for r in range(len(mid))])
        found = float(np.mean(got >= best - 1e-5))
        assert found >= 0.95, found
        acc_full = float(np.mean(full_id == ds.ids[pep]))
        acc_hyb = float(np.mean(mid == ds.ids[pep]))
        assert acc_hyb >= acc_full - 0.02, (acc_hyb, acc_full)
        net.close()
    finally:
        ctx.close()


@pytest.mark.parametrize("P,h", [(3000, 200), (3000, 1000), (700, 64), (5000, 1)])
def test_topk_matches_numpy(P, h):
    """wp_mlp_propose's selection against numpy on the network's own logits:
    the h largest by (logit, index) with ties to the larger index, written
    ascending; softmax probabilities within 1e-5 relative of an FP64 softmax;
    the candidate mass (sum of probability x count) to the same tolerance.
    Shapes cover the warp kernel's threshold path, its all-keys path (P at
    most the buffer) and the exact fallback (h too large for the threshold
    buffer)."""
    ctx, sm, ds = _ctx(P, seed=P + h)
    net = capi.ProposalNet(ctx, hidden=256, seed=3)
    rng = np.random.default_rng(P)
    rads = rng.normal(1.0, 0.7, size=(300, 8, 2))
    L = net.logits(rads)[:, :P].astype(np.float64)
    idx, prob, mass = net.propose(rads, h)
    counts = np.asarray(ds.counts, np.float64)
    for r in range(rads.shape[0]):
        order = np.lexsort((np.arange(P), L[r]))  # ascending by (logit, index)
        want = order[-h:]
        assert np.array_equal(idx[r], want), r
        z = L[r] - L[r].max()
        p = np.exp(z) / np.exp(z).sum()
        assert np.allclose(prob[r], p[want], rtol=1e-5, atol=1e-30), r
        assert abs(mass[r] - float(np.sum(p[want] * counts[want]))) <= 1e-5 * max(mass[r], 1e-30), r
    net.close()
    ctx.close()
