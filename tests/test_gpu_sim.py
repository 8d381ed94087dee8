"""The GPU read simulator (wp_simulate_reads) against the reference's own
generate_dye_track: statistics recorded from the reference
(tests/golden/sim_tracks_c3_t12.npz, 200,000 draws per dye-seq).  The
random streams differ, so the comparison is statistical: mean live dye
counts per (t, c) within 5 standard errors of both samples, undetectable
fractions within 5 binomial standard errors, and intensities standardised by
the channel model are N(0, 1)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
from whatprot_gb300.simulate import paper_model

pytestmark = pytest.mark.gpu


def _model():
    z = np.load(os.path.join(GOLDEN, "sim_tracks_c3_t12.npz"))
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block, sm.p_initial_detach, sm.p_initial_detach_decay = z["model"]
    return z, sm


def test_tracks_match_reference_statistics(gpu_ctx):
    z, sm = _model()
    T, n = int(z["T"]), 200000
    for i, s in enumerate(z["seqs"]):
        ds = DyeSeqSet(3, [parse_dye_seq(str(s))], np.array([7], np.int32), np.array([1], np.int32))
        gpu_ctx.upload_model(sm, T)
        gpu_ctx.upload_peptides(ds)
        rads, pep, tr = gpu_ctx.simulate_reads(n, seed=1000 + i, tracks=True)
        tr = tr.astype(np.float64)
        mean = tr.mean(axis=0)
        var_g = tr.var(axis=0)
        var_r = z["meansq"][i] - z["mean"][i] ** 2
        se = np.sqrt(var_g / n + var_r / int(z["n"])) + 1e-12
        assert np.all(np.abs(mean - z["mean"][i]) <= 5 * se), (s, np.max(np.abs(mean - z["mean"][i]) / se))
        triv = float(np.mean(pep == -1))
        p = z["trivial"][i]
        assert abs(triv - p) <= 5 * np.sqrt(max(p, 1e-5) * (1 - p) / n) + 1e-5
        # every read's peptide is the only one, except the undetectable ones
        assert set(np.unique(pep)) <= {-1, 0}
        # intensities standardised by the channel model (mu = 1, no interactions)
        mu = tr
        sig = np.sqrt(0.00667 ** 2 + mu * 0.16 ** 2)
        zz = (rads - mu) / sig
        assert abs(zz.mean()) < 0.01 and abs(zz.std() - 1.0) < 0.01


def test_peptides_drawn_by_count_and_deterministic(gpu_ctx):
    sm = paper_model(2)
    seqs = [parse_dye_seq(s) for s in ["0.1", "1..0.1", "00.1", ".1.1"]]
    counts = np.array([1, 2, 3, 4], np.int32)
    ds = DyeSeqSet(2, seqs, np.arange(4, dtype=np.int32), counts)
    gpu_ctx.upload_model(sm, 6)
    gpu_ctx.upload_peptides(ds)
    n = 400000
    rads, pep, _ = gpu_ctx.simulate_reads(n, seed=42)
    freq = np.array([np.sum(pep == i) for i in range(4)], np.float64)
    # undetectable reads are a few per mille; compare the drawn shares
    share = freq / freq.sum()
    expect = counts / counts.sum()
    assert np.all(np.abs(share - expect) <= 5 * np.sqrt(expect * (1 - expect) / n) + 0.002)
    rads2, pep2, _ = gpu_ctx.simulate_reads(n, seed=42)
    assert np.array_equal(rads, rads2) and np.array_equal(pep, pep2)
    rads3, _, _ = gpu_ctx.simulate_reads(1000, seed=43)
    assert not np.array_equal(rads[:1000], rads3)
