"""Dye-track generation and dedup on the device (wp_dedup_dye_tracks,
wp_simulate_dye_tracks) against the reference's dedup (committed fixture)
and the oracle, bit for bit: the same distinct tracks in the same
(canonical) order with the same (id, count, hits) sources.  The generated
instances are checked against the reference's generate_dye_tracks: one
peptide copy per per_peptide instances in order, statistics of the
reference's own generator, undetectable instances dropped."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_dedup import KEYS, fixture, random_cases, same_set
from whatprot_gb300 import capi
from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
from whatprot_gb300.simulate import paper_model, random_dye_seqs

pytestmark = pytest.mark.gpu


def test_dedup_matches_reference_fixture(gpu_ctx):
    z, out = fixture()
    got = gpu_ctx.dedup_dye_tracks(z["tracks"], z["ids"], z["cnts"])
    assert same_set(got, out)


def test_dedup_matches_oracle_edge_cases(gpu_ctx, oracle):
    for tr, ids, cnt in random_cases(seed=5):
        got = gpu_ctx.dedup_dye_tracks(tr, ids, cnt)
        want = oracle.dedup_dye_tracks(tr, ids, cnt)
        assert same_set(got, want), [k for k in KEYS if not np.array_equal(getattr(got, k), getattr(want, k))]


def test_dedup_widest_counts_and_many_instances(gpu_ctx, oracle):
    rng = np.random.default_rng(6)
    # counts up to 2^15 - 1 (15-bit fields, four words per 4 x 4 track)
    tr = rng.integers(0, 3, (40000, 4, 4)).astype(np.int16)
    tr[::7, 2, 1] = 32767
    ids = rng.integers(0, 50, len(tr)).astype(np.int32)
    cnt = rng.integers(1, 3, len(tr)).astype(np.int32)
    assert same_set(gpu_ctx.dedup_dye_tracks(tr, ids, cnt), oracle.dedup_dye_tracks(tr, ids, cnt))
    # 300,000 instances of 3 x 16 tracks with a few distinct values
    tr = np.minimum(rng.geometric(0.6, (300000, 16, 3)) - 1, 5).astype(np.int16)
    ids = rng.integers(0, 2000, len(tr)).astype(np.int32)
    cnt = np.ones(len(tr), np.int32)
    assert same_set(gpu_ctx.dedup_dye_tracks(tr, ids, cnt), oracle.dedup_dye_tracks(tr, ids, cnt))


def test_dedup_rejects_negative_counts(gpu_ctx):
    tr = np.zeros((3, 2, 2), np.int16)
    tr[1, 1, 0] = -1
    with pytest.raises(capi.WpError):
        gpu_ctx.dedup_dye_tracks(tr, np.zeros(3, np.int32), np.ones(3, np.int32))


def _peptides():
    sm = paper_model(3)
    ds = random_dye_seqs(300, 3, 6, 20, max_per_channel=5, min_total=1, seed=21)
    ds.counts[:] = np.random.default_rng(22).integers(1, 4, len(ds)).astype(np.int32)
    ds.ids[::9] = ds.ids[1::9][: len(ds.ids[::9])]  # some ids shared by two dye-seqs
    return sm, ds


def test_simulated_set_is_the_dedup_of_its_instances(gpu_ctx, oracle):
    sm, ds = _peptides()
    T, per = 12, 40
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    dts, itr, ipep = gpu_ctx.simulate_dye_track_set(per, seed=77, instances=True)
    n = per * int(ds.counts.sum())
    assert itr.shape == (n, T, 3) and ipep.shape == (n,)
    # instance r belongs to peptide copy r // per, copies in dye-seq order
    copy_pep = np.repeat(np.arange(len(ds)), ds.counts)
    expect = np.repeat(copy_pep, per)
    det = np.any(itr[:, 0, :] != 0, axis=1)
    assert np.array_equal(ipep[det], expect[det]) and np.all(ipep[~det] == -1)
    assert np.all(itr[~det] == 0)
    want = oracle.dedup_dye_tracks(itr[det].astype(np.int16), ds.ids[expect[det]], ds.counts[expect[det]])
    assert same_set(dts, want)
    # same seed, same set (also through reusable page-locked buffers);
    # another seed, another set
    again = gpu_ctx.simulate_dye_track_set(per, seed=77)
    assert same_set(again, dts)
    bufs = capi.DyeTrackBuffers(n, n, T, 3)
    assert same_set(gpu_ctx.simulate_dye_track_set(per, seed=77, into=bufs), dts)
    other = gpu_ctx.simulate_dye_track_set(per, seed=78)
    assert not same_set(other, dts)


def test_simulated_instances_match_reference_statistics(gpu_ctx):
    z = np.load(os.path.join(GOLDEN, "sim_tracks_c3_t12.npz"))
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block, sm.p_initial_detach, sm.p_initial_detach_decay = z["model"]
    T, n = int(z["T"]), 200000
    seqs = [parse_dye_seq(str(s)) for s in z["seqs"]]
    ds = DyeSeqSet(3, seqs, np.arange(len(seqs), dtype=np.int32), np.ones(len(seqs), np.int32))
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    dts, itr, ipep = gpu_ctx.simulate_dye_track_set(n, seed=500, instances=True)
    for i in range(len(seqs)):
        tr = itr[i * n:(i + 1) * n].astype(np.float64)
        mean, var_g = tr.mean(axis=0), tr.var(axis=0)
        var_r = z["meansq"][i] - z["mean"][i] ** 2
        se = np.sqrt(var_g / n + var_r / int(z["n"])) + 1e-12
        assert np.all(np.abs(mean - z["mean"][i]) <= 5 * se), np.max(np.abs(mean - z["mean"][i]) / se)
        triv = float(np.mean(ipep[i * n:(i + 1) * n] == -1))
        p = z["trivial"][i]
        assert abs(triv - p) <= 5 * np.sqrt(max(p, 1e-5) * (1 - p) / n) + 1e-5
    # hits per id add up to the detectable instances of that dye-seq
    for i in range(len(seqs)):
        assert dts.src_hits[dts.src_id == i].sum() == np.sum(ipep[i * n:(i + 1) * n] == i)


def test_simulated_set_feeds_the_knn(gpu_ctx):
    sm, ds = _peptides()
    T = 10
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    rads, _, _ = gpu_ctx.simulate_reads(300, seed=5)
    dts = gpu_ctx.simulate_dye_track_set(30, seed=6, to_nn=True)
    a = gpu_ctx.nn_classify(rads, 200, 0.5, 20)
    gpu_ctx.upload_tracks(dts)
    b = gpu_ctx.nn_classify(rads, 200, 0.5, 20)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_large_simulated_set_properties(gpu_ctx):
    """20,000 dye-seqs x 100 tracks (2,000,000 instances): tracks strictly
    increasing, sources ascending within a track, hits add up to the
    detectable instances."""
    sm = paper_model(3)
    ds = random_dye_seqs(20000, 3, 8, 30, max_per_channel=5, min_total=1, seed=1234)
    gpu_ctx.upload_model(sm, 16)
    gpu_ctx.upload_peptides(ds)
    dts, itr, ipep = gpu_ctx.simulate_dye_track_set(100, seed=4321, instances=True)
    flat = dts.tracks.reshape(len(dts), -1).astype(np.int64)
    diff = flat[1:] - flat[:-1]
    first = np.argmax(diff != 0, axis=1)
    assert np.all(diff[np.arange(len(diff)), first] > 0)
    d = np.diff(dts.src_id)
    inner = np.ones(len(d), bool)
    inner[dts.src_off[1:-1] - 1] = False
    assert np.all(d[inner] > 0)
    assert int(dts.src_hits.sum()) == int(np.sum(ipep >= 0))
    assert np.all(np.any(dts.tracks[:, 0, :] != 0, axis=1))


def test_most_labeled_positions(gpu_ctx, oracle):
    """A dye-seq with 15 dyes on each of 4 channels (60 labeled positions,
    the most an uploaded dye-seq carries): mean live counts per (t, c) of the
    device's instances against the oracle's generator (itself checked
    against the reference's), within 5 standard errors."""
    sm = paper_model(4)
    T, n = 10, 100000
    seq = np.full(72, -1, np.int16)
    seq[6:66] = np.arange(60) % 4
    ds = DyeSeqSet(4, [seq], np.array([1], np.int32), np.array([1], np.int32))
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    _, itr, ipep = gpu_ctx.simulate_dye_track_set(n, seed=31, instances=True)
    g = itr.astype(np.float64)
    odts, kept = oracle.simulate_dt(sm, T, ds, n, seed=41)
    w = odts.src_hits.astype(np.float64)[:, None, None]
    om = (w * odts.tracks).sum(axis=0) / n
    ov = (w * odts.tracks.astype(np.float64) ** 2).sum(axis=0) / n - om ** 2
    se = np.sqrt(g.var(axis=0) / n + ov / n) + 1e-12
    assert np.all(np.abs(g.mean(axis=0) - om) <= 5 * se), np.max(np.abs(g.mean(axis=0) - om) / se)
    assert abs(np.mean(ipep >= 0) - kept / n) <= 5 * np.sqrt(0.25 / n) + 1e-4
