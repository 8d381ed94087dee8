"""Dye-track dedup on the CPU: the oracle's restatement of dedup_dye_tracks
and the package's host dedup against the reference's own dedup (its
MapReduce-MPI job, compiled from source into oracle/_ref) -- through the
committed fixture everywhere, and live where the reference build exists."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
from whatprot_gb300.simulate import dedup_dye_tracks, paper_model, simulate_dye_track_set

KEYS = ("tracks", "src_off", "src_id", "src_count", "src_hits")


def same_set(a, b):
    return all(np.array_equal(getattr(a, k), getattr(b, k)) for k in KEYS)


def fixture():
    z = np.load(os.path.join(GOLDEN, "dedup_c3_t10.npz"))
    from whatprot_gb300.io import DyeTrackSet
    out = DyeTrackSet(z["out_tracks"], z["out_src_off"], z["out_src_id"], z["out_src_count"], z["out_src_hits"])
    return z, out


def random_cases(seed=3):
    """(tracks, ids, counts): empty, single, all identical, all-zero rows,
    negative and extreme ids, counts that differ within one id, wide counts."""
    rng = np.random.default_rng(seed)
    cases = [(np.zeros((0, 4, 2), np.int16), np.zeros(0, np.int32), np.zeros(0, np.int32)),
             (np.ones((1, 3, 1), np.int16), np.array([7], np.int32), np.array([2], np.int32)),
             (np.full((50, 5, 3), 2, np.int16), rng.integers(0, 3, 50).astype(np.int32),
              rng.integers(1, 5, 50).astype(np.int32))]
    for n, T, C, hi in [(3000, 6, 2, 3), (8000, 12, 3, 5), (2000, 4, 4, 300)]:
        tr = rng.integers(0, hi, (n, T, C)).astype(np.int16)
        tr[: n // 20] = 0
        ids = rng.choice(np.array([-2**31, -5, 0, 3, 2**31 - 1], np.int64), n).astype(np.int32)
        cases.append((tr, ids, rng.integers(1, 9, n).astype(np.int32)))
    return cases


def test_oracle_matches_reference_fixture(oracle):
    z, out = fixture()
    got = oracle.dedup_dye_tracks(z["tracks"], z["ids"], z["cnts"])
    assert same_set(got, out)
    # the fixture has all-zero tracks, repeated ids and differing counts
    assert np.any(np.all(out.tracks == 0, axis=(1, 2)))
    assert len(np.unique(z["ids"])) < 6


def test_host_dedup_matches_oracle(oracle):
    z, out = fixture()
    assert same_set(dedup_dye_tracks(z["tracks"], z["ids"], z["cnts"]), out)
    for tr, ids, cnt in random_cases():
        assert same_set(dedup_dye_tracks(tr, ids, cnt), oracle.dedup_dye_tracks(tr, ids, cnt))


def test_oracle_matches_live_reference(oracle, reference):
    for tr, ids, cnt in random_cases(seed=4)[1:]:
        assert same_set(oracle.dedup_dye_tracks(tr, ids, cnt), reference.dedup_dye_tracks(tr, ids, cnt))


def test_track_set_sources_keyed_on_id():
    """Dye-seqs sharing an id merge into one source per track, with the
    count of the first dye-seq of that id (hits add up)."""
    sm = paper_model(2)
    seqs = [parse_dye_seq(s) for s in ["0.1", "0.1", "1..0"]]
    ds = DyeSeqSet(2, seqs, np.array([4, 4, 2], np.int32), np.array([1, 3, 2], np.int32))
    dts = simulate_dye_track_set(sm, ds, 5, 200, seed=9)
    assert set(np.unique(dts.src_id)) <= {2, 4}
    for u in range(len(dts)):
        a, b = dts.src_off[u], dts.src_off[u + 1]
        assert np.all(np.diff(dts.src_id[a:b]) > 0)
    # the count is that of the track's first instance of the id: dye-seq 0
    # (count 1) wherever it produced the track, as on the commonest one
    c4, h4 = dts.src_count[dts.src_id == 4], dts.src_hits[dts.src_id == 4]
    assert set(np.unique(c4)) <= {1, 3} and c4[np.argmax(h4)] == 1
    # every instance of an id is a hit: 200 x (1 + 3) copies of id 4, less
    # the undetectable ones
    assert 0.9 * 800 < dts.src_hits[dts.src_id == 4].sum() <= 800


def test_oracle_generator_matches_reference_statistics(oracle):
    """The oracle's generate_dye_tracks restatement (seeded, feeding its
    dedup) against the statistics of the reference's own generator: mean
    dye counts per (t, c) over all instances and the undetectable share."""
    z = np.load(os.path.join(GOLDEN, "sim_tracks_c3_t12.npz"))
    sm = paper_model(3)
    sm.p_initial_block, sm.p_cyclic_block, sm.p_initial_detach, sm.p_initial_detach_decay = z["model"]
    T, n = int(z["T"]), 200000
    for i, s in enumerate(z["seqs"]):
        ds = DyeSeqSet(3, [parse_dye_seq(str(s))], np.array([3], np.int32), np.array([1], np.int32))
        dts, kept = oracle.simulate_dt(sm, T, ds, n, seed=700 + i)
        assert int(dts.src_hits.sum()) == kept and np.all(dts.src_id == 3)
        w = dts.src_hits.astype(np.float64)[:, None, None]
        mean = (w * dts.tracks).sum(axis=0) / n
        meansq = (w * dts.tracks.astype(np.float64) ** 2).sum(axis=0) / n
        var_o = meansq - mean ** 2
        var_r = z["meansq"][i] - z["mean"][i] ** 2
        se = np.sqrt(var_o / n + var_r / int(z["n"])) + 1e-12
        assert np.all(np.abs(mean - z["mean"][i]) <= 5 * se), np.max(np.abs(mean - z["mean"][i]) / se)
        p = z["trivial"][i]
        assert abs((n - kept) / n - p) <= 5 * np.sqrt(max(p, 1e-5) * (1 - p) / n) + 1e-5


def test_host_dedup_properties():
    """The host dedup on a larger random set: distinct tracks strictly
    increasing (lexicographic), sources ascending within a track, hits
    adding up to the instances, counts those of each id's first instance."""
    rng = np.random.default_rng(8)
    n, T, C = 20000, 8, 3
    tr = np.minimum(rng.geometric(0.5, (n, T, C)) - 1, 4).astype(np.int16)
    ids = rng.integers(-50, 50, n).astype(np.int32)
    cnt = rng.integers(1, 6, n).astype(np.int32)
    d = dedup_dye_tracks(tr, ids, cnt)
    flat = d.tracks.reshape(len(d), -1).astype(np.int64)
    diff = flat[1:] - flat[:-1]
    first = np.argmax(diff != 0, axis=1)
    assert np.all(diff[np.arange(len(diff)), first] > 0)
    for u in range(0, len(d), 97):
        a, b = d.src_off[u], d.src_off[u + 1]
        assert np.all(np.diff(d.src_id[a:b]) > 0)
        rows = np.flatnonzero(np.all(tr.reshape(n, -1) == flat[u], axis=1))
        for sid, sc, sh in zip(d.src_id[a:b], d.src_count[a:b], d.src_hits[a:b]):
            inst = rows[ids[rows] == sid]
            assert sh == len(inst) and sc == cnt[inst[0]]
    assert int(d.src_hits.sum()) == n


def test_dye_track_buffers_views():
    """Reusable download buffers (host side): views of the asked sizes,
    refusal of a set larger than the buffers or of another shape."""
    from whatprot_gb300 import capi
    b = capi.DyeTrackBuffers(10, 20, 4, 3, pinned=False)
    counts, off, sid, scnt, shit = b.views(7, 12, 4, 3)
    assert counts.shape == (7, 4, 3) and off.shape == (8,)
    with pytest.raises(ValueError):
        b.views(11, 5, 4, 3)
    with pytest.raises(ValueError):
        b.views(5, 21, 4, 3)
    with pytest.raises(ValueError):
        b.views(5, 5, 3, 3)
