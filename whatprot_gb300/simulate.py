"""Seeded synthetic data: dye-seq sets and simulated reads.

The reference's simulator is seeded from ``clock()`` (cc_code/src/util/
time.cc:28-30) and so cannot reproduce a data set.  This module restates its
generative model with a seeded numpy Generator so that every benchmark and
test input can be regenerated from a seed:

* ``simulate_dye_tracks`` follows cc_code/src/simulation/
  generate-dye-track.cc:29-110 (duds, initial/cyclic block, per-timestep
  detach, Edman failure, bleaching of the remaining dyes; counts recorded at
  the start of each timestep).
* ``simulate_radiometries`` follows generate-radiometry.cc:28-62 (reads whose
  t=0 counts are all zero are dropped; intensities ~ Normal(adjusted_mu,
  sigma(adjusted_mu))) and generate-radiometries.cc:30-64 (peptide drawn with
  probability proportional to its count).

The draws are vectorised over reads; the random stream differs from the
reference's (which is unseedable anyway), the distribution is the same.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from .model import DyeSeqSet, SequencingModel


def random_dye_seqs(num: int, num_channels: int, min_len: int, max_len: int,
                    p_label: float = 0.1, max_per_channel: Optional[int] = None,
                    min_total: int = 0, seed: int = 0) -> DyeSeqSet:
    """Dye-seqs of length U{min_len..max_len}; each position carries channel
    c with probability p_label (independently exclusive), else unlabeled.
    Optional rejection to <= max_per_channel dyes per channel and >=
    min_total dyes overall.  ids are 0..num-1, counts 1."""
    rng = np.random.default_rng(seed)
    seqs = []
    while len(seqs) < num:
        L = int(rng.integers(min_len, max_len + 1))
        u = rng.random(L)
        s = np.full(L, -1, dtype=np.int16)
        for c in range(num_channels):
            s[(u >= c * p_label) & (u < (c + 1) * p_label)] = c
        per = [int(np.sum(s == c)) for c in range(num_channels)]
        if max_per_channel is not None and max(per) > max_per_channel:
            continue
        if sum(per) < min_total:
            continue
        # The dye-seq file format trims trailing '.' (dye-seq.cc:25-28).
        n = L
        while n > 0 and s[n - 1] == -1:
            n -= 1
        seqs.append(s[:n].copy())
    return DyeSeqSet(num_channels, seqs, np.arange(num, dtype=np.int32),
                     np.ones(num, dtype=np.int32))


def _adjusted_mu_vec(cm, channel: int, counts: np.ndarray) -> np.ndarray:
    """Vectorised channel-model.h:35-54 over counts[..., C]."""
    amu = cm.mu * counts[..., channel].astype(np.float64)
    C = counts.shape[-1]
    for c in range(C):
        n = counts[..., c].astype(np.float64)
        if c == channel:
            f = np.where(n > 1, cm.flat_interactions[c] * np.power(cm.interactions[c], np.maximum(n - 1, 0)), 1.0)
        else:
            f = np.where(n > 0, cm.flat_interactions[c] * np.power(cm.interactions[c], n), 1.0)
        amu = amu * f
    return amu


def simulate_dye_tracks(model: SequencingModel, seqs: np.ndarray, lengths: np.ndarray,
                        num_timesteps: int, rng: np.random.Generator) -> np.ndarray:
    """Dye tracks [R, T, C] for R peptide instances.  seqs is [R, Lmax] int16
    (-1 padded), lengths [R].  generate-dye-track.cc:29-110."""
    R, Lmax = seqs.shape
    C = model.num_channels
    T = num_timesteps
    ds = seqs.copy()
    p_dud = np.array([cm.p_dud for cm in model.channel_models])
    p_bleach = np.array([cm.p_bleach for cm in model.channel_models])
    pos = np.arange(Lmax)[None, :]
    valid = pos < lengths[:, None]
    lab = (ds >= 0) & valid
    # Duds.
    u = rng.random((R, Lmax))
    dud = lab & (u < p_dud[np.clip(ds, 0, C - 1)])
    ds[dud] = -1
    counts = np.stack([np.sum((ds == c) & valid, axis=1) for c in range(C)], axis=1).astype(np.int16)
    e = np.zeros(R, dtype=np.int64)
    block = rng.random(R) < model.p_initial_block
    out = np.zeros((R, T, C), dtype=np.int16)
    rows = np.arange(R)
    for t in range(T):
        alive = e < lengths
        out[:, t, :] = np.where(alive[:, None], counts, 0)
        block |= alive & (rng.random(R) < model.p_cyclic_block)
        det = alive & (rng.random(R) < model.p_detach_at(t))
        e[det] = lengths[det]
        alive &= ~det
        edman_ok = alive & ~block & ~(rng.random(R) < model.p_edman_failure)
        idx = np.minimum(e, Lmax - 1)
        d_at = ds[rows, idx]
        rem = edman_ok & (d_at >= 0)
        if np.any(rem):
            np.subtract.at(counts, (rows[rem], d_at[rem].astype(np.int64)), 1)
        e[edman_ok] += 1
        # Bleaching of the remaining dyes (positions >= e).
        remaining = (pos >= e[:, None]) & valid & (ds >= 0) & alive[:, None]
        ub = rng.random((R, Lmax))
        bl = remaining & (ub < p_bleach[np.clip(ds, 0, C - 1)])
        if np.any(bl):
            for c in range(C):
                counts[:, c] -= np.sum(bl & (ds == c), axis=1).astype(np.int16)
            ds[bl] = -1
    return out


def simulate_radiometries(model: SequencingModel, dye_seqs: DyeSeqSet, num_timesteps: int,
                          num_to_generate: int, seed: int = 0
                          ) -> Tuple[np.ndarray, np.ndarray]:
    """Simulated reads (rads [R_kept, T, C] float64, true ids [R_kept]).

    ``model`` is the mu-as-one model the classifier uses (so intensities are
    already in units of mu, as read_radiometries produces)."""
    rng = np.random.default_rng(seed)
    C = model.num_channels
    P = len(dye_seqs)
    w = dye_seqs.counts.astype(np.float64)
    pick = rng.choice(P, size=num_to_generate, p=w / w.sum())
    lengths = np.array([len(dye_seqs.seqs[i]) for i in pick], dtype=np.int64)
    Lmax = max(1, int(lengths.max()) if len(lengths) else 1)
    seqs = np.full((num_to_generate, Lmax), -1, dtype=np.int16)
    for r, i in enumerate(pick):
        s = dye_seqs.seqs[i]
        seqs[r, : len(s)] = s
    tracks = simulate_dye_tracks(model, seqs, lengths, num_timesteps, rng)
    keep = np.any(tracks[:, 0, :] != 0, axis=1)
    tracks = tracks[keep]
    ids = dye_seqs.ids[pick[keep]]
    rads = np.zeros(tracks.shape, dtype=np.float64)
    for c, cm in enumerate(model.channel_models):
        mu = _adjusted_mu_vec(cm, c, tracks)
        sig = np.sqrt(cm.bg_sig * cm.bg_sig + mu * cm.sig * cm.sig)
        rads[..., c] = rng.normal(mu, sig)
    return rads, ids.astype(np.int32)


def simulate_dye_track_set(model: SequencingModel, dye_seqs: DyeSeqSet, num_timesteps: int,
                           per_peptide: int, seed: int = 0):
    """The kNN training set: per_peptide dye-tracks for every peptide (times
    its count), all-zero tracks dropped (generate-dye-tracks.cc:29-70), then
    deduplicated into unique tracks with (id, count, hits) sources
    (dedup_dye_tracks below)."""
    rng = np.random.default_rng(seed)
    C = model.num_channels
    reps = np.repeat(np.arange(len(dye_seqs)), dye_seqs.counts.astype(np.int64) * per_peptide)
    lengths = np.array([len(dye_seqs.seqs[i]) for i in reps], dtype=np.int64)
    Lmax = max(1, int(lengths.max()) if len(lengths) else 1)
    seqs = np.full((len(reps), Lmax), -1, dtype=np.int16)
    for r, i in enumerate(reps):
        s = dye_seqs.seqs[i]
        seqs[r, : len(s)] = s
    tracks = simulate_dye_tracks(model, seqs, lengths, num_timesteps, rng)
    keep = np.any(tracks[:, 0, :] != 0, axis=1)
    tracks = tracks[keep]
    pep = reps[keep]
    return dedup_dye_tracks(tracks, dye_seqs.ids[pep], dye_seqs.counts[pep])


def dedup_dye_tracks(tracks: np.ndarray, ids: np.ndarray, counts: np.ndarray):
    """dedup_dye_tracks (dedup-dye-tracks.cc:35-141) on the host: dye-tracks
    [n, T, C] from sources (ids[i], counts[i]) -> the distinct tracks, each
    with one (id, count, hits) per distinct source id (count of the id's
    first instance, hits its number of instances).  Tracks come out in
    lexicographic order of their counts, sources in ascending id."""
    from .io import DyeTrackSet
    n, T, C = tracks.shape
    if n == 0:
        return DyeTrackSet(np.zeros((0, T, C), np.int16), np.zeros(1, np.int32), np.zeros(0, np.int32),
                           np.zeros(0, np.int32), np.zeros(0, np.int32))
    flat = np.ascontiguousarray(tracks.reshape(n, -1))
    # rows as opaque byte strings: np.unique on them is much faster than
    # axis=0; big-endian int16 bytes sort in the same order as the counts
    # (all counts are non-negative)
    be = flat.astype(">i2")
    rows = be.view(np.dtype((np.void, be.dtype.itemsize * be.shape[1]))).reshape(-1)
    _, first, inv = np.unique(rows, return_index=True, return_inverse=True)
    uniq = flat[first]
    inv = inv.reshape(-1)
    ids = np.asarray(ids, np.int64)
    # instances by (track, id, instance): runs of one id within a track
    order = np.lexsort((np.arange(n), ids, inv))
    inv_s, id_s = inv[order], ids[order]
    new = np.ones(n, bool)
    new[1:] = (inv_s[1:] != inv_s[:-1]) | (id_s[1:] != id_s[:-1])
    starts = np.flatnonzero(new)
    hits = np.diff(np.append(starts, n))
    src_off = np.zeros(len(uniq) + 1, np.int64)
    np.add.at(src_off, inv_s[starts] + 1, 1)
    return DyeTrackSet(uniq.reshape(len(uniq), T, C).astype(np.int16), np.cumsum(src_off).astype(np.int32),
                       id_s[starts].astype(np.int32), np.asarray(counts)[order][starts].astype(np.int32),
                       hits.astype(np.int32))


def paper_model(num_channels: int) -> SequencingModel:
    """The error model of the benchmark configurations: p_edman_failure 0.06,
    p_detach 0.05, no initial detach or blocking; per channel p_bleach 0.05,
    p_dud 0.07, bg_sig 0.00667, mu 1, sig 0.16, no interactions."""
    from .model import ChannelModel
    sm = SequencingModel(0.06, 0.05, 0.0, 0.0, 0.0, 0.0, [])
    for _ in range(num_channels):
        sm.channel_models.append(ChannelModel(0.05, 0.07, 0.00667, 1.0, 0.16,
                                              [1.0] * num_channels, [1.0] * num_channels))
    return sm
