"""Readers and writers for whatprot's file formats.

Formats follow the reference's cc_code/src/io/:
* dye-seqs TSV: num_channels, num_dye_seqs, then ``string count id`` per line
  (dye-seqs-io.cc:63-89).
* radiometries TSV: T, C, N header lines then one read per line, t-major then
  c, tab separated; values are divided by the channel's true mu on read
  (radiometries-io.cc:33-56) and multiplied back on write (:58-82, %.17g).
* true ids: N then one id per line (radiometries-io.cc:104-114).
* dye-tracks TSV: T, C, N then per track T*C counts, num_sources and
  (id, count, hits) triples (dye-tracks-io.cc:32-104).
* predictions CSV: header ``radmat_iz,best_pep_iz,best_pep_score`` and
  ``i,id,score`` with 17 significant digits (scored-classifications-io.cc:54-68).
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from .model import DyeSeqSet, SequencingModel, dye_seq_string, parse_dye_seq


def _tokens(path):
    with open(path) as f:
        return f.read().split()


def read_dye_seqs(path) -> DyeSeqSet:
    tok = _tokens(path)
    C = int(tok[0])
    n = int(tok[1])
    seqs, ids, counts = [], [], []
    k = 2
    for _ in range(n):
        seqs.append(parse_dye_seq(tok[k]))
        counts.append(int(tok[k + 1]))
        ids.append(int(tok[k + 2]))
        k += 3
    return DyeSeqSet(C, seqs, np.asarray(ids, dtype=np.int32), np.asarray(counts, dtype=np.int32))


def write_dye_seqs(path, ds: DyeSeqSet) -> None:
    """dye-seqs-io.cc:63-89.  A dye-seq without any dye is written as "."
    (the reader trims trailing '.'): an empty field would be skipped by a
    whitespace-token reader, here and in the reference."""
    with open(path, "w") as f:
        f.write(f"{ds.num_channels}\n{len(ds)}\n")
        for s, cnt, i in zip(ds.seqs, ds.counts, ds.ids):
            f.write(f"{dye_seq_string(s) or '.'}\t{int(cnt)}\t{int(i)}\n")


def read_radiometries(path, true_model: SequencingModel) -> Tuple[int, int, np.ndarray]:
    """Returns (T, C, rads[N, T, C] float64) divided by each channel's mu."""
    with open(path) as f:
        T = int(f.readline())
        C = int(f.readline())
        N = int(f.readline())
        data = np.fromstring(f.read(), sep=" ", dtype=np.float64) if N else np.zeros(0)
    rads = data[: N * T * C].reshape(N, T, C) if N else np.zeros((0, T, C))
    mu = np.array([cm.mu for cm in true_model.channel_models], dtype=np.float64)
    return T, C, rads / mu[None, None, :]


def write_radiometries(path, true_model: SequencingModel, rads: np.ndarray) -> None:
    N, T, C = rads.shape
    mu = np.array([cm.mu for cm in true_model.channel_models], dtype=np.float64)
    vals = rads * mu[None, None, :]
    with open(path, "w") as f:
        f.write(f"{T}\n{C}\n{N}\n")
        for r in range(N):
            f.write("\t".join(f"{v:.17g}" for v in vals[r].reshape(-1)))
            f.write("\n")


def read_true_ids(path) -> np.ndarray:
    tok = _tokens(path)
    n = int(tok[0])
    return np.asarray([int(x) for x in tok[1:1 + n]], dtype=np.int32)


def write_true_ids(path, ids) -> None:
    with open(path, "w") as f:
        f.write(f"{len(ids)}\n")
        for i in ids:
            f.write(f"{int(i)}\n")


def write_predictions(path, ids, scores) -> None:
    with open(path, "w") as f:
        f.write("radmat_iz,best_pep_iz,best_pep_score\n")
        for i, (pid, sc) in enumerate(zip(ids, scores)):
            f.write(f"{i},{int(pid)},{float(sc):.17g}\n")


def read_predictions(path):
    ids, scores = [], []
    with open(path) as f:
        f.readline()
        for line in f:
            if not line.strip():
                continue
            _, pid, sc = line.strip().split(",")
            ids.append(int(pid))
            scores.append(float(sc))
    return np.asarray(ids, dtype=np.int32), np.asarray(scores, dtype=np.float64)


class DyeTrackSet:
    """Unique dye-tracks [N, T, C] with ragged (id, count, hits) sources
    (the reference's SourcedData<DyeTrack, SourceCountHitsList<int>>)."""

    def __init__(self, tracks: np.ndarray, src_off: np.ndarray, src_id: np.ndarray,
                 src_count: np.ndarray, src_hits: np.ndarray):
        self.tracks = tracks
        self.src_off = src_off
        self.src_id = src_id
        self.src_count = src_count
        self.src_hits = src_hits

    def __len__(self):
        return self.tracks.shape[0]


def read_dye_tracks(path) -> DyeTrackSet:
    tok = _tokens(path)
    T, C, N = int(tok[0]), int(tok[1]), int(tok[2])
    k = 3
    tracks = np.zeros((N, T, C), dtype=np.int16)
    off = [0]
    sid, scnt, shit = [], [], []
    for i in range(N):
        tracks[i] = np.asarray(tok[k:k + T * C], dtype=np.int16).reshape(T, C)
        k += T * C
        ns = int(tok[k])
        k += 1
        for _ in range(ns):
            sid.append(int(tok[k]))
            scnt.append(int(tok[k + 1]))
            shit.append(int(tok[k + 2]))
            k += 3
        off.append(off[-1] + ns)
    return DyeTrackSet(tracks, np.asarray(off, np.int32), np.asarray(sid, np.int32),
                       np.asarray(scnt, np.int32), np.asarray(shit, np.int32))


def write_dye_tracks(path, dts: DyeTrackSet) -> None:
    N, T, C = dts.tracks.shape
    with open(path, "w") as f:
        f.write(f"{T}\n{C}\n{N}\n")
        for i in range(N):
            parts = [str(int(v)) for v in dts.tracks[i].reshape(-1)]
            a, b = dts.src_off[i], dts.src_off[i + 1]
            f.write("\t".join(parts) + "\t" + str(b - a) + "\t")
            trip = []
            for j in range(a, b):
                trip.append(f"{dts.src_id[j]}\t{dts.src_count[j]}\t{dts.src_hits[j]}")
            f.write("\t".join(trip) + "\n")


def write_params(path, num_channels: int, models, log_ls) -> None:
    """params-io.cc:32-56: the bootstrap rounds' parameters and log(L), CSV,
    17 significant digits."""
    cols = ["p_edman_failure", "p_detach", "p_initial_detach", "p_initial_detach_decay", "p_initial_block",
            "p_cyclic_block"]
    for c in range(num_channels):
        cols += [f"ch{c}:p_bleach", f"ch{c}:p_dud"]
    with open(path, "w") as f:
        f.write(",".join(cols) + ",log(L)\n")
        for m, ll in zip(models, log_ls):
            vals = [m.p_edman_failure, m.p_detach, m.p_initial_detach, m.p_initial_detach_decay,
                    m.p_initial_block, m.p_cyclic_block]
            for c in range(num_channels):
                vals += [m.channel_models[c].p_bleach, m.channel_models[c].p_dud]
            f.write(",".join(f"{v:.17g}" for v in vals) + f",{ll:.17g}\n")
