"""ctypes bindings to the checkers: oracle/liboracle.so (the C restatement)
and, when it was built in this container, oracle/_ref/libwpref.so (the
reference's own sources).  Test infrastructure only."""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from typing import Optional

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libwpref.so")
DBL_MAX = sys.float_info.max

MAXC = 8
MAXT = 64


class WpoModel(ctypes.Structure):
    _fields_ = [("num_channels", ctypes.c_int),
                ("p_edman_failure", ctypes.c_double),
                ("p_detach", ctypes.c_double),
                ("p_initial_detach", ctypes.c_double),
                ("p_initial_detach_decay", ctypes.c_double),
                ("p_initial_block", ctypes.c_double),
                ("p_cyclic_block", ctypes.c_double),
                ("p_bleach", ctypes.c_double * MAXC),
                ("p_dud", ctypes.c_double * MAXC),
                ("bg_sig", ctypes.c_double * MAXC),
                ("mu", ctypes.c_double * MAXC),
                ("sig", ctypes.c_double * MAXC),
                ("interactions", (ctypes.c_double * MAXC) * MAXC),
                ("flat_interactions", (ctypes.c_double * MAXC) * MAXC)]


class WpoFitSums(ctypes.Structure):
    _fields_ = [("edman_num", ctypes.c_double), ("edman_den", ctypes.c_double),
                ("detach_x", ctypes.c_double * MAXT), ("detach_n", ctypes.c_double * MAXT),
                ("init_block_num", ctypes.c_double), ("init_block_den", ctypes.c_double),
                ("cyc_block_num", ctypes.c_double), ("cyc_block_den", ctypes.c_double),
                ("bleach_num", ctypes.c_double * MAXC), ("bleach_den", ctypes.c_double * MAXC),
                ("dud_num", ctypes.c_double * MAXC), ("dud_den", ctypes.c_double * MAXC),
                ("emis_w", (ctypes.c_double * 16) * MAXC), ("emis_x", (ctypes.c_double * 16) * MAXC),
                ("emis_xx", (ctypes.c_double * 16) * MAXC)]

    def as_dict(self, T, C):
        return {
            "edman": (self.edman_num, self.edman_den),
            "detach_x": np.array(self.detach_x[: T - 1]),
            "detach_n": np.array(self.detach_n[: T - 1]),
            "init_block": (self.init_block_num, self.init_block_den),
            "cyc_block": (self.cyc_block_num, self.cyc_block_den),
            "bleach": (np.array(self.bleach_num[:C]), np.array(self.bleach_den[:C])),
            "dud": (np.array(self.dud_num[:C]), np.array(self.dud_den[:C])),
            "emis_w": np.array([list(self.emis_w[c]) for c in range(C)]),
            "emis_x": np.array([list(self.emis_x[c]) for c in range(C)]),
            "emis_xx": np.array([list(self.emis_xx[c]) for c in range(C)]),
        }


def to_wpo(sm) -> WpoModel:
    m = WpoModel()
    C = sm.num_channels
    m.num_channels = C
    m.p_edman_failure = sm.p_edman_failure
    m.p_detach = sm.p_detach
    m.p_initial_detach = sm.p_initial_detach
    m.p_initial_detach_decay = sm.p_initial_detach_decay
    m.p_initial_block = sm.p_initial_block
    m.p_cyclic_block = sm.p_cyclic_block
    for c, cm in enumerate(sm.channel_models):
        m.p_bleach[c] = cm.p_bleach
        m.p_dud[c] = cm.p_dud
        m.bg_sig[c] = cm.bg_sig
        m.mu[c] = cm.mu
        m.sig[c] = cm.sig
        for o in range(MAXC):
            m.interactions[c][o] = cm.interactions[o] if o < C else 1.0
            m.flat_interactions[c][o] = cm.flat_interactions[o] if o < C else 1.0
    return m


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def canonical_dye_tracks(counts, src_off, src_id, src_count, src_hits):
    """A dye-track set with tracks in lexicographic order of their counts and
    each track's sources in ascending id (the reference's own order is that
    of its hash tables)."""
    from whatprot_gb300.io import DyeTrackSet
    N = counts.shape[0]
    order = np.lexsort(counts.reshape(N, -1).T[::-1]) if N else np.zeros(0, np.int64)
    off, ids, cnt, hits = [0], [], [], []
    for u in order:
        a, b = int(src_off[u]), int(src_off[u + 1])
        srt = np.argsort(src_id[a:b], kind="stable")
        ids.extend(src_id[a:b][srt])
        cnt.extend(src_count[a:b][srt])
        hits.extend(src_hits[a:b][srt])
        off.append(len(ids))
    return DyeTrackSet(counts[order].astype(np.int16), np.array(off, np.int32), np.array(ids, np.int32),
                       np.array(cnt, np.int32), np.array(hits, np.int32))


def _dedup_call(fn, counts, ids, cnts, canonical):
    counts = np.ascontiguousarray(counts, dtype=np.int16)
    n, T, C = counts.shape
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    cnts = np.ascontiguousarray(cnts, dtype=np.int32)
    m = max(n, 1)
    oc = np.zeros((m, T, C), np.int16)
    off = np.zeros(m + 1, np.int32)
    sid, scnt, shits = (np.zeros(m, np.int32) for _ in range(3))
    if canonical:
        ns = ctypes.c_int32(0)
        u = fn(T, C, n, _p(counts), _p(ids), _p(cnts), _p(oc), _p(off), _p(sid), _p(scnt), _p(shits),
               ctypes.byref(ns))
        ns = ns.value
    else:
        nu, nsv = ctypes.c_int(0), ctypes.c_int(0)
        fn(T, C, n, _p(counts), _p(ids), _p(cnts), ctypes.byref(nu), ctypes.byref(nsv), _p(oc), _p(off),
           _p(sid), _p(scnt), _p(shits))
        u, ns = nu.value, nsv.value
    return canonical_dye_tracks(oc[:u], off[:u + 1], sid[:ns], scnt[:ns], shits[:ns])


SELECTIONS = {"kdtree": 0, "prefix": 1}


class Oracle:
    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        self.lib = ctypes.CDLL(ORACLE_SO)
        L = self.lib
        L.wpo_peptide_probability.restype = ctypes.c_double
        L.wpo_peptide_probability.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_int, ctypes.c_void_p, ctypes.c_uint, ctypes.c_double,
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.wpo_pruned_emission_boxes.restype = ctypes.c_int
        L.wpo_pruned_emission_boxes.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_int, ctypes.c_void_p, ctypes.c_uint,
                                                ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.wpo_emission_range.restype = None
        L.wpo_emission_range.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_uint, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.wpo_classify_batch.restype = None
        L.wpo_classify_batch.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]
        L.wpo_loglik_all.restype = None
        L.wpo_loglik_all.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
        L.wpo_nn_classify_batch.restype = None
        L.wpo_nn_classify_batch.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int] + [ctypes.c_void_p, ctypes.c_int] \
            + [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int] + [ctypes.c_void_p] * 4
        L.wpo_hybrid_classify_batch.restype = None
        L.wpo_hybrid_classify_batch.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p, ctypes.c_int] \
            + [ctypes.c_void_p] * 8 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int] \
            + [ctypes.c_void_p] * 3
        L.wpo_simulate_dt.restype = ctypes.c_int
        L.wpo_simulate_dt.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int] + [ctypes.c_void_p] * 4 \
            + [ctypes.c_int, ctypes.c_int, ctypes.c_uint64] + [ctypes.c_void_p] * 7
        L.wpo_dedup_dye_tracks.restype = ctypes.c_int
        L.wpo_dedup_dye_tracks.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 9
        L.wpo_improve_fit_batch.restype = None
        L.wpo_improve_fit_batch.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_int, ctypes.POINTER(WpoFitSums), ctypes.c_void_p]
        L.wpo_improve_fit.restype = ctypes.c_double
        L.wpo_improve_fit.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_uint, ctypes.c_double,
                                      ctypes.POINTER(WpoFitSums), ctypes.POINTER(ctypes.c_double)]

    def probability(self, sm, T, seq, rad, max_num_dyes, cutoff=DBL_MAX):
        m = to_wpo(sm)
        seq = np.ascontiguousarray(seq, dtype=np.int16)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        lp = ctypes.c_double()
        fl = ctypes.c_double()
        p = self.lib.wpo_peptide_probability(ctypes.byref(m), T, _p(seq) if len(seq) else None, len(seq),
                                             _p(rad), max_num_dyes, cutoff, ctypes.byref(lp), ctypes.byref(fl))
        return p, lp.value, fl.value

    def pruned_boxes(self, sm, T, seq, rad, max_num_dyes, cutoff):
        m = to_wpo(sm)
        C = sm.num_channels
        seq = np.ascontiguousarray(seq, dtype=np.int16)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        lo = np.zeros((T, C), np.uint32)
        hi = np.zeros((T, C), np.uint32)
        empty = self.lib.wpo_pruned_emission_boxes(ctypes.byref(m), T, _p(seq) if len(seq) else None,
                                                   len(seq), _p(rad), max_num_dyes, cutoff, _p(lo), _p(hi))
        return bool(empty), lo, hi

    def emission_range(self, sm, rad, t, max_num_dyes, cutoff):
        m = to_wpo(sm)
        C = sm.num_channels
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        lo = np.zeros(C, np.uint32)
        hi = np.zeros(C, np.uint32)
        self.lib.wpo_emission_range(ctypes.byref(m), _p(rad), t, max_num_dyes, cutoff, _p(lo), _p(hi))
        return lo, hi

    def classify(self, sm, T, dye_seqs, rads, cutoff=DBL_MAX, threads=8, cand=None, cand_off=None):
        m = to_wpo(sm)
        flat, off = dye_seqs.ragged()
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        oid = np.zeros(R, np.int32)
        osc = np.zeros(R, np.float64)
        otot = np.zeros(R, np.float64)
        ids = np.ascontiguousarray(dye_seqs.ids, np.int32)
        cnt = np.ascontiguousarray(dye_seqs.counts, np.int32)
        if cand is not None:
            cand = np.ascontiguousarray(cand, np.int32)
            cand_off = np.ascontiguousarray(cand_off, np.int32)
        self.lib.wpo_classify_batch(ctypes.byref(m), T, _p(flat), _p(off), _p(ids), _p(cnt), len(dye_seqs),
                                    _p(rads), R, _p(cand), _p(cand_off), cutoff, threads,
                                    _p(oid), _p(osc), _p(otot))
        return oid, osc, otot

    def loglik_all(self, sm, T, dye_seqs, rads, cutoff=DBL_MAX, threads=8):
        m = to_wpo(sm)
        flat, off = dye_seqs.ragged()
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        out = np.zeros((R, len(dye_seqs)), np.float64)
        self.lib.wpo_loglik_all(ctypes.byref(m), T, _p(flat), _p(off), len(dye_seqs), _p(rads), R,
                                cutoff, threads, _p(out))
        return out

    def nn_classify(self, sm, T, dts, rads, k, sig, h, threads=8, selection="kdtree"):
        """kNN top-h per read: (ncand [R], ids [R,h], scores [R,h], total [R]).
        selection: "kdtree" (the reference's kd-tree search and KBest) or
        "prefix" (the shortest distance-ordered prefix reaching k hits)."""
        m = to_wpo(sm)
        R = rads.shape[0]
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        tr = np.ascontiguousarray(dts.tracks, dtype=np.int16)
        nc = np.zeros(R, np.int32)
        ids = np.zeros((R, h), np.int32)
        sc = np.zeros((R, h), np.float64)
        tot = np.zeros(R, np.float64)
        self.lib.wpo_nn_classify_batch(ctypes.byref(m), T, _p(tr), len(dts), _p(dts.src_off), _p(dts.src_id),
                                       _p(dts.src_count), _p(dts.src_hits), _p(rads), R, k, sig, h,
                                       SELECTIONS[selection], threads, _p(nc), _p(ids), _p(sc), _p(tot))
        return nc, ids, sc, tot

    def hybrid_classify(self, sm, T, dts, dye_seqs, rads, k, sig, h, cutoff, threads=8, selection="kdtree"):
        """Hybrid per read: (ids, scores, totals); selection as nn_classify."""
        m = to_wpo(sm)
        R = rads.shape[0]
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        tr = np.ascontiguousarray(dts.tracks, dtype=np.int16)
        flat, off = dye_seqs.ragged()
        pid = np.ascontiguousarray(dye_seqs.ids, dtype=np.int32)
        pc = np.ascontiguousarray(dye_seqs.counts, dtype=np.int32)
        oid = np.zeros(R, np.int32)
        osc = np.zeros(R, np.float64)
        otot = np.zeros(R, np.float64)
        self.lib.wpo_hybrid_classify_batch(ctypes.byref(m), T, _p(tr), len(dts), _p(dts.src_off),
                                           _p(dts.src_id), _p(dts.src_count), _p(dts.src_hits), _p(flat),
                                           _p(off), _p(pid), _p(pc), len(dye_seqs), _p(rads), R, k, sig, h,
                                           cutoff, SELECTIONS[selection], threads, _p(oid), _p(osc), _p(otot))
        return oid, osc, otot

    def dedup_dye_tracks(self, counts, ids, cnts):
        """Canonical dedup (tracks lexicographic, sources by id) of counts
        [n, T, C] with sources (ids, cnts); returns a DyeTrackSet."""
        return _dedup_call(self.lib.wpo_dedup_dye_tracks, counts, ids, cnts, canonical=True)

    def simulate_dt(self, sm, T, dye_seqs, per_peptide, seed):
        """generate_dye_tracks + dedup (single thread, seeded); returns the
        DyeTrackSet and the number of kept (detectable) instances."""
        from whatprot_gb300.io import DyeTrackSet
        flat, off = dye_seqs.ragged()
        ids = np.ascontiguousarray(dye_seqs.ids, dtype=np.int32)
        cnt = np.ascontiguousarray(dye_seqs.counts, dtype=np.int32)
        C = sm.num_channels
        n = max(int(per_peptide) * int(cnt.sum()), 1)
        oc = np.zeros((n, T, C), np.int16)
        soff = np.zeros(n + 1, np.int32)
        sid, scnt, shits = (np.zeros(n, np.int32) for _ in range(3))
        ns, kept = ctypes.c_int32(0), ctypes.c_int32(0)
        u = self.lib.wpo_simulate_dt(ctypes.byref(to_wpo(sm)), T, _p(flat), _p(off), _p(ids), _p(cnt),
                                     len(dye_seqs), per_peptide, seed, _p(oc), _p(soff), _p(sid), _p(scnt),
                                     _p(shits), ctypes.byref(ns), ctypes.byref(kept))
        ns = ns.value
        return DyeTrackSet(oc[:u], soff[:u + 1], sid[:ns], scnt[:ns], shits[:ns]), kept.value

    def improve_fit_batch(self, sm, T, seq, rads, threads=8, cutoff=DBL_MAX):
        """E-step over many reads on host threads: (WpoFitSums, log P [R])."""
        m = to_wpo(sm)
        seq = np.ascontiguousarray(seq, dtype=np.int16)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        sums = WpoFitSums()
        lp = np.zeros(rads.shape[0])
        self.lib.wpo_improve_fit_batch(ctypes.byref(m), T, _p(seq) if len(seq) else None, len(seq),
                                       _p(rads), rads.shape[0], cutoff, threads, ctypes.byref(sums),
                                       _p(lp))
        return sums, lp

    def improve_fit(self, sm, T, seq, rad, max_num_dyes, cutoff=DBL_MAX, sums=None):
        m = to_wpo(sm)
        seq = np.ascontiguousarray(seq, dtype=np.int16)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        if sums is None:
            sums = WpoFitSums()
        lp = ctypes.c_double()
        p = self.lib.wpo_improve_fit(ctypes.byref(m), T, _p(seq) if len(seq) else None, len(seq), _p(rad),
                                     max_num_dyes, cutoff, ctypes.byref(sums), ctypes.byref(lp))
        return p, lp.value, sums


class Reference:
    """The reference's own classes, compiled from its sources (oracle/_ref)."""

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def __init__(self):
        self.lib = ctypes.CDLL(REF_SO)
        L = self.lib
        L.ref_peptide_probability.restype = ctypes.c_double
        L.ref_peptide_probability.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_char_p,
                                              ctypes.c_void_p, ctypes.c_uint, ctypes.c_double]
        L.ref_classify.restype = None
        L.ref_classify.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.POINTER(ctypes.c_double)]
        L.ref_improve_fit.restype = ctypes.c_double
        L.ref_improve_fit.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_char_p,
                                      ctypes.c_void_p, ctypes.c_uint, ctypes.c_double,
                                      ctypes.POINTER(WpoFitSums)]
        L.ref_offset_exponential.restype = None
        L.ref_offset_exponential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_void_p]
        L.ref_improve_fit_batch.restype = ctypes.c_double
        L.ref_improve_fit_batch.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_char_p,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.ref_nn_classify.restype = None
        L.ref_nn_classify.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p, ctypes.c_int] \
            + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_int] + [ctypes.c_void_p] * 8
        L.ref_hybrid_classify.restype = None
        L.ref_hybrid_classify.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_void_p, ctypes.c_int] \
            + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int] \
            + [ctypes.c_void_p] * 4
        L.ref_generate_dye_tracks.restype = None
        L.ref_generate_dye_tracks.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                              ctypes.c_uint, ctypes.c_void_p]
        L.ref_simulate_dt.restype = ctypes.c_double
        L.ref_simulate_dt.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_uint] + [ctypes.POINTER(ctypes.c_int)] * 3
        L.ref_dedup_dye_tracks.restype = None
        L.ref_dedup_dye_tracks.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 10
        L.ref_fit.restype = ctypes.c_double
        L.ref_fit.argtypes = [ctypes.POINTER(WpoModel), ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                              ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.POINTER(WpoModel),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]

    def probability(self, sm, T, seq_str, rad, max_num_dyes, cutoff=DBL_MAX):
        m = to_wpo(sm)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        return self.lib.ref_peptide_probability(ctypes.byref(m), T, seq_str.encode(), _p(rad),
                                                max_num_dyes, cutoff)

    def classify(self, sm, T, dye_seqs, rads, cutoff=DBL_MAX, threads=8):
        m = to_wpo(sm)
        strs = [s.encode() for s in dye_seqs.strings()]
        arr = (ctypes.c_char_p * len(strs))(*strs)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        oid = np.zeros(R, np.int32)
        osc = np.zeros(R, np.float64)
        otot = np.zeros(R, np.float64)
        secs = ctypes.c_double()
        ids = np.ascontiguousarray(dye_seqs.ids, np.int32)
        cnt = np.ascontiguousarray(dye_seqs.counts, np.int32)
        self.lib.ref_classify(ctypes.byref(m), T, len(strs), arr, _p(ids), _p(cnt), R, _p(rads), cutoff,
                              threads, _p(oid), _p(osc), _p(otot), ctypes.byref(secs))
        return oid, osc, otot, secs.value

    def improve_fit(self, sm, T, seq_str, rad, max_num_dyes, cutoff=DBL_MAX):
        m = to_wpo(sm)
        rad = np.ascontiguousarray(rad, dtype=np.float64)
        sums = WpoFitSums()
        p = self.lib.ref_improve_fit(ctypes.byref(m), T, seq_str.encode(), _p(rad), max_num_dyes,
                                     cutoff, ctypes.byref(sums))
        return p, sums

    def nn_classify(self, sm, T, dts, rads, k, sig, h, threads=8):
        """NNClassifier: (ncand, ids [R,h], scores [R,h], total [R], best_id,
        best_score, best_total, seconds)."""
        m = to_wpo(sm)
        R = rads.shape[0]
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        tr = np.ascontiguousarray(dts.tracks, dtype=np.int16)
        nc = np.zeros(R, np.int32)
        ids = np.zeros((R, h), np.int32)
        sc = np.zeros((R, h), np.float64)
        tot = np.zeros(R, np.float64)
        bid = np.zeros(R, np.int32)
        bsc = np.zeros(R, np.float64)
        btot = np.zeros(R, np.float64)
        secs = np.zeros(1, np.float64)
        self.lib.ref_nn_classify(ctypes.byref(m), T, _p(tr), len(dts), _p(dts.src_off), _p(dts.src_id),
                                 _p(dts.src_count), _p(dts.src_hits), R, _p(rads), k, sig, h, threads,
                                 _p(nc), _p(ids), _p(sc), _p(tot), _p(bid), _p(bsc), _p(btot), _p(secs))
        return nc, ids, sc, tot, bid, bsc, btot, float(secs[0])

    def hybrid_classify(self, sm, T, dts, dye_seqs, rads, k, sig, h, cutoff, threads=8):
        """HybridClassifier: (ids, scores, totals, seconds)."""
        from whatprot_gb300.model import dye_seq_string
        m = to_wpo(sm)
        R = rads.shape[0]
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        tr = np.ascontiguousarray(dts.tracks, dtype=np.int16)
        strs = [dye_seq_string(s).encode() for s in dye_seqs.seqs]
        arr = (ctypes.c_char_p * len(strs))(*strs)
        pid = np.ascontiguousarray(dye_seqs.ids, dtype=np.int32)
        pc = np.ascontiguousarray(dye_seqs.counts, dtype=np.int32)
        oid = np.zeros(R, np.int32)
        osc = np.zeros(R, np.float64)
        otot = np.zeros(R, np.float64)
        secs = np.zeros(1, np.float64)
        self.lib.ref_hybrid_classify(ctypes.byref(m), T, _p(tr), len(dts), _p(dts.src_off), _p(dts.src_id),
                                     _p(dts.src_count), _p(dts.src_hits), len(strs), arr, _p(pid), _p(pc), R,
                                     _p(rads), k, sig, h, cutoff, threads, _p(oid), _p(osc), _p(otot),
                                     _p(secs))
        return oid, osc, otot, float(secs[0])

    def improve_fit_batch(self, sm, T, seq_str, rads, threads=8):
        """E-step over many reads (OpenMP over reads); returns the summed
        edman denominator as a checksum."""
        m = to_wpo(sm)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        return self.lib.ref_improve_fit_batch(ctypes.byref(m), T, seq_str.encode(), rads.shape[0],
                                              _p(rads), threads)

    def dedup_dye_tracks(self, counts, ids, cnts):
        """The reference's dedup_dye_tracks on counts [n, T, C] with sources
        (ids, cnts), canonicalised (tracks lexicographic, sources by id)."""
        return _dedup_call(self.lib.ref_dedup_dye_tracks, counts, ids, cnts, canonical=False)

    def simulate_dt(self, sm, T, dye_seqs, per_peptide, seed):
        """The reference's generate_dye_tracks + dedup_dye_tracks over a
        dye-seq set; returns (seconds, kept instances, tracks, sources)."""
        from whatprot_gb300.model import dye_seq_string
        strs = [dye_seq_string(s).encode() for s in dye_seqs.seqs]
        arr = (ctypes.c_char_p * len(strs))(*strs)
        ids = np.ascontiguousarray(dye_seqs.ids, dtype=np.int32)
        cnt = np.ascontiguousarray(dye_seqs.counts, dtype=np.int32)
        ni, nu, ns = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        secs = self.lib.ref_simulate_dt(ctypes.byref(to_wpo(sm)), T, len(strs), arr, _p(ids), _p(cnt),
                                        per_peptide, seed, ctypes.byref(ni), ctypes.byref(nu), ctypes.byref(ns))
        return secs, ni.value, nu.value, ns.value

    def generate_dye_tracks(self, sm, T, seq_str, n, seed):
        out = np.zeros((n, T, sm.num_channels), np.int16)
        self.lib.ref_generate_dye_tracks(ctypes.byref(to_wpo(sm)), T, seq_str.encode(), n, seed, _p(out))
        return out

    def offset_exponential(self, y, w, params, held=(0, 0, 0)):
        y = np.ascontiguousarray(y, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        p = np.ascontiguousarray(params, dtype=np.float64).copy()
        h = np.ascontiguousarray(held, dtype=np.int32)
        self.lib.ref_offset_exponential(_p(y), _p(w), len(y), _p(h), _p(p))
        return p

    def fit(self, sm, T, seq_str, rads, threshold, max_runtime=1e9):
        m = to_wpo(sm)
        out = WpoModel()
        step = ctypes.c_double()
        secs = ctypes.c_double()
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        ll = self.lib.ref_fit(ctypes.byref(m), T, seq_str.encode(), rads.shape[0], _p(rads), threshold,
                              max_runtime, ctypes.byref(out), ctypes.byref(step), ctypes.byref(secs))
        return out, ll, step.value, secs.value


def oracle_sums_to_wp(o):
    """The oracle's E-step sums (WpoFitSums) as the library's wp_fit_sums."""
    from whatprot_gb300.capi import WpFitSums
    s = WpFitSums()
    s.p_edman_failure_num, s.p_edman_failure_den = o.edman_num, o.edman_den
    for i in range(len(s.p_detach_x)):
        s.p_detach_x[i], s.p_detach_n[i] = o.detach_x[i], o.detach_n[i]
    s.p_initial_block_num, s.p_initial_block_den = o.init_block_num, o.init_block_den
    s.p_cyclic_block_num, s.p_cyclic_block_den = o.cyc_block_num, o.cyc_block_den
    for c in range(len(s.p_bleach_num)):
        s.p_bleach_num[c], s.p_bleach_den[c] = o.bleach_num[c], o.bleach_den[c]
        s.p_dud_num[c], s.p_dud_den[c] = o.dud_num[c], o.dud_den[c]
    return s


def params_of_model(sm):
    """A SequencingModel's rates as wp_fit_params."""
    from whatprot_gb300.capi import WpFitParams
    p = WpFitParams()
    for k in ("p_edman_failure", "p_detach", "p_initial_detach", "p_initial_detach_decay", "p_initial_block",
              "p_cyclic_block"):
        setattr(p, k, getattr(sm, k))
    for c, cm in enumerate(sm.channel_models):
        p.p_bleach[c], p.p_dud[c] = cm.p_bleach, cm.p_dud
        p.mu[c], p.sig[c], p.bg_sig[c] = cm.mu, cm.sig, cm.bg_sig
    return p


def model_of_params(p, like):
    """wp_fit_params back into a SequencingModel shaped like `like`."""
    import copy
    m = copy.deepcopy(like)
    for k in ("p_edman_failure", "p_detach", "p_initial_detach", "p_initial_detach_decay", "p_initial_block",
              "p_cyclic_block"):
        setattr(m, k, getattr(p, k))
    for c, cm in enumerate(m.channel_models):
        cm.p_bleach, cm.p_dud = p.p_bleach[c], p.p_dud[c]
    return m


def oracle_em(start, T, seq, rads, threshold, threads=8, max_iterations=1000):
    """HMMFitter::fit's EM loop (fitters/hmm-fitter.h:49-142) with the
    oracle's FP64 E-step (wpo_improve_fit_batch, unpruned as run-fit.cc:59)
    and the library's host M-step (wp_fit_mstep: dud hidden-count
    correction, p = num / den, the detach curve), so that a GPU fit compared
    with it differs only by its FP32 E-step.  Returns (fitted model, step
    size, iterations)."""
    from whatprot_gb300 import shards
    o = Oracle()
    cur = params_of_model(start)
    it = 0
    while True:
        s, _ = o.improve_fit_batch(model_of_params(cur, start), T, seq, rads, threads=threads)
        nxt, step = shards.mstep(oracle_sums_to_wp(s), start.num_channels, T, seq, rads.shape[0], cur)
        it += 1
        cur = nxt
        if step < threshold or it >= max_iterations:
            return model_of_params(cur, start), step, it
