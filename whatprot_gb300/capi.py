"""ctypes binding of the C ABI (include/whatprot_gb300.h).

Loading fails loudly when the CUDA library has not been built: there is no
CPU fallback.  Build it with ``python -c "import __graft_entry__ as g;
g.build()"`` or ``python whatprot_gb300/build.py``.
"""
from __future__ import annotations

import ctypes
import math
import os
import sys
from typing import Optional, Tuple

import numpy as np

from .model import DyeSeqSet, SequencingModel

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libwhatprot_gb300.so")
DBL_MAX = sys.float_info.max

WP_MAX_CHANNELS = 4
WP_MAX_TIMESTEPS = 64

STATUS = {0: "WP_OK", 1: "WP_ERR_INVALID", 2: "WP_ERR_OOM", 3: "WP_ERR_CUDA",
          4: "WP_ERR_TIMEOUT", 5: "WP_ERR_UNSUPPORTED", 6: "WP_ERR_STATE"}

EXPORTS = ["wp_ctx_create", "wp_ctx_destroy", "wp_last_error", "wp_model_upload",
           "wp_peptides_upload", "wp_hmm_classify", "wp_hmm_classify_device",
           "wp_hmm_loglik_all", "wp_hmm_count_flops", "wp_launch_count", "wp_ctx_stream",
           "wp_timing_enable", "wp_timing_read", "wp_probe_fp32_peak", "wp_last_batch_stats",
           "wp_fit_begin", "wp_fit_estep", "wp_hmm_fit", "wp_fit_offset_exponential", "wp_fit_set_kernel",
           "wp_hmm_bootstrap_fit", "wp_fit_mstep", "wp_fit_set_emission", "wp_fit_emission_sums",
           "wp_fit_emission_mstep",
           "wp_nn_tracks_upload", "wp_nn_classify", "wp_hybrid_classify", "wp_hybrid_classify_device",
           "wp_dev_gemm_bf16", "wp_simulate_reads", "wp_ctx_set_graphs", "wp_set_engine_config",
           "wp_autotune", "wp_mlp_create", "wp_mlp_destroy", "wp_mlp_train",
           "wp_mlp_train_step", "wp_mlp_shape", "wp_mlp_get", "wp_mlp_set", "wp_mlp_logits", "wp_mlp_propose",
           "wp_mlp_hybrid_classify", "wp_mlp_hybrid_classify_device", "wp_dedup_dye_tracks",
           "wp_simulate_dye_tracks", "wp_dye_tracks_download", "wp_dye_tracks_to_nn", "wp_fit_estep_batch",
           "wp_hmm_fit_batch", "wp_nn_set_selection", "wp_nn_kd_tree_order"]

# k-hit set of the kNN stage (wp_nn_set_selection)
NN_SELECTIONS = {"kdtree": 0, "prefix": 1}


class WpSeqModel(ctypes.Structure):
    _fields_ = [("num_channels", ctypes.c_int),
                ("p_edman_failure", ctypes.c_double),
                ("p_detach", ctypes.c_double),
                ("p_initial_detach", ctypes.c_double),
                ("p_initial_detach_decay", ctypes.c_double),
                ("p_initial_block", ctypes.c_double),
                ("p_cyclic_block", ctypes.c_double),
                ("p_bleach", ctypes.c_void_p),
                ("p_dud", ctypes.c_void_p),
                ("bg_sig", ctypes.c_void_p),
                ("mu", ctypes.c_void_p),
                ("sig", ctypes.c_void_p),
                ("interactions", ctypes.c_void_p),
                ("flat_interactions", ctypes.c_void_p)]


class WpFitSums(ctypes.Structure):
    """wp_fit_sums: the SequencingModelFitter fields of one E-step."""
    _fields_ = [("p_edman_failure_num", ctypes.c_double),
                ("p_edman_failure_den", ctypes.c_double),
                ("p_detach_x", ctypes.c_double * WP_MAX_TIMESTEPS),
                ("p_detach_n", ctypes.c_double * WP_MAX_TIMESTEPS),
                ("p_initial_block_num", ctypes.c_double),
                ("p_initial_block_den", ctypes.c_double),
                ("p_cyclic_block_num", ctypes.c_double),
                ("p_cyclic_block_den", ctypes.c_double),
                ("p_bleach_num", ctypes.c_double * WP_MAX_CHANNELS),
                ("p_bleach_den", ctypes.c_double * WP_MAX_CHANNELS),
                ("p_dud_num", ctypes.c_double * WP_MAX_CHANNELS),
                ("p_dud_den", ctypes.c_double * WP_MAX_CHANNELS)]

    def as_dict(self, T: int, C: int) -> dict:
        """Same keys as the oracle's fit sums."""
        return {
            "edman_num": self.p_edman_failure_num, "edman_den": self.p_edman_failure_den,
            "detach_x": np.array(self.p_detach_x[:max(T - 1, 0)]),
            "detach_n": np.array(self.p_detach_n[:max(T - 1, 0)]),
            "init_block_num": self.p_initial_block_num, "init_block_den": self.p_initial_block_den,
            "cyc_block_num": self.p_cyclic_block_num, "cyc_block_den": self.p_cyclic_block_den,
            "bleach_num": np.array(self.p_bleach_num[:C]), "bleach_den": np.array(self.p_bleach_den[:C]),
            "dud_num": np.array(self.p_dud_num[:C]), "dud_den": np.array(self.p_dud_den[:C]),
        }


class WpFitSettings(ctypes.Structure):
    """wp_fit_settings: FitSettings / ChannelFitSettings holds."""
    _fields_ = [("hold_p_edman_failure", ctypes.c_int),
                ("hold_p_detach", ctypes.c_int),
                ("hold_p_initial_detach", ctypes.c_int),
                ("hold_p_initial_detach_decay", ctypes.c_int),
                ("hold_p_initial_block", ctypes.c_int),
                ("hold_p_cyclic_block", ctypes.c_int),
                ("hold_p_bleach", ctypes.c_int * WP_MAX_CHANNELS),
                ("hold_p_dud", ctypes.c_int * WP_MAX_CHANNELS),
                ("fit_emission", ctypes.c_int)]


class WpFitParams(ctypes.Structure):
    """wp_fit_params: the fitted parameters of a SequencingModel."""
    _fields_ = [("p_edman_failure", ctypes.c_double),
                ("p_detach", ctypes.c_double),
                ("p_initial_detach", ctypes.c_double),
                ("p_initial_detach_decay", ctypes.c_double),
                ("p_initial_block", ctypes.c_double),
                ("p_cyclic_block", ctypes.c_double),
                ("p_bleach", ctypes.c_double * WP_MAX_CHANNELS),
                ("p_dud", ctypes.c_double * WP_MAX_CHANNELS),
                ("mu", ctypes.c_double * WP_MAX_CHANNELS),
                ("sig", ctypes.c_double * WP_MAX_CHANNELS),
                ("bg_sig", ctypes.c_double * WP_MAX_CHANNELS)]


WP_EMIS_N = 16  # dye counts 0..15


class WpEmissionSums(ctypes.Structure):
    """wp_emission_sums: posterior weight per (channel, dye count) at the
    emissions and its intensity moments (no reference counterpart)."""
    _fields_ = [("w", (ctypes.c_double * WP_EMIS_N) * WP_MAX_CHANNELS),
                ("x", (ctypes.c_double * WP_EMIS_N) * WP_MAX_CHANNELS),
                ("xx", (ctypes.c_double * WP_EMIS_N) * WP_MAX_CHANNELS)]

    def arrays(self, C: int):
        return (np.array([list(self.w[c]) for c in range(C)]), np.array([list(self.x[c]) for c in range(C)]),
                np.array([list(self.xx[c]) for c in range(C)]))


class WpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load_library(path: Optional[str] = None):
    """Load the CUDA library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} not built; run whatprot_gb300/build.py (there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.wp_ctx_create.argtypes = [ctypes.POINTER(V), I]
    lib.wp_ctx_create.restype = I
    lib.wp_ctx_destroy.argtypes = [V]
    lib.wp_ctx_destroy.restype = None
    lib.wp_last_error.argtypes = [V]
    lib.wp_last_error.restype = ctypes.c_char_p
    lib.wp_model_upload.argtypes = [V, ctypes.POINTER(WpSeqModel), I]
    lib.wp_model_upload.restype = I
    lib.wp_peptides_upload.argtypes = [V, V, V, V, V, I]
    lib.wp_peptides_upload.restype = I
    lib.wp_hmm_classify.argtypes = [V, V, I, D, V, V, V, V, V, V]
    lib.wp_hmm_classify.restype = I
    lib.wp_hmm_classify_device.argtypes = [V, V, I, D, V, V, V, I]
    lib.wp_hmm_classify_device.restype = I
    lib.wp_hmm_loglik_all.argtypes = [V, V, I, D, V]
    lib.wp_hmm_loglik_all.restype = I
    lib.wp_hmm_count_flops.argtypes = [V, V, I, D, ctypes.POINTER(D)]
    lib.wp_hmm_count_flops.restype = I
    lib.wp_launch_count.argtypes = [V]
    lib.wp_launch_count.restype = ctypes.c_longlong
    lib.wp_ctx_stream.argtypes = [V]
    lib.wp_ctx_stream.restype = V
    lib.wp_timing_enable.argtypes = [V, I]
    lib.wp_timing_enable.restype = I
    lib.wp_timing_read.argtypes = [V, I, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_longlong)]
    lib.wp_timing_read.restype = I
    lib.wp_probe_fp32_peak.argtypes = [V, ctypes.POINTER(D)]
    lib.wp_probe_fp32_peak.restype = I
    lib.wp_engine_replay.argtypes = [V, I, ctypes.POINTER(D)]
    lib.wp_engine_replay.restype = I
    lib.wp_last_batch_stats.argtypes = [V, V]
    lib.wp_last_batch_stats.restype = I
    lib.wp_fit_set_kernel.argtypes = [V, I]
    lib.wp_fit_set_kernel.restype = I
    lib.wp_fit_begin.argtypes = [V, V, I, V, I]
    lib.wp_fit_begin.restype = I
    lib.wp_fit_estep.argtypes = [V, ctypes.POINTER(WpFitSums), ctypes.POINTER(D), ctypes.POINTER(I)]
    lib.wp_fit_estep.restype = I
    lib.wp_hmm_fit.argtypes = [V, ctypes.POINTER(WpSeqModel), I, V, I, V, I,
                               ctypes.POINTER(WpFitSettings), D, D, ctypes.POINTER(WpFitParams),
                               ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(I)]
    lib.wp_hmm_fit.restype = I
    P_ = ctypes.POINTER
    lib.wp_fit_mstep.argtypes = [P_(WpFitSums), I, I, V, I, ctypes.c_longlong, P_(WpFitParams), P_(WpFitSettings),
                                 P_(WpFitParams), P_(D)]
    lib.wp_fit_mstep.restype = I
    lib.wp_hmm_bootstrap_fit.argtypes = [V, P_(WpSeqModel), I, V, I, V, I, P_(WpFitSettings), D, D, I, D,
                                         ctypes.c_ulonglong, V, V, P_(WpFitParams), P_(D), P_(D), P_(WpFitParams),
                                         P_(WpFitParams), P_(D)]
    lib.wp_hmm_bootstrap_fit.restype = I
    lib.wp_fit_offset_exponential.argtypes = [V, V, I, V, V]
    lib.wp_fit_offset_exponential.restype = I
    lib.wp_fit_set_emission.argtypes = [V, I]
    lib.wp_fit_set_emission.restype = I
    lib.wp_fit_emission_sums.argtypes = [V, P_(WpEmissionSums)]
    lib.wp_fit_emission_sums.restype = I
    lib.wp_fit_emission_mstep.argtypes = [P_(WpEmissionSums), I, P_(WpFitParams), P_(WpFitParams), P_(D)]
    lib.wp_fit_emission_mstep.restype = I
    lib.wp_nn_tracks_upload.argtypes = [V, V, I, I, I, V, V, V, V]
    lib.wp_nn_tracks_upload.restype = I
    lib.wp_nn_classify.argtypes = [V, V, I, I, D, I, V, V, V, V]
    lib.wp_nn_classify.restype = I
    lib.wp_nn_set_selection.argtypes = [V, I]
    lib.wp_nn_set_selection.restype = I
    lib.wp_nn_kd_tree_order.argtypes = [V, I, I, I, V, ctypes.POINTER(I)]
    lib.wp_nn_kd_tree_order.restype = I
    lib.wp_hybrid_classify.argtypes = [V, V, I, I, D, I, D, V, V, V]
    lib.wp_hybrid_classify.restype = I
    lib.wp_hybrid_classify_device.argtypes = [V, V, I, I, D, I, D, V, V, V]
    lib.wp_hybrid_classify_device.restype = I
    lib.wp_ctx_set_graphs.argtypes = [V, I]
    lib.wp_ctx_set_graphs.restype = I
    lib.wp_set_engine_config.argtypes = [V, V]
    lib.wp_set_engine_config.restype = I
    lib.wp_autotune.argtypes = [V, V, I, D, V, ctypes.POINTER(D)]
    lib.wp_autotune.restype = I
    lib.wp_simulate_reads.argtypes = [V, I, ctypes.c_ulonglong, V, V, V]
    lib.wp_simulate_reads.restype = I
    PI = ctypes.POINTER(I)
    lib.wp_dedup_dye_tracks.argtypes = [V, V, V, V, I, I, I, PI, PI]
    lib.wp_dedup_dye_tracks.restype = I
    lib.wp_simulate_dye_tracks.argtypes = [V, I, ctypes.c_ulonglong, PI, PI, V, V]
    lib.wp_simulate_dye_tracks.restype = I
    lib.wp_dye_tracks_download.argtypes = [V, V, V, V, V, V]
    lib.wp_dye_tracks_download.restype = I
    lib.wp_dye_tracks_to_nn.argtypes = [V]
    lib.wp_dye_tracks_to_nn.restype = I
    lib.wp_fit_estep_batch.argtypes = [V, V, I, V, I, V, V, V]
    lib.wp_fit_estep_batch.restype = I
    lib.wp_hmm_fit_batch.argtypes = [V, V, I, V, I, V, I, V, D, D, I, V, I, V, V, V]
    lib.wp_hmm_fit_batch.restype = I
    LL, U64, F = ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_float
    lib.wp_mlp_create.argtypes = [V, I, U64, ctypes.POINTER(V)]
    lib.wp_mlp_create.restype = I
    lib.wp_mlp_destroy.argtypes = [V]
    lib.wp_mlp_destroy.restype = None
    lib.wp_mlp_train.argtypes = [V, V, LL, I, F, U64, ctypes.POINTER(D)]
    lib.wp_mlp_train.restype = I
    lib.wp_mlp_train_step.argtypes = [V, V, V, V, I, F, ctypes.POINTER(D)]
    lib.wp_mlp_train_step.restype = I
    lib.wp_mlp_shape.argtypes = [V, I, ctypes.POINTER(LL), ctypes.POINTER(LL)]
    lib.wp_mlp_shape.restype = I
    lib.wp_mlp_get.argtypes = [V, I, I, V]
    lib.wp_mlp_get.restype = I
    lib.wp_mlp_set.argtypes = [V, V, I, V]
    lib.wp_mlp_set.restype = I
    lib.wp_mlp_logits.argtypes = [V, V, V, I, V]
    lib.wp_mlp_logits.restype = I
    lib.wp_mlp_propose.argtypes = [V, V, V, I, I, V, V, V]
    lib.wp_mlp_propose.restype = I
    lib.wp_mlp_hybrid_classify.argtypes = [V, V, V, I, I, D, V, V, V]
    lib.wp_mlp_hybrid_classify.restype = I
    lib.wp_mlp_hybrid_classify_device.argtypes = [V, V, V, I, I, D, V, V, V]
    lib.wp_mlp_hybrid_classify_device.restype = I
    lib.wp_dev_gemm_bf16.argtypes = [V, I, V, I, I, I, I, V, I, I, V, I, V]
    lib.wp_dev_gemm_bf16.restype = I
    if path is None:
        _lib = lib
    return lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def seq_model_struct(sm: SequencingModel):
    """A WpSeqModel view of sm, with the arrays it points to (keep them alive)."""
    C = sm.num_channels
    arr = lambda xs: np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
    cms = sm.channel_models
    keep = [arr([c.p_bleach for c in cms]), arr([c.p_dud for c in cms]),
            arr([c.bg_sig for c in cms]), arr([c.mu for c in cms]), arr([c.sig for c in cms]),
            arr([[c.interactions[o] for o in range(C)] for c in cms]).reshape(-1),
            arr([[c.flat_interactions[o] for o in range(C)] for c in cms]).reshape(-1)]
    m = WpSeqModel(C, sm.p_edman_failure, sm.p_detach, sm.p_initial_detach,
                   sm.p_initial_detach_decay, sm.p_initial_block, sm.p_cyclic_block,
                   *[k.ctypes.data for k in keep])
    return m, keep


def gemm_bf16(A, B, bias=None, act=0, out_fp32=True, want_z=False):
    """wp_dev_gemm_bf16 on torch CUDA tensors: act(A @ B.T + bias)."""
    import torch
    lib = load_library()
    M, K = A.shape
    N = B.shape[0]
    C = torch.empty(M, N, device=A.device, dtype=torch.float32 if out_fp32 else torch.bfloat16)
    Z = torch.empty(M, N, device=A.device, dtype=torch.bfloat16) if want_z else None
    st = lib.wp_dev_gemm_bf16(A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0), M, N, K, C.data_ptr(), N,
                              1 if out_fp32 else 0, bias.data_ptr() if bias is not None else None, act,
                              Z.data_ptr() if Z is not None else None)
    if st != 0:
        raise WpError(st, "wp_dev_gemm_bf16")
    return (C, Z) if want_z else C


def fit_offset_exponential(y, w, params, held=(False, False, False)):
    """wp_fit_offset_exponential: the detach M-step's bounded least squares
    (host code of the library; needs no GPU)."""
    lib = load_library()
    y = np.ascontiguousarray(y, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64).copy()
    h = np.ascontiguousarray([1 if x else 0 for x in held], dtype=np.int32)
    st = lib.wp_fit_offset_exponential(_ptr(y), _ptr(w), len(y), _ptr(h), _ptr(p))
    if st != 0:
        raise WpError(st, "wp_fit_offset_exponential")
    return p


def emission_mstep(w, x, xx, mu, sig, bg_sig):
    """wp_fit_emission_mstep (host code, no GPU): per channel the mu, sig and
    bg_sig maximising the expected log-likelihood of the intensities given
    the emission statistics w, x, xx [C, n], from the current values.
    Returns (mu, sig, bg_sig, step)."""
    lib = load_library()
    w, x, xx = (np.asarray(v, dtype=np.float64) for v in (w, x, xx))
    C = w.shape[0]
    s = WpEmissionSums()
    for c in range(C):
        for n in range(min(w.shape[1], WP_EMIS_N)):
            s.w[c][n], s.x[c][n], s.xx[c][n] = w[c, n], x[c, n], xx[c, n]
    cur = WpFitParams()
    for c in range(C):
        cur.mu[c], cur.sig[c], cur.bg_sig[c] = mu[c], sig[c], bg_sig[c]
    nxt = WpFitParams()
    step = ctypes.c_double(0.0)
    st = lib.wp_fit_emission_mstep(ctypes.byref(s), C, ctypes.byref(cur), ctypes.byref(nxt), ctypes.byref(step))
    if st != 0:
        raise WpError(st, "wp_fit_emission_mstep")
    return (np.array(nxt.mu[:C]), np.array(nxt.sig[:C]), np.array(nxt.bg_sig[:C]), step.value)


class DyeTrackBuffers:
    """Reusable host buffers for downloaded dye-track sets, page-locked when
    torch is importable (device-to-host copies then run at the link's
    rate): up to max_tracks tracks of T x C counts and max_sources sources."""

    def __init__(self, max_tracks: int, max_sources: int, T: int, C: int, pinned: bool = True):
        def alloc(n, dtype):
            if pinned:
                try:
                    import torch
                    tdt = {np.int16: torch.int16, np.int32: torch.int32}[dtype]
                    return torch.empty(max(n, 1), dtype=tdt, pin_memory=True).numpy()
                except Exception:
                    pass
            return np.zeros(max(n, 1), dtype)
        self.max_tracks, self.max_sources, self.T, self.C = max_tracks, max_sources, T, C
        self.counts = alloc(max_tracks * T * C, np.int16)
        self.off = alloc(max_tracks + 1, np.int32)
        self.sid, self.scnt, self.shit = (alloc(max_sources, np.int32) for _ in range(3))

    def views(self, U: int, S: int, T: int, C: int):
        if U > self.max_tracks or S > self.max_sources or (T, C) != (self.T, self.C):
            raise ValueError("dye-track set larger than the buffers")
        return (self.counts[: max(U, 1) * T * C].reshape(max(U, 1), T, C), self.off[: U + 1], self.sid,
                self.scnt, self.shit)


class Context:
    """One wp_ctx on one CUDA device (the C ABI's handle)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        st = self.lib.wp_ctx_create(ctypes.byref(h), device)
        if st != 0:
            raise WpError(st, "wp_ctx_create failed (no CUDA device?)")
        self.h = h
        self.num_timesteps = None
        self.num_channels = None
        self._keep = []

    def close(self):
        if self.h:
            self.lib.wp_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != 0:
            raise WpError(st, self.lib.wp_last_error(self.h).decode())

    def upload_model(self, sm: SequencingModel, num_timesteps: int) -> None:
        C = sm.num_channels
        m, keep = seq_model_struct(sm)
        self._check(self.lib.wp_model_upload(self.h, ctypes.byref(m), num_timesteps))
        self.num_timesteps = num_timesteps
        self.num_channels = C

    def upload_peptides(self, ds: DyeSeqSet) -> None:
        flat, off = ds.ragged()
        ids = np.ascontiguousarray(ds.ids, dtype=np.int32)
        counts = np.ascontiguousarray(ds.counts, dtype=np.int32)
        self._check(self.lib.wp_peptides_upload(self.h, _ptr(flat), _ptr(off), _ptr(ids),
                                                _ptr(counts), len(ds)))
        self.num_peptides = len(ds)
        self._pep_counts = counts.copy()

    def classify(self, rads: np.ndarray, dist_cutoff: float = DBL_MAX,
                 cand: Optional[np.ndarray] = None, cand_off: Optional[np.ndarray] = None, out=None):
        """wp_hmm_classify: (best id, score, total, log score) per read.  out:
        four caller-owned arrays (int32, float64 x 3, at least R each) to
        write into and return instead of fresh ones (e.g. pinned buffers
        reused across batches)."""
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        if out is not None:
            oid, osc, otot, olog = out
            for arr, dt in zip(out, (np.int32, np.float64, np.float64, np.float64)):
                if arr.dtype != dt or arr.shape[0] < R or not arr.flags.c_contiguous:
                    raise ValueError("out arrays: int32, float64, float64, float64, contiguous, at least R long")
        else:
            oid = np.zeros(R, np.int32)
            osc = np.zeros(R, np.float64)
            otot = np.zeros(R, np.float64)
            olog = np.zeros(R, np.float64)
        if cand is not None:
            cand = np.ascontiguousarray(cand, np.int32)
            cand_off = np.ascontiguousarray(cand_off, np.int32)
        self._check(self.lib.wp_hmm_classify(self.h, _ptr(rads), R, dist_cutoff, _ptr(cand),
                                             _ptr(cand_off), _ptr(oid), _ptr(osc), _ptr(otot),
                                             _ptr(olog)))
        return oid, osc, otot, olog

    def classify_device(self, d_rads_ptr: int, R: int, dist_cutoff: float, d_id: int,
                        d_score: int, d_total: int, async_: bool = True) -> None:
        self._check(self.lib.wp_hmm_classify_device(self.h, ctypes.c_void_p(d_rads_ptr), R,
                                                    dist_cutoff, ctypes.c_void_p(d_id),
                                                    ctypes.c_void_p(d_score),
                                                    ctypes.c_void_p(d_total), 1 if async_ else 0))

    def loglik_all(self, rads: np.ndarray, dist_cutoff: float = DBL_MAX) -> np.ndarray:
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        out = np.zeros((R, self.num_peptides), np.float64)
        self._check(self.lib.wp_hmm_loglik_all(self.h, _ptr(rads), R, dist_cutoff, _ptr(out)))
        return out

    def count_flops(self, rads: np.ndarray, dist_cutoff: float = DBL_MAX) -> float:
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        out = ctypes.c_double()
        self._check(self.lib.wp_hmm_count_flops(self.h, _ptr(rads), rads.shape[0], dist_cutoff,
                                                ctypes.byref(out)))
        return out.value

    def fit_begin(self, dye_seq, rads: np.ndarray) -> None:
        """wp_fit_begin: stage one dye-seq (int list, -1 unlabeled) and its
        reads [R, T, C] (divided by mu) for E-steps."""
        seq = np.ascontiguousarray(dye_seq, dtype=np.int16)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        self._check(self.lib.wp_fit_begin(self.h, _ptr(seq) if len(seq) else None, len(seq),
                                          _ptr(rads), rads.shape[0]))

    def fit_set_kernel(self, kind: int) -> None:
        """wp_fit_set_kernel: 0 CTA per read where it fits (default), 1 thread per read."""
        self._check(self.lib.wp_fit_set_kernel(self.h, kind))

    def fit_set_emission(self, enable: bool) -> None:
        """wp_fit_set_emission: later E-steps also gather the emission statistics."""
        self._check(self.lib.wp_fit_set_emission(self.h, 1 if enable else 0))

    def fit_emission_sums(self) -> "WpEmissionSums":
        """wp_fit_emission_sums: the emission statistics of the last E-step."""
        s = WpEmissionSums()
        self._check(self.lib.wp_fit_emission_sums(self.h, ctypes.byref(s)))
        return s

    def fit_estep(self):
        """wp_fit_estep with the current model: (WpFitSums, sum log P, reads with P == 0)."""
        s = WpFitSums()
        sl = ctypes.c_double(0.0)
        nz = ctypes.c_int(0)
        self._check(self.lib.wp_fit_estep(self.h, ctypes.byref(s), ctypes.byref(sl), ctypes.byref(nz)))
        return s, sl.value, nz.value

    def fit_estep_batch(self, models, read_idx: np.ndarray):
        """wp_fit_estep_batch: one E-step per model over its row of read_idx
        (indices into the staged reads): (list of WpFitSums, sum log P [B],
        reads with P == 0 [B])."""
        B = len(models)
        idx = np.ascontiguousarray(read_idx, dtype=np.int32).reshape(B, -1)
        built = [seq_model_struct(m) for m in models]
        arr = (WpSeqModel * B)(*[b[0] for b in built])
        out = (WpFitSums * B)()
        sl = np.zeros(B, np.float64)
        nz = np.zeros(B, np.int32)
        self._check(self.lib.wp_fit_estep_batch(self.h, ctypes.byref(arr), B, _ptr(idx), idx.shape[1],
                                                ctypes.byref(out), _ptr(sl), _ptr(nz)))
        return [out[b] for b in range(B)], sl, nz

    def hmm_fit_batch(self, start: SequencingModel, num_timesteps: int, dye_seq, rads: np.ndarray,
                      read_idx: np.ndarray, stopping_threshold: float, max_runtime: float = 1e300,
                      holds: Optional[dict] = None):
        """wp_hmm_fit_batch: B fits from `start` at once, fit b on the reads
        rads[read_idx[b]]: (fitted SequencingModels, log-likelihoods [B],
        step sizes [B])."""
        m, keep = seq_model_struct(start)
        seq = np.ascontiguousarray(dye_seq, dtype=np.int16)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        idx = np.ascontiguousarray(read_idx, dtype=np.int32)
        B = idx.shape[0]
        fs = WpFitSettings()
        for k, v in (holds or {}).items():
            if k in ("hold_p_bleach", "hold_p_dud"):
                arr = getattr(fs, k)
                for c, h in enumerate(v):
                    arr[c] = 1 if h else 0
            else:
                setattr(fs, k, 1 if v else 0)
        out = (WpFitParams * B)()
        lls = np.zeros(B, np.float64)
        steps = np.zeros(B, np.float64)
        self._check(self.lib.wp_hmm_fit_batch(self.h, ctypes.byref(m), num_timesteps,
                                              _ptr(seq) if len(seq) else None, len(seq), _ptr(rads), rads.shape[0],
                                              ctypes.byref(fs), stopping_threshold, max_runtime, B, _ptr(idx),
                                              idx.shape[1], ctypes.byref(out), _ptr(lls), _ptr(steps)))
        self.num_timesteps = num_timesteps
        self.num_channels = start.num_channels
        return [self._params_to_model(start, out[b]) for b in range(B)], lls, steps

    def hmm_fit(self, start: SequencingModel, num_timesteps: int, dye_seq, rads: np.ndarray,
                stopping_threshold: float, max_runtime: float = 1e300, holds: Optional[dict] = None,
                fit_emission: bool = False):
        """wp_hmm_fit: (fitted SequencingModel, step size, log-likelihood, iterations).
        fit_emission also fits each channel's mu, sig and bg_sig (no
        reference counterpart)."""
        import copy
        m, keep = seq_model_struct(start)
        seq = np.ascontiguousarray(dye_seq, dtype=np.int16)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        fs = WpFitSettings()
        for k, v in (holds or {}).items():
            if k in ("hold_p_bleach", "hold_p_dud"):
                arr = getattr(fs, k)
                for c, h in enumerate(v):
                    arr[c] = 1 if h else 0
            else:
                setattr(fs, k, 1 if v else 0)
        fs.fit_emission = 1 if fit_emission else 0
        out = WpFitParams()
        step = ctypes.c_double(0.0)
        ll = ctypes.c_double(0.0)
        it = ctypes.c_int(0)
        self._check(self.lib.wp_hmm_fit(self.h, ctypes.byref(m), num_timesteps,
                                        _ptr(seq) if len(seq) else None, len(seq), _ptr(rads),
                                        rads.shape[0], ctypes.byref(fs), stopping_threshold,
                                        max_runtime, ctypes.byref(out), ctypes.byref(step),
                                        ctypes.byref(ll), ctypes.byref(it)))
        fitted = self._params_to_model(start, out)
        self.num_timesteps = num_timesteps
        self.num_channels = start.num_channels
        return fitted, step.value, ll.value, it.value

    def upload_tracks(self, dts) -> None:
        """wp_nn_tracks_upload: the kNN training set (io.DyeTrackSet)."""
        tr = np.ascontiguousarray(dts.tracks, dtype=np.int16)
        N, T, C = tr.shape
        arr = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        off, sid, scnt, shit = arr(dts.src_off), arr(dts.src_id), arr(dts.src_count), arr(dts.src_hits)
        self._check(self.lib.wp_nn_tracks_upload(self.h, _ptr(tr), N, T, C, _ptr(off), _ptr(sid), _ptr(scnt),
                                                 _ptr(shit)))

    def dedup_dye_tracks(self, counts: np.ndarray, ids: np.ndarray, src_counts: np.ndarray):
        """wp_dedup_dye_tracks on dye-tracks counts [n, T, C] from sources
        (ids, src_counts); returns the deduplicated io.DyeTrackSet."""
        tr = np.ascontiguousarray(counts, dtype=np.int16)
        n, T, C = tr.shape
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        cnt = np.ascontiguousarray(src_counts, dtype=np.int32)
        if ids.shape != (n,) or cnt.shape != (n,):
            raise ValueError("ids and src_counts need one entry per dye-track")
        nu, ns = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.lib.wp_dedup_dye_tracks(self.h, _ptr(tr), _ptr(ids), _ptr(cnt), n, T, C,
                                                 ctypes.byref(nu), ctypes.byref(ns)))
        return self._download_dye_tracks(nu.value, ns.value, T, C)

    def simulate_dye_track_set(self, per_peptide: int, seed: int = 0, instances: bool = False,
                               to_nn: bool = False, download: bool = True, into=None):
        """wp_simulate_dye_tracks: the kNN training set of per_peptide
        dye-tracks per peptide copy, generated and deduplicated on the device
        with the uploaded model and peptides.  Returns the io.DyeTrackSet
        (None when download is False), plus the instances (tracks [n, T, C]
        uint8, peptide index [n]) when asked; to_nn makes the set the kNN /
        hybrid training set without a host round trip of the caller's.
        `into` (a DyeTrackBuffers) receives the set in reusable (pinned)
        host memory; the returned arrays are views of it, valid until its
        next use."""
        T, C = self.num_timesteps, self.num_channels
        n = int(per_peptide) * int(np.sum(getattr(self, "_pep_counts", np.zeros(0)), dtype=np.int64))
        itr = np.zeros((max(n, 1), T, C), np.uint8) if instances else None
        ipep = np.zeros(max(n, 1), np.int32) if instances else None
        nu, ns = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.lib.wp_simulate_dye_tracks(self.h, int(per_peptide), ctypes.c_ulonglong(seed),
                                                    ctypes.byref(nu), ctypes.byref(ns), _ptr(itr), _ptr(ipep)))
        if to_nn:
            self._check(self.lib.wp_dye_tracks_to_nn(self.h))
        dts = self._download_dye_tracks(nu.value, ns.value, T, C, into) if download else None
        if instances:
            return dts, itr[:n], ipep[:n]
        return dts

    def _download_dye_tracks(self, U: int, S: int, T: int, C: int, into=None):
        from .io import DyeTrackSet
        if into is not None:
            counts, off, sid, scnt, shit = into.views(U, S, T, C)
        else:
            counts = np.zeros((max(U, 1), T, C), np.int16)
            off = np.zeros(U + 1, np.int32)
            sid, scnt, shit = (np.zeros(max(S, 1), np.int32) for _ in range(3))
        self._check(self.lib.wp_dye_tracks_download(self.h, _ptr(counts), _ptr(off), _ptr(sid), _ptr(scnt),
                                                    _ptr(shit)))
        return DyeTrackSet(counts[:U], off[:U + 1], sid[:S], scnt[:S], shit[:S])

    def set_nn_selection(self, selection: str) -> None:
        """wp_nn_set_selection: "kdtree" (the reference's kd-tree search
        with KBest, the default) or "prefix" (the shortest distance-ordered
        prefix reaching k hits)."""
        if selection not in NN_SELECTIONS:
            raise ValueError(f"unknown kNN selection {selection!r}")
        self._check(self.lib.wp_nn_set_selection(self.h, NN_SELECTIONS[selection]))

    def nn_classify(self, rads: np.ndarray, k: int, sig: float, h: int):
        """wp_nn_classify: (ncand [R], ids [R,h], scores [R,h], total [R])."""
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        nc = np.zeros(R, np.int32)
        ids = np.zeros((R, h), np.int32)
        sc = np.zeros((R, h), np.float64)
        tot = np.zeros(R, np.float64)
        self._check(self.lib.wp_nn_classify(self.h, _ptr(rads), R, k, sig, h, _ptr(nc), _ptr(ids), _ptr(sc),
                                            _ptr(tot)))
        return nc, ids, sc, tot

    def hybrid_classify(self, rads: np.ndarray, k: int, sig: float, h: int, dist_cutoff: float):
        """wp_hybrid_classify: (ids, scores, totals) per read."""
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        ids = np.zeros(R, np.int32)
        sc = np.zeros(R, np.float64)
        tot = np.zeros(R, np.float64)
        self._check(self.lib.wp_hybrid_classify(self.h, _ptr(rads), R, k, sig, h, dist_cutoff, _ptr(ids),
                                                _ptr(sc), _ptr(tot)))
        return ids, sc, tot

    def hybrid_classify_device(self, d_rads_ptr: int, R: int, k: int, sig: float, h: int, dist_cutoff: float,
                               d_id: int, d_score: int, d_total: int) -> None:
        """wp_hybrid_classify_device on device pointers (e.g. torch tensors)."""
        self._check(self.lib.wp_hybrid_classify_device(self.h, ctypes.c_void_p(d_rads_ptr), R, k, sig, h,
                                                       dist_cutoff, ctypes.c_void_p(d_id), ctypes.c_void_p(d_score),
                                                       ctypes.c_void_p(d_total)))

    def set_graphs(self, enable: bool) -> None:
        self._check(self.lib.wp_ctx_set_graphs(self.h, 1 if enable else 0))

    def set_engine_config(self, cfg=None) -> None:
        """(pass-1 threads, pass-1 CTAs/SM, pass-2 threads, pass-2 CTAs/SM) or None."""
        arr = None if cfg is None else np.ascontiguousarray(cfg, dtype=np.int32)
        self._check(self.lib.wp_set_engine_config(self.h, _ptr(arr)))

    def autotune(self, rads: np.ndarray, dist_cutoff: float = DBL_MAX):
        """wp_autotune on a sample of reads: (chosen shape, its ms)."""
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        cfg = np.zeros(4, np.int32)
        ms = ctypes.c_double()
        self._check(self.lib.wp_autotune(self.h, _ptr(rads), rads.shape[0], dist_cutoff, _ptr(cfg),
                                         ctypes.byref(ms)))
        return tuple(int(x) for x in cfg), ms.value

    def simulate_reads(self, R: int, seed: int, tracks: bool = False):
        """wp_simulate_reads: (rads [R,T,C], peptide index [R] (-1: not
        detectable), tracks [R,T,C] uint8 or None)."""
        T, C = self.num_timesteps, self.num_channels
        rads = np.zeros((R, T, C), np.float64)
        pep = np.zeros(R, np.int32)
        trk = np.zeros((R, T, C), np.uint8) if tracks else None
        self._check(self.lib.wp_simulate_reads(self.h, R, seed, _ptr(rads), _ptr(pep), _ptr(trk)))
        return rads, pep, trk

    @staticmethod
    def _params_to_model(start: SequencingModel, out: "WpFitParams") -> SequencingModel:
        import copy
        m = copy.deepcopy(start)
        for k in ("p_edman_failure", "p_detach", "p_initial_detach", "p_initial_detach_decay",
                  "p_initial_block", "p_cyclic_block"):
            setattr(m, k, getattr(out, k))
        for c, cm in enumerate(m.channel_models):
            cm.p_bleach = out.p_bleach[c]
            cm.p_dud = out.p_dud[c]
            cm.mu = out.mu[c]
            cm.sig = out.sig[c]
            cm.bg_sig = out.bg_sig[c]
        return m

    def bootstrap_fit(self, start: SequencingModel, num_timesteps: int, dye_seq, rads: np.ndarray,
                      stopping_threshold: float, num_rounds: int, confidence_interval: float, seed: int = 1,
                      max_runtime: float = 1e300, holds: Optional[dict] = None, fit_emission: bool = False) -> dict:
        """wp_hmm_bootstrap_fit: per-round models and log-likelihoods, the fit
        on all reads, and the confidence bounds."""
        m, keep = seq_model_struct(start)
        seq = np.ascontiguousarray(dye_seq, dtype=np.int16)
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        fs = WpFitSettings()
        for k, v in (holds or {}).items():
            if k in ("hold_p_bleach", "hold_p_dud"):
                arr = getattr(fs, k)
                for c, h in enumerate(v):
                    arr[c] = 1 if h else 0
            else:
                setattr(fs, k, 1 if v else 0)
        fs.fit_emission = 1 if fit_emission else 0
        rounds = (WpFitParams * num_rounds)()
        lls = np.zeros(num_rounds, np.float64)
        best, lo, hi = WpFitParams(), WpFitParams(), WpFitParams()
        step, bll, worst = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.wp_hmm_bootstrap_fit(self.h, ctypes.byref(m), num_timesteps,
                                                  _ptr(seq) if len(seq) else None, len(seq), _ptr(rads),
                                                  rads.shape[0], ctypes.byref(fs), stopping_threshold, max_runtime,
                                                  num_rounds, confidence_interval, seed, ctypes.byref(rounds),
                                                  _ptr(lls), ctypes.byref(best), ctypes.byref(step),
                                                  ctypes.byref(bll), ctypes.byref(lo), ctypes.byref(hi),
                                                  ctypes.byref(worst)))
        self.num_timesteps = num_timesteps
        self.num_channels = start.num_channels
        return {"models": [self._params_to_model(start, rounds[i]) for i in range(num_rounds)],
                "log_ls": lls, "best": self._params_to_model(start, best), "step_size": step.value,
                "log_l": bll.value, "ci_min": self._params_to_model(start, lo),
                "ci_max": self._params_to_model(start, hi), "worst_round_step": worst.value}

    def launch_count(self) -> int:
        return int(self.lib.wp_launch_count(self.h))

    def stream_handle(self) -> int:
        return int(self.lib.wp_ctx_stream(self.h) or 0)

    def timing_enable(self, on: bool = True) -> None:
        self._check(self.lib.wp_timing_enable(self.h, 1 if on else 0))

    KIND_FORWARD, KIND_PREP, KIND_COMBINE, KIND_FLOPS, KIND_KNN_DIST, KIND_KNN_SELECT = 0, 1, 2, 3, 4, 5
    KIND_SIM, KIND_DEDUP, KIND_KNN_TREE = 6, 7, 8

    def timing_read(self, kind: int) -> Tuple[float, int]:
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        self._check(self.lib.wp_timing_read(self.h, kind, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def last_batch_stats(self) -> dict:
        out = np.zeros(4, np.int64)
        self._check(self.lib.wp_last_batch_stats(self.h, _ptr(out)))
        return {"slots": int(out[0]), "nonempty": int(out[1]), "pass2": int(out[2]), "dense": int(out[3])}

    def fp32_peak_tflops(self) -> float:
        out = ctypes.c_double()
        self._check(self.lib.wp_probe_fp32_peak(self.h, ctypes.byref(out)))
        return out.value

    def engine_replay(self, reps: int) -> float:
        """wp_engine_replay: the last classify batch's engine passes run
        `reps` more times; their elapsed ms."""
        out = ctypes.c_double()
        self._check(self.lib.wp_engine_replay(self.h, int(reps), ctypes.byref(out)))
        return out.value


class ScoredClassification:
    """common/scored-classification.{h,cc}: id, score, total; adjusted_score =
    score / total."""
    __slots__ = ("id", "score", "total")

    def __init__(self, id: int, score: float, total: float):
        self.id = id
        self.score = score
        self.total = total

    def adjusted_score(self) -> float:
        return self.score / self.total


class HMMClassifier:
    """Mirror of the reference's HMMClassifier (classifiers/hmm-classifier.h:
    32-43): construct with (num_timesteps, num_channels, seq_model,
    seq_settings dist_cutoff, dye_seqs) and classify one or many radiometries,
    optionally restricted to candidate peptide indices.  Runs on the GPU
    through the C ABI."""

    def __init__(self, num_timesteps: int, num_channels: int, seq_model: SequencingModel,
                 dist_cutoff: float, dye_seqs: DyeSeqSet, device: int = 0,
                 context: Optional[Context] = None):
        if seq_model.num_channels != num_channels or dye_seqs.num_channels != num_channels:
            raise ValueError("num_channels mismatch")
        self.ctx = context or Context(device)
        self.ctx.upload_model(seq_model, num_timesteps)
        self.ctx.upload_peptides(dye_seqs)
        self.num_timesteps = num_timesteps
        self.num_channels = num_channels
        self.dist_cutoff = dist_cutoff
        self.dye_seqs = dye_seqs

    def classify(self, radiometries: np.ndarray, candidate_indices=None):
        """radiometries: [T, C] (one read) or [R, T, C].  candidate_indices:
        one list (single read) or a list of lists (one per read)."""
        rads = np.asarray(radiometries, dtype=np.float64)
        single = rads.ndim == 2
        if single:
            rads = rads[None]
            if candidate_indices is not None:
                candidate_indices = [candidate_indices]
        cand = cand_off = None
        if candidate_indices is not None:
            cand_off = np.zeros(len(candidate_indices) + 1, np.int32)
            for i, c in enumerate(candidate_indices):
                cand_off[i + 1] = cand_off[i] + len(c)
            cand = (np.concatenate([np.asarray(c, np.int32) for c in candidate_indices])
                    if cand_off[-1] else np.zeros(1, np.int32))
        ids, sc, tot, _ = self.ctx.classify(rads, self.dist_cutoff, cand, cand_off)
        res = [ScoredClassification(int(i), float(s), float(t)) for i, s, t in zip(ids, sc, tot)]
        return res[0] if single else res


class HMMFitter:
    """Host mirror of HMMFitter (fitters/hmm-fitter.h:35-150): Baum-Welch on
    one dye-seq with GPU E-steps.  ``fit_settings`` maps the FitSettings hold
    names (``hold_p_edman_failure`` ... ``hold_p_cyclic_block``,
    ``hold_p_bleach`` / ``hold_p_dud`` as per-channel lists) to booleans."""

    def __init__(self, num_timesteps: int, num_channels: int, stopping_threshold: float,
                 max_runtime: float, seq_model: SequencingModel, fit_settings: Optional[dict],
                 dye_seq, device: int = 0):
        from .model import parse_dye_seq
        self.num_timesteps = num_timesteps
        self.num_channels = num_channels
        self.stopping_threshold = stopping_threshold
        self.max_runtime = max_runtime
        self.seq_model = seq_model
        self.fit_settings = dict(fit_settings or {})
        self.dye_seq = (parse_dye_seq(dye_seq) if isinstance(dye_seq, str)
                        else np.asarray(dye_seq, dtype=np.int16))
        self.ctx = Context(device)
        self.step_size = None
        self.iterations = None

    def fit(self, radiometries: np.ndarray):
        """(fitted SequencingModel, log-likelihood); step size and iteration
        count are kept in .step_size and .iterations."""
        fitted, step, ll, it = self.ctx.hmm_fit(self.seq_model, self.num_timesteps, self.dye_seq,
                                                radiometries, self.stopping_threshold,
                                                self.max_runtime, self.fit_settings)
        self.step_size = step
        self.iterations = it
        return fitted, ll

    def log_likelihood(self, radiometries: np.ndarray, seq_model: SequencingModel) -> float:
        """Sum of log P over the reads (fitters/hmm-fitter.h:119-142); -inf
        when some read has P == 0."""
        self.ctx.upload_model(seq_model, self.num_timesteps)
        self.ctx.fit_begin(self.dye_seq, radiometries)
        _, sl, nz = self.ctx.fit_estep()
        return float("-inf") if nz else sl


def kd_tree_order(coords: np.ndarray, k: int):
    """wp_nn_kd_tree_order (host only): the kd-tree NNClassifier builds
    over coords [N, D] for k; returns (perm [N], number of nodes), perm[i]
    the input index of the entry at tree position i."""
    lib = load_library()
    x = np.ascontiguousarray(coords, dtype=np.float64)
    N, D = x.shape
    perm = np.zeros(max(N, 1), np.int32)
    nn = ctypes.c_int(0)
    st = lib.wp_nn_kd_tree_order(_ptr(x), N, D, int(k), _ptr(perm), ctypes.byref(nn))
    if st != 0:
        raise WpError(st, STATUS.get(st, str(st)))
    return perm[:N], nn.value


class NNClassifier:
    """Host mirror of NNClassifier (classifiers/nn-classifier.h:60-82) on the
    GPU kNN stage.  The reference's constructor moves the dye-tracks out of
    the caller's vector; this one copies them to the device."""

    def __init__(self, num_timesteps: int, num_channels: int, seq_model: SequencingModel, k: int,
                 sig: float, dye_tracks, device: int = 0, selection: str = "kdtree"):
        self.ctx = Context(device)
        self.ctx.upload_model(seq_model, num_timesteps)
        self.ctx.upload_tracks(dye_tracks)
        self.ctx.set_nn_selection(selection)
        self.k, self.sig = k, sig

    def classify(self, radiometries: np.ndarray, h: Optional[int] = None):
        """One read [T, C] or many [R, T, C].  Without h: the best
        ScoredClassification per read (NaN patched, nn-classifier.cc:164-181);
        with h: up to h ScoredClassifications per read in ascending score."""
        rads = np.asarray(radiometries, dtype=np.float64)
        single = rads.ndim == 2
        if single:
            rads = rads[None]
        nc, ids, sc, tot = self.ctx.nn_classify(rads, self.k, self.sig, 1 if h is None else h)
        out = []
        for r in range(rads.shape[0]):
            if h is None:
                if nc[r] == 0:
                    res = ScoredClassification(-1, -1.0, float(tot[r]))
                else:
                    res = ScoredClassification(int(ids[r, nc[r] - 1]), float(sc[r, nc[r] - 1]), float(tot[r]))
                if math.isnan(res.adjusted_score()):
                    res.score, res.total = 0.0, 1.0
                out.append(res)
            else:
                out.append([ScoredClassification(int(ids[r, i]), float(sc[r, i]), float(tot[r]))
                            for i in range(nc[r])])
        return out[0] if single else out


class HybridClassifier:
    """Host mirror of HybridClassifier (classifiers/hybrid-classifier.h:31-51):
    kNN candidates, then the HMM over them, on the GPU."""

    def __init__(self, num_timesteps: int, num_channels: int, seq_model: SequencingModel,
                 dist_cutoff: float, k: int, sig: float, dye_tracks, h: int, dye_seqs: DyeSeqSet,
                 device: int = 0, selection: str = "kdtree"):
        self.ctx = Context(device)
        self.ctx.upload_model(seq_model, num_timesteps)
        self.ctx.upload_peptides(dye_seqs)
        self.ctx.upload_tracks(dye_tracks)
        self.ctx.set_nn_selection(selection)
        self.k, self.sig, self.h, self.dist_cutoff = k, sig, h, dist_cutoff

    def classify(self, radiometries: np.ndarray):
        rads = np.asarray(radiometries, dtype=np.float64)
        single = rads.ndim == 2
        if single:
            rads = rads[None]
        ids, sc, tot = self.ctx.hybrid_classify(rads, self.k, self.sig, self.h, self.dist_cutoff)
        res = [ScoredClassification(int(i), float(s), float(t)) for i, s, t in zip(ids, sc, tot)]
        return res[0] if single else res


class ProposalNet:
    """The learned proposal network on a Context (wp_mlp_*): built for the
    context's current model and peptide set."""

    PARAMS = ("W1", "b1", "W2", "b2", "W3", "b3")

    def __init__(self, ctx: "Context", hidden: int = 1024, seed: int = 1):
        self.ctx = ctx
        self.lib = ctx.lib
        h = ctypes.c_void_p()
        ctx._check(self.lib.wp_mlp_create(ctx.h, hidden, seed, ctypes.byref(h)))
        self.h = h
        self.hidden = hidden

    def close(self):
        if self.h:
            self.lib.wp_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def train(self, num_reads: int, batch: int = 4096, lr: float = 1e-3, seed: int = 7) -> float:
        loss = ctypes.c_double(0.0)
        self.ctx._check(self.lib.wp_mlp_train(self.ctx.h, self.h, num_reads, batch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def train_step(self, d_x_ptr: int, d_labels_ptr: int, B: int, lr: float) -> float:
        loss = ctypes.c_double(0.0)
        self.ctx._check(self.lib.wp_mlp_train_step(self.ctx.h, self.h, ctypes.c_void_p(d_x_ptr),
                                                   ctypes.c_void_p(d_labels_ptr), B, lr, ctypes.byref(loss)))
        return loss.value

    def shape(self, which: int):
        r, c = ctypes.c_longlong(), ctypes.c_longlong()
        self.lib.wp_mlp_shape(self.h, which, ctypes.byref(r), ctypes.byref(c))
        return int(r.value), int(c.value)

    def get(self, which: int, grad: bool = False) -> np.ndarray:
        r, c = self.shape(which)
        out = np.zeros((r, c), np.float32)
        st = self.lib.wp_mlp_get(self.h, which, 1 if grad else 0, _ptr(out))
        if st != 0:
            raise WpError(st, "wp_mlp_get")
        return out if c > 1 else out.reshape(-1)

    def set(self, which: int, value: np.ndarray) -> None:
        v = np.ascontiguousarray(value, dtype=np.float32)
        self.ctx._check(self.lib.wp_mlp_set(self.ctx.h, self.h, which, _ptr(v)))

    def logits(self, rads: np.ndarray) -> np.ndarray:
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        out = np.zeros((rads.shape[0], self.ctx.num_peptides), np.float32)
        self.ctx._check(self.lib.wp_mlp_logits(self.ctx.h, self.h, _ptr(rads), rads.shape[0], _ptr(out)))
        return out

    def propose(self, rads: np.ndarray, h: int):
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        idx = np.zeros((R, h), np.int32)
        prob = np.zeros((R, h), np.float32)
        mass = np.zeros(R, np.float64)
        self.ctx._check(self.lib.wp_mlp_propose(self.ctx.h, self.h, _ptr(rads), R, h, _ptr(idx), _ptr(prob),
                                                _ptr(mass)))
        return idx, prob, mass

    def hybrid_classify(self, rads: np.ndarray, h: int, dist_cutoff: float):
        rads = np.ascontiguousarray(rads, dtype=np.float64)
        R = rads.shape[0]
        ids = np.zeros(R, np.int32)
        sc = np.zeros(R, np.float64)
        tot = np.zeros(R, np.float64)
        self.ctx._check(self.lib.wp_mlp_hybrid_classify(self.ctx.h, self.h, _ptr(rads), R, h, dist_cutoff, _ptr(ids),
                                                        _ptr(sc), _ptr(tot)))
        return ids, sc, tot

    def hybrid_classify_device(self, d_rads_ptr: int, R: int, h: int, dist_cutoff: float, d_id: int, d_score: int,
                               d_total: int) -> None:
        self.ctx._check(self.lib.wp_mlp_hybrid_classify_device(self.ctx.h, self.h, ctypes.c_void_p(d_rads_ptr), R, h,
                                                               dist_cutoff, ctypes.c_void_p(d_id),
                                                               ctypes.c_void_p(d_score), ctypes.c_void_p(d_total)))
