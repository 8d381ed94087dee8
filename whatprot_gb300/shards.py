"""Reads sharded over GPUs (one process per GPU, torch.distributed).

Classification and the fit's E-step shard by reads with no exchange on the
data path: each rank classifies its own slice and the results are gathered
on the host; the fit adds the ranks' expected-count sums (one FP64
all-reduce per EM iteration) and every rank then takes the same M-step
(wp_fit_mstep, host code), so the models stay identical on all ranks.
Timings are reduced by max over ranks.  The same functions run over NCCL
(GPU tensors) or gloo (CPU tensors)."""
from __future__ import annotations

import ctypes
from typing import Callable, Optional, Sequence

import numpy as np


def shard_range(n: int, rank: int, world: int):
    """[lo, hi) of rank's contiguous share of n items (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def _device():
    import torch
    dist = _dist()
    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(x: float) -> float:
    """The largest x over all ranks (x itself without a process group)."""
    import torch
    dist = _dist()
    if dist is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v: np.ndarray) -> np.ndarray:
    """Element-wise FP64 sum over ranks."""
    import torch
    dist = _dist()
    if dist is None:
        return np.asarray(v, dtype=np.float64)
    t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def gather_rows(local: np.ndarray, n_total: int) -> np.ndarray:
    """Concatenate every rank's rows (rank order), on every rank."""
    import torch
    dist = _dist()
    if dist is None:
        return local
    world = dist.get_world_size()
    shape = local.shape[1:]
    sizes = [shard_range(n_total, r, world) for r in range(world)]
    maxn = max(hi - lo for lo, hi in sizes)
    pad = np.zeros((maxn,) + shape, dtype=local.dtype)
    pad[: local.shape[0]] = local
    t = torch.from_numpy(pad).to(_device())
    out = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(out, t)
    parts = [o.cpu().numpy()[: hi - lo] for o, (lo, hi) in zip(out, sizes)]
    return np.concatenate(parts, axis=0)


def sharded_classify(classify: Callable[[np.ndarray], Sequence[np.ndarray]], rads: np.ndarray, rank: int,
                     world: int):
    """Each rank classifies its slice of the reads with `classify` (returns
    per-read arrays); the per-read results of all ranks are gathered."""
    lo, hi = shard_range(rads.shape[0], rank, world)
    outs = classify(rads[lo:hi])
    return [gather_rows(np.asarray(o), rads.shape[0]) for o in outs]


# wp_fit_sums as a flat FP64 vector (the all-reduce unit)
def sums_to_vector(s) -> np.ndarray:
    v = [s.p_edman_failure_num, s.p_edman_failure_den]
    v += list(s.p_detach_x) + list(s.p_detach_n)
    v += [s.p_initial_block_num, s.p_initial_block_den, s.p_cyclic_block_num, s.p_cyclic_block_den]
    v += list(s.p_bleach_num) + list(s.p_bleach_den) + list(s.p_dud_num) + list(s.p_dud_den)
    return np.asarray(v, dtype=np.float64)


def vector_to_sums(v: np.ndarray):
    from .capi import WP_MAX_CHANNELS, WP_MAX_TIMESTEPS, WpFitSums
    s = WpFitSums()
    k = 0

    def take(n):
        nonlocal k
        out = v[k:k + n]
        k += n
        return out
    s.p_edman_failure_num, s.p_edman_failure_den = take(2)
    for i, x in enumerate(take(WP_MAX_TIMESTEPS)):
        s.p_detach_x[i] = x
    for i, x in enumerate(take(WP_MAX_TIMESTEPS)):
        s.p_detach_n[i] = x
    (s.p_initial_block_num, s.p_initial_block_den, s.p_cyclic_block_num, s.p_cyclic_block_den) = take(4)
    for name in ("p_bleach_num", "p_bleach_den", "p_dud_num", "p_dud_den"):
        arr = getattr(s, name)
        for i, x in enumerate(take(WP_MAX_CHANNELS)):
            arr[i] = x
    return s


def mstep(sums, num_channels: int, num_timesteps: int, dye_seq, num_reads: int, current,
          holds: Optional[dict] = None):
    """wp_fit_mstep: (next WpFitParams, step size)."""
    from .capi import WpError, WpFitParams, WpFitSettings, _ptr, load_library
    lib = load_library()
    seq = np.ascontiguousarray(dye_seq, dtype=np.int16)
    fs = WpFitSettings()
    for k, v in (holds or {}).items():
        if k in ("hold_p_bleach", "hold_p_dud"):
            arr = getattr(fs, k)
            for c, h in enumerate(v):
                arr[c] = 1 if h else 0
        else:
            setattr(fs, k, 1 if v else 0)
    nxt = WpFitParams()
    step = ctypes.c_double()
    st = lib.wp_fit_mstep(ctypes.byref(sums), num_channels, num_timesteps, _ptr(seq) if len(seq) else None,
                          len(seq), num_reads, ctypes.byref(current), ctypes.byref(fs), ctypes.byref(nxt),
                          ctypes.byref(step))
    if st != 0:
        raise WpError(st, "wp_fit_mstep")
    return nxt, step.value


def sharded_fit(estep: Callable[[object], object], start, num_channels: int, num_timesteps: int, dye_seq,
                num_reads_total: int, stopping_threshold: float, max_iterations: int = 10000,
                holds: Optional[dict] = None):
    """HMMFitter::fit over reads sharded across ranks: estep(params) returns
    this rank's wp_fit_sums for the current parameters; the sums are added
    over ranks and every rank takes the same M-step.  Returns (params, step,
    iterations)."""
    cur = start
    it = 0
    while True:
        local = sums_to_vector(estep(cur))
        total = vector_to_sums(sum_over_ranks(local))
        nxt, step = mstep(total, num_channels, num_timesteps, dye_seq, num_reads_total, cur, holds)
        it += 1
        if step < stopping_threshold or it >= max_iterations:
            return nxt, step, it
        cur = nxt
