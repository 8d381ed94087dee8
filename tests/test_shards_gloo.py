"""The multi-GPU path's host logic with two gloo ranks on the CPU: reads
sharded with no exchange on the data path (classification gathered on the
host), the fit's E-step sums added over ranks with every rank taking the
same M-step (wp_fit_mstep), timings reduced by max.  The per-rank compute is
the CPU oracle here (the GPU calls are the same functions with the CUDA
E-step and classifier plugged in)."""
import os
import socket

import numpy as np
import pytest

from whatprot_gb300 import shards

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _data():
    from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
    from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_radiometries
    sm = paper_model(2)
    ds = random_dye_seqs(15, 2, 6, 12, seed=3)
    rads, _ = simulate_radiometries(sm, ds, 8, 31, seed=4)  # odd count: uneven shards
    seq = parse_dye_seq("..0.1.0..1")
    one = DyeSeqSet(2, [seq], np.array([0], np.int32), np.array([1], np.int32))
    frads, _ = simulate_radiometries(sm, one, 8, 61, seed=5)
    return sm, ds, rads, seq, frads


def _to_wp_sums(o):
    from oracle_lib import oracle_sums_to_wp
    return oracle_sums_to_wp(o)


def _params_model(p, sm):
    import copy
    m = copy.deepcopy(sm)
    m.p_edman_failure, m.p_detach, m.p_initial_detach = p.p_edman_failure, p.p_detach, p.p_initial_detach
    m.p_initial_detach_decay, m.p_initial_block, m.p_cyclic_block = (p.p_initial_detach_decay, p.p_initial_block,
                                                                       p.p_cyclic_block)
    for c, cm in enumerate(m.channel_models):
        cm.p_bleach, cm.p_dud = p.p_bleach[c], p.p_dud[c]
    return m


def _start_params(sm):
    from whatprot_gb300.capi import WpFitParams
    p = WpFitParams()
    p.p_edman_failure, p.p_detach = sm.p_edman_failure * 1.3, sm.p_detach * 0.7
    for c, cm in enumerate(sm.channel_models):
        p.p_bleach[c], p.p_dud[c] = cm.p_bleach * 1.2, cm.p_dud * 0.8
    return p


def _run(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, HERE)
    import torch.distributed as dist
    from oracle_lib import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sm, ds, rads, seq, frads = _data()
    o = Oracle()
    ids, sc, tot = shards.sharded_classify(lambda x: o.classify(sm, 8, ds, x, 5.0, threads=1), rads, rank, world)
    lo, hi = shards.shard_range(frads.shape[0], rank, world)

    def estep(p):
        s, _ = o.improve_fit_batch(_params_model(p, sm), 8, seq, frads[lo:hi], threads=1)
        return _to_wp_sums(s)

    params, step, it = shards.sharded_fit(estep, _start_params(sm), 2, 8, seq, frads.shape[0], 1e-6)
    tmax = shards.max_over_ranks(float(rank + 1) * 1.5)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), ids=ids, sc=sc, tot=tot, tmax=tmax, it=it, step=step,
             fit=np.array([params.p_edman_failure, params.p_detach, params.p_initial_detach,
                           params.p_initial_detach_decay] + list(params.p_bleach[:2]) + list(params.p_dud[:2])))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_range_covers_everything():
    for n in (0, 1, 7, 31, 100):
        for world in (1, 2, 3, 8):
            parts = [shards.shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            assert max(h - l for l, h in parts) - min(h - l for l, h in parts) <= 1


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_run, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r = [np.load(tmp_path / f"rank{i}.npz") for i in range(world)]
    # single process, all reads
    import sys
    sys.path.insert(0, HERE)
    from oracle_lib import Oracle
    sm, ds, rads, seq, frads = _data()
    o = Oracle()
    ids, sc, tot = o.classify(sm, 8, ds, rads, 5.0, threads=1)
    for k in range(world):
        assert np.array_equal(r[k]["ids"], ids)
        assert np.array_equal(r[k]["sc"], sc) and np.array_equal(r[k]["tot"], tot)
        assert float(r[k]["tmax"]) == 3.0

    def estep(p):
        s, _ = o.improve_fit_batch(_params_model(p, sm), 8, seq, frads, threads=1)
        return _to_wp_sums(s)

    params, step, it = shards.sharded_fit(estep, _start_params(sm), 2, 8, seq, frads.shape[0], 1e-6)
    full = np.array([params.p_edman_failure, params.p_detach, params.p_initial_detach,
                     params.p_initial_detach_decay] + list(params.p_bleach[:2]) + list(params.p_dud[:2]))
    # both ranks took identical steps, equal to the single-process fit up to
    # the order of the FP64 additions of the shards' sums
    assert np.array_equal(r[0]["fit"], r[1]["fit"])
    assert np.allclose(r[0]["fit"], full, rtol=0, atol=1e-9)
    assert int(r[0]["it"]) == it
