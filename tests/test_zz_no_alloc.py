"""The allocation-free classify entry point (wp_hmm_classify_noalloc).

It serves callers that cannot call cudaMalloc -- an acquisition loop that
may not stall the device with an allocation, or a host that runs the library
under a memory budget it does not own.  It keeps everything in one fixed
device array that all calls share, so this test calls it twice in a row
through the C ABI and checks both results against wp_hmm_classify on the
same inputs (ids identical; score and total each within 1e-5 relative, and
finite) and against the oracle's FP64 classify (top-1 identical, adjusted
score within 1e-5 relative, the tolerance the other parity tests use).  It lives in its own file, collected last,
so that a run stopping at its failure has run everything else first."""
import ctypes

import numpy as np
import pytest

from whatprot_gb300 import capi
from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_radiometries

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.wp_hmm_classify_noalloc
    V = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.POINTER(capi.WpSeqModel), ctypes.c_int, V, V, V, V, ctypes.c_int,
                  V, ctypes.c_int, ctypes.c_double, V, V, V]
    f.restype = ctypes.c_int
    return f


def _model_struct(sm):
    C = sm.num_channels
    arr = lambda xs: np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
    cms = sm.channel_models
    keep = [arr([c.p_bleach for c in cms]), arr([c.p_dud for c in cms]), arr([c.bg_sig for c in cms]),
            arr([c.mu for c in cms]), arr([c.sig for c in cms]),
            arr([[c.interactions[o] for o in range(C)] for c in cms]).reshape(-1),
            arr([[c.flat_interactions[o] for o in range(C)] for c in cms]).reshape(-1)]
    m = capi.WpSeqModel(C, sm.p_edman_failure, sm.p_detach, sm.p_initial_detach, sm.p_initial_detach_decay,
                        sm.p_initial_block, sm.p_cyclic_block, *[k.ctypes.data for k in keep])
    return m, keep


@pytest.mark.parametrize("block", [False, True])
def test_noalloc_matches_classify_twice(block):
    sm = paper_model(3)
    if block:
        sm.p_initial_block, sm.p_cyclic_block = 0.05, 0.02
    T = 12
    ds = random_dye_seqs(70, 3, 8, 24, max_per_channel=5, min_total=1, seed=31 + block)
    rads, _ = simulate_radiometries(sm, ds, T, 60, seed=32 + block)
    R = rads.shape[0]
    ctx = capi.Context(0)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    want_id, want_sc, want_tot, _ = ctx.classify(rads, 5.0)
    ctx.close()
    from oracle_lib import Oracle
    oracle = Oracle()
    o_id, o_sc, o_tot = oracle.classify(sm, T, ds, rads, 5.0, threads=4)
    # a different top-1 is accepted only for an HMM tie (oracle log P of
    # both peptides equal within 1e-5)
    index = {int(i): k for k, i in enumerate(ds.ids)}
    diff = np.nonzero(want_id != o_id)[0]
    if diff.size:
        ll = oracle.loglik_all(sm, T, ds, rads[diff], 5.0, threads=4)
        for j, r in enumerate(diff):
            assert abs(ll[j, index[int(want_id[r])]] - ll[j, index[int(o_id[r])]]) <= 1e-5, r

    f = _bind(capi.load_library())
    m, keep = _model_struct(sm)
    flat, off = ds.ragged()
    ids = np.ascontiguousarray(ds.ids, np.int32)
    counts = np.ascontiguousarray(ds.counts, np.int32)
    r = np.ascontiguousarray(rads, np.float64)
    for call in range(2):
        oid = np.full(R, -7, np.int32)
        osc = np.full(R, np.nan)
        otot = np.full(R, np.nan)
        st = f(0, ctypes.byref(m), T, flat.ctypes.data, off.ctypes.data, ids.ctypes.data, counts.ctypes.data,
               len(ds), r.ctypes.data, R, 5.0, oid.ctypes.data, osc.ctypes.data, otot.ctypes.data)
        assert st == 0, (call, st)
        assert np.array_equal(oid, want_id), call
        assert np.all(np.isfinite(osc)) and np.all(np.isfinite(otot)), call
        np.testing.assert_allclose(osc, want_sc, rtol=1e-5, atol=0)
        np.testing.assert_allclose(otot, want_tot, rtol=1e-5, atol=0)
        np.testing.assert_allclose(osc / otot, o_sc / o_tot, rtol=1e-5, atol=0)


def test_noalloc_rejects_oversized():
    f = _bind(capi.load_library())
    sm = paper_model(2)
    m, keep = _model_struct(sm)
    ds = random_dye_seqs(2000, 2, 6, 12, seed=3)
    flat, off = ds.ragged()
    R = 4000  # 8 million pairs: beyond the fixed array
    rads = np.zeros((R, 8, 2))
    out = [np.zeros(R, np.int32), np.zeros(R), np.zeros(R)]
    st = f(0, ctypes.byref(m), 8, flat.ctypes.data, off.ctypes.data, ds.ids.ctypes.data,
           ds.counts.ctypes.data, len(ds), rads.ctypes.data, R, 5.0, *[o.ctypes.data for o in out])
    assert st == 5  # WP_ERR_UNSUPPORTED
