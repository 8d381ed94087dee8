"""The C++ drop-in classes (whatprot_gb300/cpp/whatprot_gpu.h): whatprot's
HMMClassifier, NNClassifier, HybridClassifier and HMMFitter signatures over
the C ABI.

tests/cpp/dropin_driver.cc is compiled here with g++ against the library's
own data types and libwhatprot_gb300.so, and driven as whatprot's
run-classify-*.cc / run-fit.cc drive the CPU classes, on the committed
fixtures recorded from the compiled reference:
  * its results equal the Python mirror's (both are the same C ABI calls);
  * against the reference's recorded outputs with the tolerances of the
    other reference-fixture tests: top-1 ids equal except HMM ties (oracle
    log P equal to 1e-5), adjusted scores within 1e-5 relative (hybrid:
    reads without a kNN tie at the h-th place), the kNN best score and
    total within 1e-5, the fit's rates within 1e-4.
The CPU test beside it (test_cpp_dropin_build.py) compiles the same files
against whatprot's own headers."""
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_fixture
from oracle_lib import DBL_MAX

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from whatprot_gb300 import capi
    capi.load_library()
    libdir = os.path.dirname(capi.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_driver")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(REPO, "whatprot_gb300", "cpp"),
           os.path.join(HERE, "cpp", "dropin_driver.cc"), os.path.join(REPO, "whatprot_gb300", "cpp", "whatprot_gpu.cc"),
           "-L", libdir, "-lwhatprot_gb300", f"-Wl,-rpath,{libdir}", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def _fmt(x):
    return "max" if x >= DBL_MAX else repr(float(x))


def _write_input(path, sm, T, cutoff, ds, rads, dts=None, k=0, sig=0.0, h=0, fit=None):
    C = sm.num_channels
    out = [f"{C} {T} {_fmt(cutoff)}",
           " ".join(repr(float(v)) for v in (sm.p_edman_failure, sm.p_detach, sm.p_initial_detach,
                                             sm.p_initial_detach_decay, sm.p_initial_block, sm.p_cyclic_block))]
    for cm in sm.channel_models:
        out.append(" ".join(repr(float(v)) for v in (cm.p_bleach, cm.p_dud, cm.bg_sig, cm.mu, cm.sig)))
    strs = ds.strings() if ds is not None else []
    out.append(str(len(strs)))
    for i, s in enumerate(strs):
        out.append(f"{int(ds.ids[i])} {int(ds.counts[i])} {s if s else '-'}")
    if dts is None:
        out.append("0")
    else:
        out.append(str(len(dts)))
        for e in range(len(dts)):
            a, b = int(dts.src_off[e]), int(dts.src_off[e + 1])
            src = " ".join(f"{int(dts.src_id[j])} {int(dts.src_count[j])} {int(dts.src_hits[j])}" for j in range(a, b))
            out.append(" ".join(str(int(v)) for v in dts.tracks[e].reshape(-1)) + f" {b - a} {src}")
    out.append(f"{k} {sig!r} {h}")
    out.append(str(rads.shape[0]))
    for r in rads:
        out.append(" ".join(repr(float(v)) for v in r.reshape(-1)))
    if fit is not None:
        out.append(f"{fit[0]!r} {fit[1] if fit[1] else '-'}")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def _run(driver, mode, path):
    r = subprocess.run([driver, mode, str(path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip().splitlines()


def _scored(lines):
    ids = np.array([int(l.split()[0]) for l in lines], np.int32)
    sc = np.array([float(l.split()[1]) for l in lines])
    tot = np.array([float(l.split()[2]) for l in lines])
    return ids, sc, tot


@pytest.mark.parametrize("name", ["classify_c3_t16.npz", "classify_c2_t6_block_nocut.npz"])
def test_hmm_classifier_dropin(driver, tmp_path, gpu_ctx, oracle, name):
    from test_gpu_forward import _model, _tie_ok
    z, ds = load_fixture(name)
    C, T = int(z["C"]), int(z["T"])
    sm = _model(C, block=bool(z["block"]), detach_decay=bool(z["block"]))
    cut = DBL_MAX if np.isnan(z["cutoff"]) else float(z["cutoff"])
    _write_input(tmp_path / "in.txt", sm, T, cut, ds, z["rads"])
    ids, sc, tot = _scored(_run(driver, "hmm", tmp_path / "in.txt"))
    # the Python mirror's results (the same C ABI call)
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    pid, psc, ptot, _ = gpu_ctx.classify(z["rads"], cut)
    assert np.array_equal(ids, pid)
    np.testing.assert_allclose(sc, psc, rtol=1e-15, atol=0)
    np.testing.assert_allclose(tot, ptot, rtol=1e-15, atol=0)
    # the reference's recorded outputs
    mism = np.nonzero(ids != z["ref_id"])[0]
    if len(mism):
        allp = np.exp(oracle.loglik_all(sm, T, ds, z["rads"][mism], cut, threads=8))
        for k, i in enumerate(mism):
            assert _tie_ok(allp, k), f"read {i}: drop-in {ids[i]} reference {z['ref_id'][i]}"
    np.testing.assert_allclose(sc / tot, z["ref_score"] / z["ref_total"], rtol=1e-5, atol=1e-300)


def test_nn_and_hybrid_classifier_dropin(driver, tmp_path, gpu_ctx, oracle):
    from test_gpu_nn import _compare
    from test_oracle import nn_fixture_inputs
    z, ds, dts, sm = nn_fixture_inputs(oracle, "nn_c2_t8.npz")
    T = int(z["T"])
    k, sig, h, cut = int(z["k"]), float(z["sig"]), int(z["h"]), float(z["cutoff"])
    rads = z["rads"]
    _write_input(tmp_path / "in.txt", sm, T, cut, ds, rads, dts, k, sig, h)
    nid, nsc, ntot = _scored(_run(driver, "nn", tmp_path / "in.txt"))
    hid, hsc, htot = _scored(_run(driver, "hybrid", tmp_path / "in.txt"))
    # the Python mirror
    gpu_ctx.upload_model(sm, T)
    gpu_ctx.upload_peptides(ds)
    gpu_ctx.upload_tracks(dts)
    gpu_ctx.set_nn_selection("kdtree")
    pid, psc, ptot = gpu_ctx.hybrid_classify(rads, k, sig, h, cut)
    assert np.array_equal(hid, pid)
    np.testing.assert_allclose(hsc, psc, rtol=1e-15, atol=0)
    np.testing.assert_allclose(htot, ptot, rtol=1e-15, atol=0)
    # NNClassifier::classify(vector): the best kNN score and the total of
    # the reference; the id wherever the best score is not tied
    np.testing.assert_allclose(nsc, z["nn_best_score"], rtol=1e-5, atol=1e-300)
    np.testing.assert_allclose(ntot, z["nn_best_total"], rtol=1e-5, atol=1e-300)
    for r in range(len(nid)):
        if nid[r] != z["nn_best_id"][r]:
            sc_r = z["nn_scores"][r, :z["nn_ncand"][r]]
            assert np.sum(np.abs(sc_r - nsc[r]) <= 1e-5 * nsc[r]) >= 2, (r, nid[r], z["nn_best_id"][r])
    # HybridClassifier::classify(vector) against the reference: ids equal
    # except HMM ties, adjusted scores within 1e-5, on every read whose kNN
    # candidate list is not cut inside a tie at the h-th place (there the
    # kept candidate, and so the subfraction, is the heap's choice)
    h_ties = _compare(gpu_ctx.nn_classify(rads, k, sig, h),
                      (z["nn_ncand"], z["nn_ids"], z["nn_scores"], z["nn_total"]), "reference nn_c2_t8", "kdtree")
    index = {int(i): n for n, i in enumerate(ds.ids)}
    ties = 0
    for r in range(len(hid)):
        if r in h_ties:
            continue
        if hid[r] != z["hy_id"][r]:
            ll = oracle.loglik_all(sm, T, ds, rads[r:r + 1], cut)[0]
            a, b = index[int(hid[r])], index[int(z["hy_id"][r])]
            assert abs(ll[a] - ll[b]) <= 1e-5, (r, hid[r], z["hy_id"][r])
            ties += 1
        adj, ref = hsc[r] / htot[r], z["hy_score"][r] / z["hy_total"][r]
        assert abs(adj - ref) <= 1e-5 * abs(ref) + 1e-300, (r, adj, ref)
    assert ties <= 0.05 * len(hid)


def test_hmm_fitter_dropin(driver, tmp_path):
    from whatprot_gb300.simulate import paper_model
    z = np.load(os.path.join(GOLDEN, "fit_c2_t8.npz"))
    C, T = int(z["C"]), int(z["T"])
    st = z["start"]
    sm = paper_model(C)
    (sm.p_edman_failure, sm.p_detach, sm.p_initial_detach, sm.p_initial_detach_decay,
     sm.p_initial_block, sm.p_cyclic_block) = st[:6]
    for c in range(C):
        sm.channel_models[c].p_bleach = st[6 + c]
        sm.channel_models[c].p_dud = st[6 + C + c]
    _write_input(tmp_path / "in.txt", sm, T, DBL_MAX, None, z["rads"], fit=(float(z["threshold"]), str(z["seq_str"])))
    lines = _run(driver, "fit", tmp_path / "in.txt")
    vals = np.array([float(v) for v in lines[0].split()])
    got, log_l, step = vals[:6 + 2 * C], vals[6 + 2 * C], vals[7 + 2 * C]
    ref = z["ref_params"]
    assert step < float(z["threshold"])
    keep = [0, 4, 5] + list(range(6, 6 + 2 * C))
    assert np.max(np.abs(got[keep] - ref[keep])) <= 1e-4, (got, ref)
    curve = lambda p: np.array([p[1] + p[2] * math.exp(-t * p[3]) for t in range(T)])
    assert np.max(np.abs(curve(got) - curve(ref))) <= 1e-4, (got, ref)
    assert abs(log_l - float(z["ref_log_l"])) <= 1e-6 * abs(float(z["ref_log_l"])) + 1e-3
    # HMMFitter::log_likelihood of the fitted model agrees with fit's value
    ll2 = float(lines[1].split()[1])
    assert abs(ll2 - log_l) <= 1e-6 * abs(log_l)
