"""The command line end to end on the GPU: the reference's file formats in
and out, predictions compared with the reference's on the same files."""
import json
import os

import numpy as np
import pytest

from conftest import load_fixture
from whatprot_gb300 import cli, io
from whatprot_gb300.simulate import paper_model

pytestmark = pytest.mark.gpu


def _write_inputs(tmp_path, C, ds, rads):
    sm = paper_model(C)
    P = tmp_path / "seq-params.json"
    with open(P, "w") as f:
        json.dump(sm.to_json_dict(), f)
    S = tmp_path / "dye-seqs.tsv"
    io.write_dye_seqs(S, ds)
    R = tmp_path / "radiometries.tsv"
    io.write_radiometries(R, sm, rads)
    return sm, str(P), str(S), str(R)


def test_classify_hmm_matches_reference(tmp_path, capsys):
    z, ds = load_fixture("classify_c2_t8.npz")
    sm, P, S, R = _write_inputs(tmp_path, 2, ds, z["rads"])
    Y = str(tmp_path / "predictions.csv")
    assert cli.main(["classify", "hmm", "-P", P, "-S", S, "-R", R, "-Y", Y, "-p", "5"]) == 0
    out = capsys.readouterr().out
    for line in ("Read 100 dye seqs", "Finished basic setup", "Built classifier", "Finished classification",
                 "Finished saving results", "Total run time"):
        assert line in out
    ids, scores = io.read_predictions(Y)
    assert len(ids) == z["rads"].shape[0]
    assert np.mean(ids == z["ref_id"]) >= 0.98
    same = ids == z["ref_id"]
    ref_adj = z["ref_score"] / z["ref_total"]
    assert np.allclose(scores[same], ref_adj[same], rtol=1e-5)


def test_simulate_then_classify_nn_hybrid_and_fit(tmp_path, capsys):
    z, ds = load_fixture("classify_c2_t8.npz")
    sm, P, S, R0 = _write_inputs(tmp_path, 2, ds, z["rads"][:2])
    R = str(tmp_path / "sim-rads.tsv")
    Yt = str(tmp_path / "true-ids.tsv")
    assert cli.main(["simulate", "rad", "-P", P, "-t", "8", "-g", "300", "-S", S, "-R", R, "-Y", Yt]) == 0
    T, C, rads = io.read_radiometries(R, sm)
    true = io.read_true_ids(Yt)
    # undetectable reads (no dye at the first timestep) are dropped, as the reference does
    assert T == 8 and C == 2 and rads.shape[0] == len(true) and 150 <= len(true) < 300
    Tt = str(tmp_path / "dye-tracks.tsv")
    assert cli.main(["simulate", "dt", "-P", P, "-t", "8", "-g", "20", "-S", S, "-T", Tt]) == 0
    dts = io.read_dye_tracks(Tt)
    assert len(dts) > 0 and dts.tracks.shape[1:] == (8, 2)
    Yn = str(tmp_path / "nn.csv")
    assert cli.main(["classify", "nn", "-P", P, "-k", "50", "-s", "0.5", "-T", Tt, "-R", R, "-Y", Yn]) == 0
    ids, _ = io.read_predictions(Yn)
    assert len(ids) == len(true) and np.mean(ids == true) > 0.2
    Yh = str(tmp_path / "hybrid.csv")
    assert cli.main(["classify", "hybrid", "-P", P, "-k", "50", "-s", "0.5", "-H", "10", "-S", S, "-T", Tt,
                     "-R", R, "-Y", Yh, "-p", "5"]) == 0
    hid, _ = io.read_predictions(Yh)
    assert len(hid) == len(true) and np.mean(hid == true) > 0.2
    capsys.readouterr()
    fz = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fit_c2_t8.npz"))
    Rf = str(tmp_path / "fit-rads.tsv")
    io.write_radiometries(Rf, sm, fz["rads"])
    assert cli.main(["fit", "-P", P, "-L", "1e-4", "-x", str(fz["seq_str"]), "-R", Rf]) == 0
    out = capsys.readouterr().out
    assert "Parameters:" in out and "log(L): " in out and "Final step-size: " in out


def test_fit_with_emission_settings(tmp_path, capsys):
    """`fit -F settings.json` with "fit_emission": true (an extension) fits
    mu, sig and bg_sig too and prints them after the reference's parameter
    line; the reference's own settings keys still apply (a held rate stays
    at its start)."""
    sm = paper_model(2)
    P = tmp_path / "seq-params.json"
    with open(P, "w") as f:
        json.dump(sm.to_json_dict(), f)
    fz = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fit_c2_t8.npz"))
    Rf = str(tmp_path / "fit-rads.tsv")
    io.write_radiometries(Rf, sm, fz["rads"])
    F = tmp_path / "fit-settings.json"
    with open(F, "w") as f:
        json.dump({"hold_p_edman_failure": True, "fit_emission": True}, f)
    capsys.readouterr()
    assert cli.main(["fit", "-P", str(P), "-L", "1e-4", "-x", str(fz["seq_str"]), "-R", Rf, "-F", str(F)]) == 0
    out = capsys.readouterr().out
    assert "Channel 0 emission: (mu: " in out and "Channel 1 emission: (mu: " in out
    assert f"Edman failure rate: {sm.p_edman_failure:.6f}" in out
