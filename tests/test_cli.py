"""The command line's validation (main/main.cc:218-480): every invalid
combination prints INCORRECT USAGE and exits 1 (no GPU needed)."""
import pytest

from whatprot_gb300 import cli

BAD = [
    [],
    ["classify"],
    ["classify", "hmm"],
    ["classify", "hmm", "-P", "a", "-S", "b", "-R", "c"],                       # no -Y
    ["classify", "hmm", "-P", "a", "-S", "b", "-R", "c", "-Y", "d", "-k", "3"],  # extra option
    ["classify", "hybrid", "-P", "a", "-S", "b", "-R", "c", "-Y", "d", "-k", "3", "-s", "0.5"],  # no -H -T
    ["classify", "nn", "-P", "a", "-T", "b", "-R", "c", "-Y", "d", "-k", "3"],    # no -s
    ["classify", "svm", "-P", "a"],
    ["fit", "-P", "a", "-L", "0.1", "-x", "..0", "-R", "r", "-b", "3"],           # -b without -c
    ["fit", "-P", "a", "-L", "0.1", "-x", "..0"],                                  # no -R
    ["fit", "extra", "-P", "a", "-L", "0.1", "-x", "..0", "-R", "r"],
    ["fit", "-P", "a", "-L", "0.1", "-x", "..0", "-R", "r", "-Y", "out"],          # -Y only with -b -c
    ["simulate", "rad", "-P", "a", "-t", "8", "-g", "10", "-S", "s", "-R", "r"],  # no -Y
    ["simulate", "dt", "-P", "a", "-t", "8", "-g", "10", "-S", "s"],              # no -T
    ["simulate", "xyz"],
    ["frobnicate"],
]


@pytest.mark.parametrize("argv", BAD, ids=[" ".join(a) or "empty" for a in BAD])
def test_incorrect_usage(argv, capsys):
    assert cli.main(argv) == 1
    assert "INCORRECT USAGE" in capsys.readouterr().out


def test_help(capsys):
    assert cli.main(["--help"]) == 0
    assert "MODE is one of classify, fit, or simulate" in capsys.readouterr().out


def test_option_forms():
    opts, pos, _ = cli.parse(["classify", "hmm", "-P", "p.json", "--dyeseqs=s.tsv", "-Rr.tsv", "--results", "y",
                              "-p", "5"])
    assert pos == ["classify", "hmm"]
    assert opts == {"seqparams": "p.json", "dyeseqs": "s.tsv", "radiometries": "r.tsv", "results": "y",
                    "hmmprune": 5.0}


def test_dye_seq_file_round_trip_with_an_empty_dye_seq(tmp_path):
    import numpy as np
    from whatprot_gb300 import io
    from whatprot_gb300.model import DyeSeqSet, parse_dye_seq
    ds = DyeSeqSet(2, [parse_dye_seq("..0.1"), parse_dye_seq("...."), parse_dye_seq("1")],
                   np.array([4, 5, 6], np.int32), np.array([1, 2, 3], np.int32))
    io.write_dye_seqs(tmp_path / "d.tsv", ds)
    back = io.read_dye_seqs(tmp_path / "d.tsv")
    assert [list(s) for s in back.seqs] == [list(s) for s in ds.seqs]
    assert np.array_equal(back.ids, ds.ids) and np.array_equal(back.counts, ds.counts)
