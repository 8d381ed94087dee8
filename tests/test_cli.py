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
