"""The radiometry converter (python/convert_radiometries.py behaviour): a
radmat in .npy or .tsv becomes a radiometry TSV the readers accept, mocks
dropped, cycle-major, optional range filter."""
import numpy as np

from whatprot_gb300 import io
from whatprot_gb300.convert import convert_radiometries
from whatprot_gb300.simulate import paper_model


def test_npy_and_tsv_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    R, C, M, N = 7, 2, 1, 5
    radmat = rng.normal(1.0, 0.3, size=(R, C, M + N))
    np.save(tmp_path / "r.npy", radmat)
    np.savetxt(tmp_path / "r.tsv", radmat.reshape(R, -1), delimiter="\t")
    for src in ("r.npy", "r.tsv"):
        out = tmp_path / (src + ".out.tsv")
        assert convert_radiometries(C, M, N, str(tmp_path / src), str(out)) == R
        lines = open(out).read().splitlines()
        assert lines[:3] == [str(N), str(C), str(R)]
        assert all(line.startswith("\t") for line in lines[3:])  # mock cycles: leading tab, as the reference
        T, C2, rads = io.read_radiometries(out, paper_model(C))  # mu = 1
        assert (T, C2) == (N, C)
        assert np.allclose(rads, np.transpose(radmat[:, :, M:], (0, 2, 1)))


def test_range_filter(tmp_path):
    radmat = np.array([[[0.5, 1.5], [0.2, 0.3]], [[0.5, 9.0], [0.2, 0.3]]])  # read 1 has 9.0 out of range
    np.save(tmp_path / "r.npy", radmat)
    n = convert_radiometries(2, 0, 2, str(tmp_path / "r.npy"), str(tmp_path / "o.tsv"),
                             ranges_by_channel=[[(0.0, 2.0)], [(0.0, 1.0)]])
    assert n == 1
    assert open(tmp_path / "o.tsv").read().splitlines()[3] == "0.5\t0.2\t1.5\t0.3"
