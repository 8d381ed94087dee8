import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

GOLDEN = os.path.join(HERE, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle_lib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle_lib import Reference
    if not Reference.available():
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    return Reference()


@pytest.fixture(scope="session")
def goldens():
    with open(os.path.join(GOLDEN, "peptide_hmm_goldens.json")) as f:
        return json.load(f)


def load_fixture(name):
    from whatprot_gb300.model import DyeSeqSet
    z = np.load(os.path.join(GOLDEN, name))
    off = z["offsets"]
    seqs = [z["seqs"][off[i]:off[i + 1]].astype(np.int16) for i in range(len(off) - 1)]
    ds = DyeSeqSet(int(z["C"]), seqs, z["ids"].astype(np.int32), z["counts"].astype(np.int32))
    return z, ds


@pytest.fixture(scope="session")
def gpu_ctx():
    import torch  # noqa: F401  (device present check below)
    from whatprot_gb300 import capi
    ctx = capi.Context(0)
    yield ctx
    ctx.close()


def nn_lists_match(ids_a, sc_a, na, ids_b, sc_b, nb, rel):
    """Two kNN top-h lists (ids and scores, ascending) name the same
    candidates: the same number, scores equal to `rel` (of the largest),
    and the same ids except among those scoring the list's smallest score,
    where the reference's heap keeps an unspecified subset of equal scores
    when more tie than fit in h.  Returns (match, boundary_tie)."""
    if na != nb:
        return False, False
    if na == 0:
        return True, False
    a, b = np.asarray(sc_a[:na], np.float64), np.asarray(sc_b[:nb], np.float64)
    sa, sb = np.sort(a), np.sort(b)
    tol = rel * max(abs(sa[-1]), abs(sb[-1])) + 1e-300
    if np.any(np.abs(sa - sb) > tol):
        return False, False
    lo = sa[0]
    ia = {int(i) for i, v in zip(ids_a[:na], a) if v > lo + tol}
    ib = {int(i) for i, v in zip(ids_b[:nb], b) if v > lo + tol}
    if ia != ib:
        return False, False
    tie = {int(i) for i in ids_a[:na]} != {int(i) for i in ids_b[:nb]}
    return True, tie
