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
