"""The kd-tree the exact kNN selection replays (host build in the library,
wp_nn_kd_tree_order) against the reference's KDTree (oracle/_ref, where the
reference was compiled) and against the oracle's restatement: the same
permutation of the entries, including coordinates with many equal values
(the reference's nth_element moves the split around runs of equal
values)."""
import ctypes

import numpy as np
import pytest

from whatprot_gb300 import capi


class _Node(ctypes.Structure):
    _fields_ = [("leaf", ctypes.c_int), ("s", ctypes.c_int), ("begin", ctypes.c_int), ("end", ctypes.c_int),
                ("left", ctypes.c_int), ("right", ctypes.c_int), ("max_left", ctypes.c_double),
                ("min_right", ctypes.c_double), ("split", ctypes.c_double)]


class _Tree(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("D", ctypes.c_int), ("root", ctypes.c_int), ("num_nodes", ctypes.c_int),
                ("cap", ctypes.c_int), ("nodes", ctypes.POINTER(_Node)), ("pos", ctypes.POINTER(ctypes.c_int32))]


def _cases():
    rng = np.random.default_rng(17)
    out = []
    for trial in range(24):
        N = int(rng.integers(1, 4000))
        D = int(rng.integers(1, 20))
        k = int(rng.integers(1, 300))
        x = rng.integers(0, 4, size=(N, D)).astype(np.float64) * (1.0 if trial % 2 else 0.7)
        if trial % 3 == 0:
            x += rng.normal(size=(N, D))
        out.append((x, k))
    out.append((np.zeros((50, 4)), 3))           # every value equal
    out.append((np.arange(64.0).reshape(16, 4), 1))  # k = 1, distinct
    out.append((np.ones((7, 48)), 10))           # fewer entries than 2k: one leaf
    return out


def _oracle_order(oracle, x, k):
    L = oracle.lib
    L.wpo_kd_tree_build.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(_Tree)]
    L.wpo_kd_tree_free.argtypes = [ctypes.POINTER(_Tree)]
    t = _Tree()
    x = np.ascontiguousarray(x)
    L.wpo_kd_tree_build(x.ctypes.data, x.shape[0], x.shape[1], k, ctypes.byref(t))
    perm = np.array([t.pos[i] for i in range(x.shape[0])], np.int32)
    n = t.num_nodes
    L.wpo_kd_tree_free(ctypes.byref(t))
    return perm, n


@pytest.mark.parametrize("i", range(27))
def test_tree_order_matches_oracle(oracle, i):
    x, k = _cases()[i]
    perm, nodes = capi.kd_tree_order(x, k)
    operm, onodes = _oracle_order(oracle, x, k)
    assert np.array_equal(perm, operm)
    assert nodes == onodes


def test_tree_order_matches_reference(reference):
    L = reference.lib
    L.ref_kd_tree_order.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    for x, k in _cases():
        x = np.ascontiguousarray(x)
        rp = np.zeros(x.shape[0], np.int32)
        L.ref_kd_tree_order(x.ctypes.data, x.shape[0], x.shape[1], k, rp.ctypes.data)
        perm, _ = capi.kd_tree_order(x, k)
        assert np.array_equal(perm, rp)


def test_tree_order_rejects_bad_shapes():
    with pytest.raises(capi.WpError):
        capi.kd_tree_order(np.zeros((3, 65)), 2)
