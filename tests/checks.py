"""Comparison helpers shared by the parity tests.

Tolerances (the hot-path contract's): block pattern bit-exact; K per scalar row within
1e-12 x the largest |entry| of that row, penalty entries exactly 1e20; M and F within
1e-12 x their largest |entry|; stresses per node within 1e-10 x the node's largest |value|.
"""
import numpy as np

REL_K = 1e-12
REL_S = 1e-10


def assert_K_close(Kg, Ko, rel=REL_K):
    assert Kg.shape == Ko.shape
    assert np.array_equal(Kg.indptr, Ko.indptr), "row pointers differ"
    assert np.array_equal(Kg.indices, Ko.indices), "column indices differ"
    pen = Ko.data >= 1e19
    assert np.array_equal(Kg.data[pen], Ko.data[pen])
    assert np.all(Kg.data[Kg.data >= 1e19] == 1e20)
    a = np.where(pen, 0.0, Kg.data)
    b = np.where(pen, 0.0, Ko.data)
    rows = np.repeat(np.arange(Ko.shape[0]), np.diff(Ko.indptr))
    rmax = np.zeros(Ko.shape[0])
    np.maximum.at(rmax, rows, np.abs(b))
    dev = np.abs(a - b)
    assert np.all(dev <= rel * rmax[rows]), f"max rel dev {np.max(dev / np.maximum(rmax[rows], 1e-300))}"


def assert_vec_close(x, y, rel=REL_K):
    s = np.abs(y).max()
    assert np.abs(np.asarray(x) - np.asarray(y)).max() <= rel * s


def assert_stress_close(S, So, rel=REL_S):
    assert S.shape == So.shape
    fin = np.isfinite(So)
    assert np.array_equal(np.isfinite(S), fin), "NaN / Inf positions differ"
    So0, S0 = np.where(fin, So, 0.0), np.where(fin, S, 0.0)
    sc = np.abs(So0).max(axis=1, keepdims=True)
    dev = np.abs(S0 - So0)
    assert np.all(dev <= rel * sc), f"max rel dev {np.max(dev / np.maximum(sc, 1e-300))}"


def assert_rows_close(y, y_ref, scale, rel=REL_K):
    """Linear-functional check: |y - y_ref| <= rel * scale per entry (scale = |A|.|v|)."""
    dev = np.abs(np.asarray(y) - np.asarray(y_ref))
    assert np.all(dev <= rel * np.asarray(scale)), f"max rel dev {np.max(dev / np.maximum(scale, 1e-300))}"
