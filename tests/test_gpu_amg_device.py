"""Multigrid setup on the device (fem_amg_setup_device) against the host setup
(fem_amg_setup) of the same matrix: the same hierarchy, bit for bit.

Both setups run the same sequence of IEEE operations (no multiply-add contraction on either
side, every sum in the host's order), so every exported array is compared for exact
equality: aggregates, Dirichlet flags, Lanczos estimates, inverse diagonal blocks, P, R and the
coarse operators (patterns and values), and the dense coarsest inverse.  A solve
preconditioned by either hierarchy then takes the same iterations and matches SuperLU to 1e-8.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import fem_taichi_gb300 as F
from tests.fixtures import STEEL

pytestmark = pytest.mark.gpu


def _systems():
    slab = F.hex_block(40, 8, 4, size=(40.0, 4.0, 1.0), jitter=0.05, twist_deg=45, seed=3, fix="xmin",
                       load_face="xmax", load=(0, 0, -1.0))
    block = F.hex_block(14, 12, 10, jitter=0.12, seed=5, fix="zmin", load_face="zmax", load=(0.3, 0, -1.0))
    return {"slab": slab, "block": block}


@pytest.fixture(scope="module", params=["slab", "block"])
def pair(request):
    P = _systems()[request.param]
    M = F.Model(request.param, P, STEEL)
    S = F.DeviceSystem(M)
    Hd = S.amg_variant(setup="device", max_coarse=200)
    Hh = S.amg_variant(setup="host", max_coarse=200)
    yield P, M, S, Hd, Hh
    Hd.close()
    Hh.close()


def test_device_setup_is_bit_identical_to_the_host_setup(pair):
    P, M, S, Hd, Hh = pair
    ld, lh = Hd.levels(), Hh.levels()
    assert [(l["n"], l["b"], l["nnzb_A"], l["nnzb_P"]) for l in ld] == \
        [(l["n"], l["b"], l["nnzb_A"], l["nnzb_P"]) for l in lh]
    assert len(ld) >= 3
    for l, (a, b) in enumerate(zip(ld, lh)):
        assert a["lmax"] == b["lmax"] and a["omega"] == b["omega"], l
        if l + 1 < len(ld):
            assert np.array_equal(Hd.export(l, 4), Hh.export(l, 4)), l
            assert np.array_equal(Hd.export(l, 6), Hh.export(l, 6)), l
        assert np.array_equal(Hd.export(l, 3), Hh.export(l, 3)), l
        for what in ((0, 1, 2) if l + 1 < len(ld) else (0,)):
            if what == 0 and l == 0:
                continue
            for x, y in zip(Hd.export(l, what), Hh.export(l, what)):
                assert np.array_equal(x, y), (l, what)
    assert np.array_equal(Hd.export(len(ld) - 1, 5), Hh.export(len(lh) - 1, 5))


def test_device_hierarchy_solves_like_the_host_hierarchy(pair):
    """Both hierarchies precondition the FP64 solve to the same iteration count, and both
    reach SuperLU's solution to 1e-8 when refined on compensated residuals."""
    P, M, S, Hd, Hh = pair
    K, Fv = M.Get_MatrixKL(), M.Get_VectorF()
    Ur = spla.splu(K.tocsc()).solve(Fv)
    its = {}
    for name, H in (("device", Hd), ("host", Hh)):
        _, st = S.solve(rtol=1e-7, mixed=False, precond=H)
        assert st["status"] == 0, (name, st)
        its[name] = st["iterations"]
        U, st = S.solve(rtol=1e-9, mixed=False, precond=H, residual="extra")
        U = U.cpu().numpy().reshape(-1)
        assert np.linalg.norm(U - Ur) <= 1e-8 * np.linalg.norm(Ur), name
    assert its["device"] == its["host"], its


def _exports(H):
    out = []
    info = H.levels()
    for l, inf in enumerate(info):
        out.append(("lmax", l, inf["lmax"], inf["n"], inf["b"], inf["nnzb_A"], inf["nnzb_P"]))
        out.append(("dinv", l, H.export(l, 3)))
        if l > 0:
            out.append(("A", l) + tuple(H.export(l, 0)))
        if l + 1 < len(info):
            out += [("agg", l, H.export(l, 4)), ("iso", l, H.export(l, 6))]
            out += [("P", l) + tuple(H.export(l, 1)), ("R", l) + tuple(H.export(l, 2))]
    out.append(("coarse", H.export(len(info) - 1, 5)))
    return out


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert len(x) == len(y) and x[0] == y[0], (x[0], y[0])
        for u, v in zip(x[1:], y[1:]):
            if isinstance(u, np.ndarray):
                assert np.array_equal(u, v), x[:2]
            else:
                assert u == v, x[:2]


@pytest.mark.parametrize("case", ["unsmoothed", "single_dense_level", "all_penalised", "theta0_two_levels"])
def test_device_setup_edge_cases_bit_identical(case):
    """Options and shapes off the main path, device vs host setup, every array exactly equal:
    P = T (smooth = 0), a system small enough to be one dense level, a mesh whose every node
    is penalised (no aggregate: one dense level), and theta = 0 with a two-level cap."""
    if case == "all_penalised":
        from fem_taichi_gb300.mesh import block_arrays
        b = block_arrays(3, 3, 2, jitter=0.1, seed=2, fix=None)
        P = F.Physics(b["ids"], b["xyz"], b["elem"], [[np.arange(b["xyz"].shape[0]), [0, 0, 0]]], [], name="fixed")
    else:
        P = F.hex_block(10, 8, 6, jitter=0.1, seed=7, fix="zmin", load_face="zmax", load=(0, 0, -1.0))
    opts = {"unsmoothed": dict(smooth=0, max_coarse=60), "single_dense_level": dict(max_coarse=100000),
            "all_penalised": dict(max_coarse=10), "theta0_two_levels": dict(theta=0.0, max_levels=2,
                                                                           max_coarse=10)}[case]
    S = F.DeviceSystem(F.Model(case, P, STEEL))
    Hd = S.amg_variant(setup="device", **opts)
    Hh = S.amg_variant(setup="host", **opts)
    try:
        if case in ("single_dense_level", "all_penalised"):
            assert len(Hd.levels()) == 1
        else:
            assert len(Hd.levels()) >= 2
        _same(_exports(Hd), _exports(Hh))
    finally:
        Hd.close()
        Hh.close()


def test_device_setup_without_a_host_pattern(pair):
    """The level-0 pattern downloaded by the setup itself (no host copy given) builds the same
    hierarchy bit for bit."""
    P, M, S, Hd, Hh = pair
    from fem_taichi_gb300.solve import AmgHierarchy
    Hn = AmgHierarchy.on_device(S, host_pattern=False, max_coarse=200)
    try:
        _same(_exports(Hn), _exports(Hd))
    finally:
        Hn.close()
