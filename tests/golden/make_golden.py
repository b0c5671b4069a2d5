"""Regenerates the committed fixtures under tests/golden/ (run in a checkout that has the
reference tree; it is not needed at test time).

mesh2.npz        -- the reference's only mesh fixture, Mesh/2.cdb, parsed the way
                    READ_physics.py:64-97 does (NBLOCK/EBLOCK text, '-' -> ' -' token
                    split, 18 tokens per element row, ids - 1), plus the node ids of
                    Boundary/2_bot_in.lis and 2_bot_out.lis (READ_physics.py:99-117).
mesh2_golden.npz -- oracle outputs on that mesh (steel, Omegas=(0,0,100), both bot
                    files fixed, no top file): pattern digests, seeded samples of K, M, F
                    and of the stress table for a seeded displacement field.  They pin
                    the oracle across machines; the reference itself cannot run here.

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
"""
from __future__ import annotations

import hashlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def parse_cdb_like_reference(path):
    with open(path, "r", errors="replace") as f:
        lines = [s for s in f.read().splitlines() if s.strip() != ""]
    # pandas read_csv(sep='\t') makes the first line a header and skips blank lines
    body = lines[1:]
    n_sta = next(i for i, s in enumerate(body) if "NBLOCK" in s) + 2
    n_end = next(i for i, s in enumerate(body) if "N,R5" in s)
    e_sta = next(i for i, s in enumerate(body) if "EBLOCK" in s) + 2
    e_end = next(i for i, s in enumerate(body) if re.match(r"\s*-1", s))
    toks = " ".join(s.replace("-", " -").replace("E -", "E-") for s in body[n_sta:n_end]).split()
    node = np.array(toks, dtype=np.float64).reshape(-1, 6)
    etoks = " ".join(body[e_sta:e_end]).split()
    elem = np.array(etoks, dtype=np.int64).reshape(-1, 18)
    return node.T, elem.T - 1


def parse_lis_like_reference(path):
    with open(path, "r", errors="replace") as f:
        lines = [s for s in f.read().splitlines() if s.strip() != ""]
    keep = [s for s in lines[1:] if not re.search("NAME|NODE|LIST", s)]
    return np.array(" ".join(keep).split(), dtype=np.int64)


def main(ref_root):
    Node, Elem = parse_cdb_like_reference(os.path.join(ref_root, "Mesh", "2.cdb"))
    bot_in = parse_lis_like_reference(os.path.join(ref_root, "Boundary", "2_bot_in.lis"))
    bot_out = parse_lis_like_reference(os.path.join(ref_root, "Boundary", "2_bot_out.lis"))
    np.savez_compressed(os.path.join(HERE, "mesh2.npz"), node_ids=Node[0].astype(np.int32),
                        xyz=np.ascontiguousarray(Node[3:6].T), elem=Elem[-8:].astype(np.int32),
                        bot_in=bot_in.astype(np.int32), bot_out=bot_out.astype(np.int32))

    from oracle import fem_oracle as O
    from tests.fixtures import mesh2_physics
    P = mesh2_physics()
    mat = {'DE': 7.8e-9, 'EX': 200000.0, 'PO': 0.3}
    topo = O.pre_process(P.Node, P.Elem)
    OM = O.OracleModel(P, mat, (0, 0, 100))
    K = OM.Get_MatrixKL()
    M = OM.Get_MatrixM()
    F = OM.Get_VectorF()
    rng = np.random.default_rng(20240601)
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
    S = O.oracle_stress(P, mat, u, gmat_mode="written")
    Sa = O.oracle_stress(P, mat, u, gmat_mode="aliased")
    ks = rng.choice(K.nnz, size=4096, replace=False)
    ms = rng.choice(M.nnz, size=1024, replace=False)
    ns = rng.choice(P.Num_Node, size=512, replace=False)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()  # noqa: E731
    Kc = K.tocoo()
    np.savez_compressed(
        os.path.join(HERE, "mesh2_golden.npz"),
        smnode_sha=sha(topo["SmNode"]), renode_sha=sha(topo["ReNode"]), coelem_sha=sha(topo["CoElem"]),
        nnzb=int(topo["SmNode"][-1]),
        k_row=Kc.row[ks].astype(np.int32), k_col=Kc.col[ks].astype(np.int32), k_val=Kc.data[ks],
        k_indptr_sha=sha(K.indptr), k_indices_sha=sha(K.indices),
        m_idx=ms.astype(np.int64), m_val=M.data[ms], m_indices_sha=sha(M.indices), m_sum=M.data.sum(),
        f=F, u_seed=20240601, s_nodes=ns.astype(np.int32), s_val=S[ns], s_alias_val=Sa[ns],
        k_fro=np.sqrt(np.sum(np.where(K.data < 1e19, K.data, 0.0) ** 2)),
        n_penalty=int(np.sum(K.data == 1e20)))
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT")
    main(sys.argv[1])
