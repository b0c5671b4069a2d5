"""CPU oracle for the hex8 assembly / stress hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in vectorised numpy, the arithmetic of the Taichi reference
(tianshao1992/FEM_taichi) for the path

    topology  -> K, M, F element integrals + scatter -> penalty -> CSR / BSR
    stress    -> Gauss-point stresses -> nodal extrapolation -> average -> principal / "VM"

It is the checker against which the CUDA path is compared.  Nothing in the product
package imports it; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg may use it.

PARITY PINNED to the reference's own execution: the reference ships no golden vectors for
this path (its only test file exercises a third-party Pardiso wrapper) and its JIT (taichi
0.6.28) is not installed, so its unmodified FEM_model_csr.py / FEM_model_bsr.py /
POST_process.py were run under a pure-Python restatement of the Taichi constructs they use
(``oracle/refexec``), producing ``tests/golden/refexec_*.npz``; this module agrees with
those outputs (``tests/test_refexec.py``).  It is also cross-checked against an independent
C restatement (``fem_oracle.c``) and analytic known-answer properties (rigid-body null space,
symmetry, total mass, centrifugal resultant, constant-stress patch test).

GMat reading: the reference's shape-2 GMat field read with indices 0..7 resolves, under
Taichi 0.6's dense addressing, to entry j & 1 ('aliased', the default here); 'written'
(the eight assigned corners) is kept for comparison.

Every function cites the reference file:line it follows.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

# ---------------------------------------------------------------------------
# Constants: FEM_model_bsr.py:97 (GS), :425-432 (RMat order, zeta fastest),
# :435-449 (DMat), POST_process.py:280 (same GS), :310-317 (GMat).
# ---------------------------------------------------------------------------
GS1 = 0.57735026918962            # literal abscissa, not 1/sqrt(3)
GS = (-GS1, GS1)
RMAT = np.array([[GS[i], GS[j], GS[k]] for i in (0, 1) for j in (0, 1) for k in (0, 1)],
                dtype=np.float64)   # (8,3), g = 4i + 2j + k

# GMat as the assignment statements write it (POST_process.py:310-317), GP order.
GMAT_WRITTEN = np.array([[-1, -1, -1], [-1, -1, 1], [-1, 1, -1], [-1, 1, 1],
                         [1, -1, -1], [1, -1, 1], [1, 1, -1], [1, 1, 1]], dtype=np.float64)
# GMat is declared with shape=2 (POST_process.py:145).  Under a runtime that maps an
# index of a 2-entry dense field by its low bit, entry j aliases entry j & 1, and the
# last writes (j = 6, 7) win: (1,1,-1) for even j, (1,1,1) for odd j.
GMAT_ALIASED = np.array([GMAT_WRITTEN[6 + (j & 1)] for j in range(8)], dtype=np.float64)


def shape_func(r):
    """N_a at natural point r; node sign order of FEM_model_bsr.py:371-382."""
    r0, r1, r2 = r
    return np.array([
        0.125 * (1 + r0) * (1 + r1) * (1 - r2),
        0.125 * (1 - r0) * (1 + r1) * (1 - r2),
        0.125 * (1 - r0) * (1 - r1) * (1 - r2),
        0.125 * (1 + r0) * (1 - r1) * (1 - r2),
        0.125 * (1 + r0) * (1 + r1) * (1 + r2),
        0.125 * (1 - r0) * (1 + r1) * (1 + r2),
        0.125 * (1 - r0) * (1 - r1) * (1 + r2),
        0.125 * (1 + r0) * (1 - r1) * (1 + r2)], dtype=np.float64)


def shape_derv(r):
    """dN_a/dxi_d as an (8,3) matrix; FEM_model_bsr.py:384-419 (same literals)."""
    r0, r1, r2 = r
    d = np.zeros((8, 3), dtype=np.float64)
    d[2, 0] = 0.125 * (-1) * (1 - r1) * (1 - r2)
    d[2, 1] = 0.125 * (1 - r0) * (-1) * (1 - r2)
    d[2, 2] = 0.125 * (1 - r0) * (1 - r1) * (-1)
    d[6, 0] = 0.125 * (-1) * (1 - r1) * (1 + r2)
    d[6, 1] = 0.125 * (1 - r0) * (-1) * (1 + r2)
    d[6, 2] = 0.125 * (1 - r0) * (1 - r1) * (+1)
    d[7, 0] = 0.125 * (+1) * (1 - r1) * (1 + r2)
    d[7, 1] = 0.125 * (1 + r0) * (-1) * (1 + r2)
    d[7, 2] = 0.125 * (1 + r0) * (1 - r1) * (+1)
    d[3, 0] = 0.125 * (+1) * (1 - r1) * (1 - r2)
    d[3, 1] = 0.125 * (1 + r0) * (-1) * (1 - r2)
    d[3, 2] = 0.125 * (1 + r0) * (1 - r1) * (-1)
    d[1, 0] = 0.125 * (-1) * (1 + r1) * (1 - r2)
    d[1, 1] = 0.125 * (1 - r0) * (+1) * (1 - r2)
    d[1, 2] = 0.125 * (1 - r0) * (1 + r1) * (-1)
    d[5, 0] = 0.125 * (-1) * (1 + r1) * (1 + r2)
    d[5, 1] = 0.125 * (1 - r0) * (+1) * (1 + r2)
    d[5, 2] = 0.125 * (1 - r0) * (1 + r1) * (+1)
    d[4, 0] = 0.125 * (+1) * (1 + r1) * (1 + r2)
    d[4, 1] = 0.125 * (1 + r0) * (+1) * (1 + r2)
    d[4, 2] = 0.125 * (1 + r0) * (1 + r1) * (+1)
    d[0, 0] = 0.125 * (+1) * (1 + r1) * (1 - r2)
    d[0, 1] = 0.125 * (1 + r0) * (+1) * (1 - r2)
    d[0, 2] = 0.125 * (1 + r0) * (1 + r1) * (-1)
    return d


def shapefunc_gs(rtr):
    """Extrapolation weights at GMat point; POST_process.py:212-223 (divides by GS[1])."""
    a, b, c = rtr[0] / GS1, rtr[1] / GS1, rtr[2] / GS1
    return np.array([
        0.125 * (1 + a) * (1 + b) * (1 - c),
        0.125 * (1 - a) * (1 + b) * (1 - c),
        0.125 * (1 - a) * (1 - b) * (1 - c),
        0.125 * (1 + a) * (1 - b) * (1 - c),
        0.125 * (1 + a) * (1 + b) * (1 + c),
        0.125 * (1 - a) * (1 + b) * (1 + c),
        0.125 * (1 - a) * (1 - b) * (1 + c),
        0.125 * (1 + a) * (1 - b) * (1 + c)], dtype=np.float64)


def extrapolation_table(gmat_mode: str = "aliased") -> np.ndarray:
    """W[j, k]: weight of GP k's stress in node j's value (POST_process.py:176-181)."""
    g = GMAT_WRITTEN if gmat_mode == "written" else GMAT_ALIASED
    return np.stack([shapefunc_gs(g[j]) for j in range(8)])


NR = np.stack([shape_func(RMAT[g]) for g in range(8)])     # (8 GP, 8 nodes)
DNR = np.stack([shape_derv(RMAT[g]) for g in range(8)])    # (8 GP, 8 nodes, 3)


def dmats(EX, PO):
    """DMat[0] (normal 3x3) and DMat[1] (shear, mu*I); FEM_model_bsr.py:435-449."""
    d0 = np.empty((3, 3))
    dd = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO)
    do = EX * PO / (1 + PO) / (1 - 2 * PO)
    d0[:] = do
    d0[0, 0] = d0[1, 1] = d0[2, 2] = dd
    d1 = np.eye(3) * (EX / 2 / (1 + PO))
    return d0, d1


def det3(J):
    """Cofactor expansion along column 0 (the 3x3 determinant form of the Taichi matrix lib)."""
    a = lambda i, j: J[..., i, j]  # noqa: E731
    return (a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2))
            - a(1, 0) * (a(0, 1) * a(2, 2) - a(2, 1) * a(0, 2))
            + a(2, 0) * (a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2)))


def inv3(J):
    """Adjugate / det with cyclic cofactors (closed-form 3x3 inverse)."""
    inv_det = 1.0 / det3(J)
    out = np.empty_like(J)
    E = lambda x, y: J[..., x % 3, y % 3]  # noqa: E731
    for i in range(3):
        for j in range(3):
            out[..., j, i] = inv_det * (E(i + 1, j + 1) * E(i + 2, j + 2) - E(i + 2, j + 1) * E(i + 1, j + 2))
    return out


# ---------------------------------------------------------------------------
# Topology: READ_physics.py:42-61
# ---------------------------------------------------------------------------
def pre_process(Node, Elem):
    """Nind, SmNode, ReNode, CoNode, CoElem exactly as READ_physics.py:42-61 (scipy SpGEMM)."""
    Num_Node = Node.shape[-1]
    Num_Elem = Elem.shape[-1]
    Num_MaxN = int(Node[0, :].max())
    Nind = np.zeros((Num_MaxN,), dtype=np.int64)
    Nind[Node[0, :].astype(np.int64) - 1] = np.linspace(0, Num_Node - 1, num=Num_Node, dtype=np.int64)
    Row_Elem = np.linspace(0, Num_Elem - 1, num=Num_Elem, dtype=np.int64).repeat(8)
    Col_Node = Nind[Elem[-8:].T.flatten()]
    Val_Rela = np.ones_like(Row_Elem)
    Elem_Node = sp.coo_matrix((Val_Rela, (Row_Elem, Col_Node)), shape=(Num_Elem, Num_Node)).tocsc()
    Node_Node = Elem_Node.T * Elem_Node
    Node_Node.sort_indices()
    SmNode = Node_Node.indptr
    CoNode = Node_Node.indptr[1:] - Node_Node.indptr[:-1]
    CoElem = Elem_Node.indptr[1:] - Elem_Node.indptr[:-1]
    ReNode = Node_Node.indices
    return dict(Nind=Nind, SmNode=SmNode, ReNode=ReNode, CoNode=CoNode, CoElem=CoElem,
                Num_Node=Num_Node, Num_Elem=Num_Elem, Num_MaxN=Num_MaxN)


def _coords(Physics):
    """Coord[e] = 3x8 node coordinates; FEM_CONST loop FEM_model_bsr.py:451-453."""
    node_xyz = np.asarray(Physics.Node[-3:, :], dtype=np.float64)       # (3, N)
    idx = np.asarray(Physics.Nind)[np.asarray(Physics.Elem[-8:, :])]     # (8, E) node index
    return node_xyz[:, idx].transpose(2, 0, 1), idx.T                   # (E,3,8), (E,8)


def _slots(Physics, nodes):
    """Slot of column node k in block row j for every (e, j, k).

    FEM_model_bsr.py:167-175: linear search over ReNode[SmNode[row] : +CoNode[row]] for
    the first entry equal to the column node.  Row columns are sorted and unique, so the
    first match equals the searchsorted position.
    """
    SmNode = np.asarray(Physics.SmNode, dtype=np.int64)
    ReNode = np.asarray(Physics.ReNode, dtype=np.int64)
    E = nodes.shape[0]
    rows = np.repeat(nodes[:, :, None], 8, axis=2)          # (E,8,8) row node j
    cols = np.repeat(nodes[:, None, :], 8, axis=1)          # (E,8,8) col node k
    key = rows.astype(np.int64) * (ReNode.max() + 1 if ReNode.size else 1)
    # global search: rows are contiguous & sorted in ReNode, so search on (row, col) keys
    n_row = np.diff(SmNode)
    row_of_slot = np.repeat(np.arange(SmNode.size - 1, dtype=np.int64), n_row)
    gkey = row_of_slot * (ReNode.max() + 1) + ReNode
    q = key + cols
    slot = np.searchsorted(gkey, q.ravel()).reshape(E, 8, 8)
    if not np.array_equal(gkey[np.minimum(slot, gkey.size - 1)], q):
        raise ValueError("pattern does not contain an element node pair")
    return slot


def _bounds_packed(Physics):
    """FEM_model_bsr.py:68-77: (4, nb) array [point; dof0; dof1; dof2]."""
    parts = []
    for b in Physics.Bounds:
        p = np.asarray(b[0])[np.newaxis, :]
        c = np.repeat(np.array(b[1], dtype=np.float64)[:, np.newaxis], p.shape[-1], axis=-1)
        parts.append(np.concatenate((p, c), axis=0))
    return np.concatenate(parts, axis=-1) if parts else np.zeros((4, 1))


def _forces_packed(Physics):
    """FEM_model_bsr.py:79-88: load values are cast to int (np.int) before packing."""
    parts = []
    for f in Physics.Forces:
        p = np.asarray(f[0])[np.newaxis, :]
        v = np.repeat(np.array(f[1], dtype=np.int64)[:, np.newaxis], p.shape[-1], axis=-1)
        parts.append(np.concatenate((p, v), axis=0))
    return np.concatenate(parts, axis=-1).astype(np.float64) if parts else np.zeros((4, 1))


def _btdb(B, D):
    """(n,8,8,3,3) blocks B_j^T D B_k from B (n,8,3,3) indexed [e, node, row r, col p]."""
    n = B.shape[0]
    BtD = np.einsum('ejrp,rs->ejps', B, D).reshape(n, 24, 3)        # [(j,p), s]
    Bk = B.transpose(0, 2, 1, 3).reshape(n, 3, 24)                   # [s, (k,q)]
    return np.matmul(BtD, Bk).reshape(n, 8, 3, 8, 3).transpose(0, 1, 3, 2, 4)


class OracleModel:
    """CPU restatement of ``Model`` (FEM_model_csr.py / FEM_model_bsr.py, linear part)."""

    def __init__(self, Physics, Materials, Omegas=(0, 0, 100), chunk=2048):
        self.P = Physics
        self.DE, self.EX, self.PO = Materials['DE'], Materials['EX'], Materials['PO']
        self.OM = np.array(Omegas, dtype=np.float64)
        self.N = int(Physics.Num_Node)
        self.E = int(Physics.Num_Elem)
        self.chunk = chunk
        self.coord, self.nodes = _coords(Physics)
        self.slot = _slots(Physics, self.nodes)
        self.D0, self.D1 = dmats(self.EX, self.PO)

    # -- element integrals ------------------------------------------------------
    def element_K(self, e0, e1):
        """UnitMatrixK, FEM_model_bsr.py:262-274 with installLocalB :303-347 (B2 rows yz,xz,xy)."""
        C = self.coord[e0:e1]
        n = C.shape[0]
        K = np.zeros((n, 8, 8, 3, 3))
        for g in range(8):
            DNr = DNR[g]
            J = C @ DNr                                      # (n,3,3)
            Jinv = inv3(J)
            DN = DNr[None] @ Jinv                            # (n,8,3)
            Jdet = det3(J)
            B1 = np.zeros((n, 8, 3, 3))
            B1[:, :, 0, 0], B1[:, :, 1, 1], B1[:, :, 2, 2] = DN[..., 0], DN[..., 1], DN[..., 2]
            B2 = np.zeros((n, 8, 3, 3))
            B2[:, :, 0, 1], B2[:, :, 0, 2] = DN[..., 2], DN[..., 1]
            B2[:, :, 1, 0], B2[:, :, 1, 2] = DN[..., 2], DN[..., 0]
            B2[:, :, 2, 0], B2[:, :, 2, 1] = DN[..., 1], DN[..., 0]
            # B_j^T D B_k for all (j, k) as one batched (24x3)(3x3)(3x24) product per element
            t1 = _btdb(B1, self.D0)
            t2 = _btdb(B2, self.D1)
            K += Jdet[:, None, None, None, None] * (t1 + t2)
        return K

    def element_M(self, e0, e1):
        """UnitMatrixM, FEM_model_bsr.py:276-287 (J_det = DE * det)."""
        C = self.coord[e0:e1]
        M = np.zeros((C.shape[0], 8, 8))
        for g in range(8):
            Jdet = self.DE * det3(C @ DNR[g])
            M += Jdet[:, None, None] * NR[g][None, :, None] * NR[g][None, None, :]
        return M

    def element_F(self, e0, e1):
        """InstallVectorF body, FEM_model_bsr.py:229-245 with UnitVectorF :291-300."""
        C = self.coord[e0:e1]
        w = self.OM
        F = np.zeros((C.shape[0], 8, 3))
        for g in range(8):
            R = C @ NR[g]                                    # (n,3)
            J = C @ DNR[g]
            f = np.empty_like(R)
            f[:, 0] = w[1] * w[1] * R[:, 0] + w[2] * w[2] * R[:, 0] - w[0] * w[1] * R[:, 1] - w[0] * w[2] * R[:, 2]
            f[:, 1] = w[0] * w[0] * R[:, 1] + w[2] * w[2] * R[:, 1] - w[1] * w[2] * R[:, 2] - w[1] * w[0] * R[:, 0]
            f[:, 2] = w[1] * w[1] * R[:, 2] + w[0] * w[0] * R[:, 2] - w[2] * w[0] * R[:, 0] - w[2] * w[1] * R[:, 1]
            Jdet = self.DE * det3(J)
            F += (Jdet[:, None, None] * NR[g][None, :, None]) * f[:, None, :]
        return F

    def element_KN(self, e0, e1, U):
        """UnitK, FEM_model_bsr.py:476-515 (large displacement): tangent KT and secant KM blocks
        of elements [e0, e1) at nodal displacements U (N, 3).

        T = CoordU . DN is the displacement gradient; BN1/BN2 (InslocalBN, :544-592) its
        nonlinear strain operators.  S accumulates D (B + BN/2) u_j over corners j and over
        Gauss points in order without being reset between Gauss points (:491-494), and the
        geometric term of Gauss point g uses the sum reached after g (MatrixS, :517-525;
        :508-513).  KT += det (A + B), KM += det (A + B/2) with A = (B1+BN1)^T D0 B1 +
        (B2+BN2)^T D1 B2 and B the same with BN in place of B on the right (:496-506)."""
        C = self.coord[e0:e1]
        n = C.shape[0]
        Ue = np.asarray(U, dtype=np.float64)[self.nodes[e0:e1]]          # (n, 8, 3) corner u
        CU = Ue.transpose(0, 2, 1)                                       # (n, 3, 8) CoordU
        S0 = np.zeros((n, 3))
        S1 = np.zeros((n, 3))
        KT = np.zeros((n, 8, 8, 3, 3))
        KM = np.zeros((n, 8, 8, 3, 3))
        for g in range(8):
            DNr = DNR[g]
            J = C @ DNr
            DN = DNr[None] @ inv3(J)                                     # (n, 8, 3)
            Jdet = det3(J)
            T = CU @ DN                                                  # (n, 3, 3)
            B1 = np.zeros((n, 8, 3, 3))
            B1[:, :, 0, 0], B1[:, :, 1, 1], B1[:, :, 2, 2] = DN[..., 0], DN[..., 1], DN[..., 2]
            B2 = np.zeros((n, 8, 3, 3))
            B2[:, :, 0, 1], B2[:, :, 0, 2] = DN[..., 2], DN[..., 1]
            B2[:, :, 1, 0], B2[:, :, 1, 2] = DN[..., 2], DN[..., 0]
            B2[:, :, 2, 0], B2[:, :, 2, 1] = DN[..., 1], DN[..., 0]
            BN1 = np.zeros((n, 8, 3, 3))
            BN2 = np.zeros((n, 8, 3, 3))
            for m in range(3):                                           # BN1[m, k] = T[k, m] DN[j, m]
                BN1[:, :, m, :] = T[:, None, :, m] * DN[:, :, m, None]
            BN2[:, :, 0, :] = T[:, None, :, 2] * DN[:, :, 1, None] + T[:, None, :, 1] * DN[:, :, 2, None]
            BN2[:, :, 1, :] = T[:, None, :, 2] * DN[:, :, 0, None] + T[:, None, :, 0] * DN[:, :, 2, None]
            BN2[:, :, 2, :] = T[:, None, :, 1] * DN[:, :, 0, None] + T[:, None, :, 0] * DN[:, :, 1, None]
            for j in range(8):
                t1 = np.einsum('erp,ep->er', B1[:, j] + 0.5 * BN1[:, j], Ue[:, j])
                t2 = np.einsum('erp,ep->er', B2[:, j] + 0.5 * BN2[:, j], Ue[:, j])
                S0 += t1 @ self.D0.T
                S1 += t2 @ self.D1.T
            P1, P2 = B1 + BN1, B2 + BN2
            A = (np.einsum('ejrp,rs,eksq->ejkpq', P1, self.D0, B1, optimize=True)
                 + np.einsum('ejrp,rs,eksq->ejkpq', P2, self.D1, B2, optimize=True))
            Bm = (np.einsum('ejrp,rs,eksq->ejkpq', P1, self.D0, BN1, optimize=True)
                  + np.einsum('ejrp,rs,eksq->ejkpq', P2, self.D1, BN2, optimize=True))
            w = Jdet[:, None, None, None, None]
            KT += w * (A + Bm)
            KM += w * (A + 0.5 * Bm)
            s = np.empty((n, 3, 3))
            s[:, 0, 0], s[:, 1, 1], s[:, 2, 2] = S0[:, 0], S0[:, 1], S0[:, 2]
            s[:, 0, 1] = s[:, 1, 0] = S1[:, 2]
            s[:, 0, 2] = s[:, 2, 0] = S1[:, 1]
            s[:, 1, 2] = s[:, 2, 1] = S1[:, 0]
            geo = np.einsum('ejp,epq,ekq->ejk', DN, s, DN)
            KT += (Jdet[:, None, None] * geo)[:, :, :, None, None] * np.eye(3)[None, None, None]
        return KT, KM

    def Get_MatrixKN(self, U):
        """FEM_model_bsr.py:134-145: (KT, KM) as CSR after InstallMatrixKN (:178-191) and the
        penalty on both (ModifyMatrixK, :248-259)."""
        nnzb = int(self.P.SmNode[-1])
        VT = np.zeros((nnzb, 3, 3))
        VM = np.zeros((nnzb, 3, 3))
        for e0 in range(0, self.E, self.chunk):
            e1 = min(self.E, e0 + self.chunk)
            KT, KM = self.element_KN(e0, e1, np.asarray(U).reshape(-1, 3))
            np.add.at(VT, self.slot[e0:e1].ravel(), KT.reshape(-1, 3, 3))
            np.add.at(VM, self.slot[e0:e1].ravel(), KM.reshape(-1, 3, 3))
        self._penalty(VT)
        self._penalty(VM)
        n = 3 * self.N
        mk = lambda V: sp.bsr_matrix((V, np.asarray(self.P.ReNode), np.asarray(self.P.SmNode)),  # noqa: E731
                                     shape=(n, n), dtype=np.float64).tocsr()
        return mk(VT), mk(VM)

    # -- assembly ---------------------------------------------------------------
    def ValKT(self):
        """InstallMatrixKL scatter (FEM_model_bsr.py:163-175) + ModifyMatrixK (:248-259)."""
        nnzb = int(self.P.SmNode[-1])
        V = np.zeros((nnzb, 3, 3))
        for e0 in range(0, self.E, self.chunk):
            e1 = min(self.E, e0 + self.chunk)
            Ke = self.element_K(e0, e1)
            np.add.at(V, self.slot[e0:e1].ravel(), Ke.reshape(-1, 3, 3))
        self._penalty(V)
        return V

    def _penalty(self, V):
        B = _bounds_packed(self.P)
        if len(self.P.Bounds) == 0:
            # ModifyMatrixK still runs on the zero placeholder column (point 0).
            pass
        Nind = np.asarray(self.P.Nind)
        SmNode, ReNode = np.asarray(self.P.SmNode), np.asarray(self.P.ReNode)
        for i in range(B.shape[-1]):
            idx = Nind[int(B[0, i])]
            s0, s1 = SmNode[idx], SmNode[idx + 1]
            k = np.nonzero(ReNode[s0:s1] == idx)[0]
            if k.size:
                for j in range(3):
                    if B[j + 1, i] != -1:
                        V[s0 + k[0], j, j] = 1e20

    def ValMB(self):
        """Per-block scalar mass (InstallMatrixM scatter, FEM_model_bsr.py:193-208)."""
        nnzb = int(self.P.SmNode[-1])
        V = np.zeros((nnzb,))
        for e0 in range(0, self.E, self.chunk):
            e1 = min(self.E, e0 + self.chunk)
            np.add.at(V, self.slot[e0:e1].ravel(), self.element_M(e0, e1).ravel())
        return V

    def ValF(self):
        """InstallVectorF (FEM_model_bsr.py:229-245) then LoadF (:220-226); returns (N,3)."""
        F = np.zeros((self.N, 3))
        for e0 in range(0, self.E, self.chunk):
            e1 = min(self.E, e0 + self.chunk)
            np.add.at(F, self.nodes[e0:e1].ravel(), self.element_F(e0, e1).reshape(-1, 3))
        Fo = _forces_packed(self.P)
        Nind = np.asarray(self.P.Nind)
        for i in range(Fo.shape[-1]):
            point = int(Fo[0, i])
            F[Nind[point], :] += Fo[1:4, i]
        return F

    # -- reference getters --------------------------------------------------------
    def Get_MatrixKL(self):
        """FEM_model_bsr.py:123-131: BSR (ValKT, ReNode, SmNode) -> tocsr()."""
        n = 3 * self.N
        KT = sp.bsr_matrix((self.ValKT(), np.asarray(self.P.ReNode), np.asarray(self.P.SmNode)),
                           shape=(n, n), dtype=np.float64)
        return KT.tocsr()

    def Get_MatrixM(self):
        """FEM_model_bsr.py:147-155 / :193-217: scalar CSR with 3 entries per block."""
        SmNode = np.asarray(self.P.SmNode, dtype=np.int64)
        CoNode = np.diff(SmNode)
        ReNode = np.asarray(self.P.ReNode, dtype=np.int64)
        mb = self.ValMB()
        nnzb = mb.size
        RowM = np.zeros(3 * self.N + 1, dtype=np.int64)
        for p in range(3):
            RowM[3 * np.arange(self.N) + 1 + p] = (p + 1) * CoNode + 3 * SmNode[:-1]
        row_of_slot = np.repeat(np.arange(self.N), CoNode)
        m = np.arange(nnzb) - SmNode[row_of_slot]
        ValM = np.zeros(3 * nnzb)
        ColM = np.zeros(3 * nnzb, dtype=np.int64)
        for p in range(3):
            idx = 3 * SmNode[row_of_slot] + p * CoNode[row_of_slot] + m
            ValM[idx] = mb
            ColM[idx] = 3 * ReNode + p
        return sp.csr_matrix((ValM, ColM.astype(np.int32), RowM.astype(np.int32)),
                             shape=(3 * self.N, 3 * self.N), dtype=np.float64)

    def Get_VectorF(self):
        """FEM_model_bsr.py:157-161: ValF (3,N) -> .T.flatten() (node-major)."""
        return self.ValF().reshape(-1)


def csr_direct_K(Physics, ValKT):
    """CSR K written in place, FEM_model_csr.py:150-173 (ColK/RowK index formulas)."""
    SmNode = np.asarray(Physics.SmNode, dtype=np.int64)
    CoNode = np.diff(SmNode)
    ReNode = np.asarray(Physics.ReNode, dtype=np.int64)
    N = SmNode.size - 1
    nnzb = ReNode.size
    RowK = np.zeros(3 * N + 1, dtype=np.int64)
    for p in range(3):
        RowK[3 * np.arange(N) + 1 + p] = CoNode * 3 * (p + 1) + SmNode[:-1] * 9
    row_of_slot = np.repeat(np.arange(N), CoNode)
    m = np.arange(nnzb) - SmNode[row_of_slot]
    ValK = np.zeros(9 * nnzb)
    ColK = np.zeros(9 * nnzb, dtype=np.int64)
    for p in range(3):
        for q in range(3):
            idx = 9 * SmNode[row_of_slot] + 3 * p * CoNode[row_of_slot] + m * 3 + q
            ColK[idx] = ReNode * 3 + q
            ValK[idx] = ValKT[:, p, q]
    return sp.csr_matrix((ValK, ColK.astype(np.int32), RowK.astype(np.int32)),
                         shape=(3 * N, 3 * N), dtype=np.float64)


# ---------------------------------------------------------------------------
# Stress recovery: POST_process.py
# ---------------------------------------------------------------------------
def oracle_stress(Physics, Materials, Solutions, gmat_mode="aliased", chunk=4096):
    """Post.Get_Stress (POST_process.py:72-99) with get_NdSol :172-181, get_NdAve :183-187,
    UnitVectorS :190-209 (B2 rows xy, yz, xz) and shapefunc_GS :212-223.

    ``Solutions`` is (N,3) or (N,3,1); returns (N,10): 6 components
    [xx,yy,zz,xy,yz,xz], 3 principal (descending) and the reference's "VM".
    """
    EX, PO = Materials['EX'], Materials['PO']
    D0, D1 = dmats(EX, PO)
    coord, nodes = _coords(Physics)
    U = np.asarray(Solutions, dtype=np.float64).reshape(-1, 3)          # (N,3)
    N = U.shape[0]
    E = nodes.shape[0]
    W = extrapolation_table(gmat_mode)
    S = np.zeros((N, 6))
    for e0 in range(0, E, chunk):
        e1 = min(E, e0 + chunk)
        C = coord[e0:e1]
        Ue = U[nodes[e0:e1]]                                           # (n,8,3)
        n = C.shape[0]
        SV = np.zeros((n, 8, 6))
        for j in range(8):
            DNr = DNR[j]
            J = C @ DNr
            DN = DNr[None] @ inv3(J)                                   # (n,8,3)
            for k in range(8):
                d = DN[:, k, :]
                u = Ue[:, k, :]
                e_n = d * u                                            # B1 @ Disp
                e_s = np.stack([d[:, 1] * u[:, 0] + d[:, 0] * u[:, 1],
                                d[:, 2] * u[:, 1] + d[:, 1] * u[:, 2],
                                d[:, 2] * u[:, 0] + d[:, 0] * u[:, 2]], axis=1)
                SV[:, j, :3] += e_n @ D0.T
                SV[:, j, 3:] += e_s @ D1.T
        contrib = np.einsum('jk,nkc->njc', W, SV)                      # (n,8 nodes,6)
        np.add.at(S, nodes[e0:e1].ravel(), contrib.reshape(-1, 6))
    CoElem = np.asarray(Physics.CoElem, dtype=np.float64)
    S /= CoElem[:, None]
    return stress_table(S)


def stress_table(vector):
    """POST_process.py:80-95: tensor -> eigh -> descending -> "VM" as written."""
    tensor = np.zeros((vector.shape[0], 3, 3))
    tensor[:, 0, 0] = vector[:, 0]
    tensor[:, 1, 1] = vector[:, 1]
    tensor[:, 2, 2] = vector[:, 2]
    tensor[:, 0, 1] = tensor[:, 1, 0] = vector[:, 3]
    tensor[:, 1, 2] = tensor[:, 2, 1] = vector[:, 4]
    tensor[:, 0, 2] = tensor[:, 2, 0] = vector[:, 5]
    principle, _ = np.linalg.eigh(tensor)
    principle = principle[:, ::-1]
    vm = np.sqrt(np.square(principle[:, 0] - principle[:, 1]) + np.square(principle[:, 1] - principle[:, 2])
                 + np.square(principle[:, 2] - principle[:, 1]))[:, None]
    return np.concatenate((vector, principle, vm), axis=-1)


# ---------------------------------------------------------------------------
# Static solve stand-in for Pardiso (SOLVE_static.py:31-33): FP64 direct LU.
# ---------------------------------------------------------------------------
def oracle_solve(K, F):
    """FP64 direct solve (SuperLU) standing in for MKL Pardiso mtype=2."""
    import scipy.sparse.linalg as spla
    return spla.spsolve(K.tocsc(), F)
