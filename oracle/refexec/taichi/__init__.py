"""Pure-Python stand-in for the part of Taichi 0.6.28 that the reference's FE modules use
-- TEST INFRASTRUCTURE ONLY.

The reference (tianshao1992/FEM_taichi) pins ``taichi==0.6.28`` (Readme.md:18), which is not
installed here.  This module restates the documented semantics of the handful of Taichi
constructs that ``FEM_model_csr.py``, ``FEM_model_bsr.py`` and ``POST_process.py`` use, so that
those files can be imported and run UNMODIFIED to produce golden outputs of the reference's
own code:

* ``ti.field(dtype, shape)`` / ``ti.Matrix.field(n, m, dtype|dt, shape)``: zero-initialised
  dense fields.  Indexing follows Taichi 0.6's default (non-packed) dense addressing: every
  axis is padded to the next power of two and an index is reduced to its low
  ``log2(padded)`` bits (the compiler lowers a dense access to a bit extract; no bounds
  check outside debug mode).  In-range indices are unaffected; an out-of-range index aliases
  a cell of the same field.  The reference relies on this once: ``Post.GMat`` is declared
  with shape 2 (POST_process.py:145) and written / read with indices 0..7
  (POST_process.py:177, 310-317), so entry j aliases entry j & 1.
  Scalar reads return ``numpy.float64`` (f64 fields) or ``int`` (i32 fields) so that FP
  arithmetic keeps IEEE semantics (0/0 -> nan, as compiled Taichi code does); stores cast to
  the field type (float -> i32 truncates toward zero).
* ``ti.Matrix``: small dense float64 matrices with ``@``, ``+``, ``-``, scalar ``*``, ``/``,
  ``.transpose()``, ``.determinant()``, ``.inverse()`` (3x3 by the adjugate times the
  reciprocal of the cofactor-expanded determinant), ``Matrix.zero(dt, n, m=1)`` (n rows,
  m columns) and ``Matrix.diag(dim, val)``.  A single subscript ``A[i]`` addresses entry
  ``(i, 0)``, as Taichi 0.6 does.  ``field[idx]`` of a matrix field returns a matrix that
  writes through to the field, so ``F[i][p, q] = v`` and ``F[i] += A`` store like Taichi.
* ``@ti.kernel``: runs the Python body serially.  The reference's parallel ``+=`` are
  atomic in Taichi; a serial run is one of the orders Taichi may produce, so results agree
  with a Taichi run up to summation order (the 1e-12 relative parity tolerance).
  ``@ti.func`` and ``@ti.data_oriented`` are the identity; ``ti.static`` returns its
  argument; ``ti.ndrange`` is the Cartesian product of ranges; iterating a field yields its
  (logical) index tuples (struct-for).
* ``ti.init`` / ``ti.reset``: no-ops (every field belongs to the object that created it).

Nothing in the product imports this; it is put on ``sys.path`` only by
``oracle/refexec/reference_runner.py``.
"""
from __future__ import annotations

import functools
import itertools

import numpy as np

__version__ = "0.6.28-standin"

cpu = "cpu"
gpu = "gpu"
f64 = np.float64
f32 = np.float32
i32 = np.int32
i64 = np.int64


def init(arch=None, default_fp=None, default_ip=None, **kwargs):
    return None


def reset():
    return None


def data_oriented(cls):
    return cls


def func(fn):
    return fn


def kernel(fn):
    @functools.wraps(fn)
    def run(*args, **kwargs):
        # compiled Taichi code computes IEEE results silently (inf / nan, no exceptions)
        with np.errstate(all="ignore"):
            return fn(*args, **kwargs)
    return run


def static(x, *more):
    return (x,) + more if more else x


def ndrange(*dims):
    rs = [range(d) if np.ndim(d) == 0 else range(int(d[0]), int(d[1])) for d in dims]
    return itertools.product(*rs)


def _pow2(n: int) -> int:
    p = 1
    while p < n:
        p <<= 1
    return p


def _as_shape(shape):
    if shape is None:
        return ()
    if np.ndim(shape) == 0:
        return (int(shape),)
    return tuple(int(s) for s in shape)


class Matrix:
    """Small dense float64 matrix (n rows x m columns)."""

    __slots__ = ("a",)
    __array_ufunc__ = None          # numpy scalars defer to Matrix.__rmul__ etc.

    def __init__(self, data, dt=None):
        a = np.array(data, dtype=np.float64)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        object.__setattr__(self, "a", a)

    @classmethod
    def _wrap(cls, arr):
        obj = object.__new__(cls)
        object.__setattr__(obj, "a", arr)
        return obj

    # -- constructors ------------------------------------------------------------------------
    @staticmethod
    def zero(dt=None, n=1, m=1):
        return Matrix._wrap(np.zeros((int(n), int(m)), dtype=np.float64))

    @staticmethod
    def diag(dim, val):
        return Matrix._wrap(np.eye(int(dim), dtype=np.float64) * float(val))

    @staticmethod
    def field(n, m, dtype=None, shape=None, dt=None, **kwargs):
        return _Field(dtype if dtype is not None else dt, _as_shape(shape), (int(n), int(m)))

    # -- shape and element access --------------------------------------------------------------
    @property
    def n(self):
        return self.a.shape[0]

    @property
    def m(self):
        return self.a.shape[1]

    @staticmethod
    def _key(idx):
        if isinstance(idx, tuple):
            return (int(idx[0]), int(idx[1])) if len(idx) == 2 else (int(idx[0]), 0)
        return (int(idx), 0)

    def __getitem__(self, idx):
        return self.a[self._key(idx)]

    def __setitem__(self, idx, v):
        self.a[self._key(idx)] = v

    # -- arithmetic ----------------------------------------------------------------------------
    def __matmul__(self, other):
        return Matrix._wrap(self.a @ other.a)

    def __add__(self, other):
        return Matrix._wrap(self.a + (other.a if isinstance(other, Matrix) else other))

    __radd__ = __add__

    def __sub__(self, other):
        return Matrix._wrap(self.a - (other.a if isinstance(other, Matrix) else other))

    def __rsub__(self, other):
        return Matrix._wrap((other.a if isinstance(other, Matrix) else other) - self.a)

    def __mul__(self, other):
        return Matrix._wrap(self.a * (other.a if isinstance(other, Matrix) else other))

    __rmul__ = __mul__

    def __truediv__(self, other):
        return Matrix._wrap(self.a / (other.a if isinstance(other, Matrix) else other))

    def __neg__(self):
        return Matrix._wrap(-self.a)

    def __iadd__(self, other):
        self.a += other.a if isinstance(other, Matrix) else other
        return self

    def __isub__(self, other):
        self.a -= other.a if isinstance(other, Matrix) else other
        return self

    def __imul__(self, other):
        self.a *= other.a if isinstance(other, Matrix) else other
        return self

    def __itruediv__(self, other):
        self.a /= other.a if isinstance(other, Matrix) else other
        return self

    def transpose(self):
        return Matrix._wrap(self.a.T.copy())

    def determinant(self):
        a = self.a
        if a.shape == (2, 2):
            return a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]
        if a.shape != (3, 3):
            raise NotImplementedError("determinant of a %dx%d matrix" % a.shape)
        # cofactor expansion along the first column
        return (a[0, 0] * (a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2])
                - a[1, 0] * (a[0, 1] * a[2, 2] - a[2, 1] * a[0, 2])
                + a[2, 0] * (a[0, 1] * a[1, 2] - a[1, 1] * a[0, 2]))

    def inverse(self):
        a = self.a
        if a.shape != (3, 3):
            raise NotImplementedError("inverse of a %dx%d matrix" % a.shape)
        r = 1.0 / self.determinant()
        out = np.empty((3, 3), dtype=np.float64)
        for i in range(3):
            for j in range(3):
                # adjugate: out[j, i] = cofactor (i, j)
                i1, i2, j1, j2 = (i + 1) % 3, (i + 2) % 3, (j + 1) % 3, (j + 2) % 3
                out[j, i] = r * (a[i1, j1] * a[i2, j2] - a[i2, j1] * a[i1, j2])
        return Matrix._wrap(out)

    def to_numpy(self):
        return self.a.copy()

    def __repr__(self):
        return "Matrix(%r)" % (self.a.tolist(),)


class _Field:
    """Dense field of scalars (elem=None) or n x m matrices, zero-initialised."""

    def __init__(self, dtype, shape, elem=None):
        self.dtype = np.dtype(dtype if dtype is not None else np.float64)
        self._shape = shape
        self._elem = elem
        self._mask = tuple(_pow2(s) - 1 for s in shape)
        padded = tuple(_pow2(s) for s in shape)
        self._data = np.zeros(padded + (elem if elem else ()), dtype=self.dtype)
        self._is_float = self.dtype.kind == "f"

    @property
    def shape(self):
        return self._shape

    def _addr(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        if len(idx) != len(self._shape):
            raise IndexError("field of rank %d indexed with %d indices" % (len(self._shape), len(idx)))
        return tuple(int(i) & m for i, m in zip(idx, self._mask))

    def __getitem__(self, idx):
        a = self._addr(idx)
        if self._elem:
            return Matrix._wrap(self._data[a])          # a view: stores write through
        v = self._data[a]
        return v if self._is_float else int(v)

    def __setitem__(self, idx, v):
        a = self._addr(idx)
        if self._elem:
            self._data[a] = v.a if isinstance(v, Matrix) else v
        else:
            self._data[a] = v

    def __iter__(self):                                  # struct-for over the index space
        return itertools.product(*[range(s) for s in self._shape])

    def _logical(self):
        return tuple(slice(0, s) for s in self._shape)

    def from_numpy(self, arr):
        arr = np.asarray(arr)
        want = self._shape + (self._elem if self._elem else ())
        if self._elem and self._elem[1] == 1 and arr.shape == self._shape + (self._elem[0],):
            arr = arr[..., None]
        if arr.shape != want:
            raise ValueError("from_numpy: shape %s does not match field shape %s" % (arr.shape, want))
        self._data[self._logical()] = arr.astype(self.dtype)

    def to_numpy(self):
        out = self._data[self._logical()].copy()
        if self._elem and self._elem[1] == 1:
            out = out[..., 0]                            # n x 1 matrices come back as vectors
        return out

    def fill(self, v):
        self._data[...] = v


def field(dtype=None, shape=None, **kwargs):
    return _Field(dtype if dtype is not None else kwargs.get("dt"), _as_shape(shape))


var = field
