"""A minimal stand-in for the ``taichi`` package (test infrastructure only).

It lets the reference's own solver module (taichi-dev/taichi_elements
engine/mpm_solver.py) be imported and its kernels run as plain Python on tiny
scenes, so that their outputs become golden vectors for the oracle and the
GPU engine.  Taichi 1.1.0 itself (the reference's pinned runtime,
requirements.txt:1) has no wheel for this Python and there is no network, so
the real runtime cannot run here.

What it reproduces of Taichi 1.x's documented semantics:

* ``@ti.kernel`` and ``@ti.func`` bodies run serially in Python.  Struct-for
  loops (``for p in field``, ``for I in ti.grouped(field)``) visit the
  field's active elements; ``ti.static`` and ``ti.grouped(ti.ndrange(...))``
  unroll as in Python.
* Kernel-scope semantics that differ from Python are restored by an AST
  rewrite of each kernel / func body before it runs:
  - assigning an expression to a local name copies it (kernel locals are
    values, not references into fields);
  - ``max`` / ``min`` / ``abs`` / ``int`` / ``float`` are the elementwise
    Taichi forms (``ti.max`` ..., ``ti.cast``);
  - ``ti.atomic_max(local, v)`` on a kernel-level local is a reduction;
  - literal floats are constants of the default float type, and arithmetic
    on literals alone is folded in Python first (as Taichi evaluates
    Python-scope expressions).
* Sparse grids: a pointer / pointer / dense tree with 4^3 leaf blocks and
  field offsets.  Reading an inactive node gives 0; writing a node, or
  ``ti.append`` to a block's particle list, activates its leaf block (and so
  every field placed under that block); ``deactivate_all`` clears the tree.
  ``ti.append`` takes physical indices and iteration yields offset
  (virtual) indices, as Taichi's SNode-level ops do.
* Dynamic particle SNodes grow to the highest written index.
* Precision (``set_precision``): ``"f64"`` stores fields and computes in
  float64 (a reference run with default_fp=f64 and f64 storage);
  ``"f32"`` stores float32 and rounds every operation to float32 (numpy
  float32 scalars and arrays; python scalars are weak).
* ``ti.svd`` (3x3): numpy's SVD in float64 put into the rotation
  convention of Taichi's 3-D SVD (U, V proper rotations; sigma_0 >= sigma_1 >=
  |sigma_2|; sigma_2 < 0 exactly when det < 0), then rounded to the mode's
  type.  Products the solver uses (U V^T, U f(sigma) V^T) do not depend on
  the remaining freedom of the decomposition.
* ``Matrix.norm(eps) = sqrt(norm_sqr + eps)`` and
  ``Matrix.normalized(eps) = v / (norm() + eps)`` (Taichi 1.1.0).

Not reproduced: quantized types, GUI, random number streams (seeding goes
through read_restart with explicit arrays), the profiler, BLS (a hint).
"""
from __future__ import annotations

import ast
import inspect
import math
import operator
import sys
import textwrap
import types

import numpy as np


class _Cfg:
    fp = np.float64


cfg = _Cfg()


def set_precision(p: str):
    cfg.fp = np.float32 if p == "f32" else np.float64


# ------------------------------------------------------------------ types --

class _DType:
    def __init__(self, name, kind):
        self.name, self.kind = name, kind

    def __repr__(self):
        return f"ti.{self.name}"


f16 = _DType("f16", "f")
f32 = _DType("f32", "f")
f64 = _DType("f64", "f")
i8 = _DType("i8", "i")
i16 = _DType("i16", "i")
i32 = _DType("i32", "i")
i64 = _DType("i64", "i")
u8 = _DType("u8", "i")
u16 = _DType("u16", "i")
u32 = _DType("u32", "i")
u64 = _DType("u64", "i")


def _kind(dt):
    if dt is int:
        return "i"
    if dt is float:
        return "f"
    return dt.kind


class _Template:
    pass


def template():
    return _Template()


class _NdarrayT:
    pass


types_ns = types.SimpleNamespace(ndarray=lambda *a, **k: _NdarrayT(), quant=types.SimpleNamespace())
types = types_ns  # noqa: F811  (ti.types.ndarray / ti.types.quant)

i = "i"
ij = ("i", "j")
ijk = ("i", "j", "k")


def axes(*a):
    return a


# ------------------------------------------------------- scalar helpers --

def _isfloat(x):
    if isinstance(x, np.ndarray):
        return x.dtype.kind == "f"
    return isinstance(x, (float, np.floating))


def _tofp(x):
    if isinstance(x, np.ndarray):
        return x if x.dtype == cfg.fp else x.astype(cfg.fp)
    if isinstance(x, (np.floating, np.integer)):
        return cfg.fp(x)
    return x  # python scalars stay weak


def _wrap(r):
    if isinstance(r, np.ndarray):
        return Matrix._of(r)
    if isinstance(r, np.integer):
        return int(r)
    return r


def _binop(op, a, b):
    A = a.a if isinstance(a, Matrix) else a
    B = b.a if isinstance(b, Matrix) else b
    if _isfloat(A) or _isfloat(B) or op is operator.truediv:
        A, B = _tofp(A), _tofp(B)
        if op is operator.truediv and not _isfloat(A) and not _isfloat(B):
            A = cfg.fp(A)
    return _wrap(op(A, B))


# ----------------------------------------------------------------- Matrix --

class Matrix:
    """Small vectors and matrices over numpy arrays (1-D or 2-D)."""
    __slots__ = ("a",)
    __array_priority__ = 1000

    def __init__(self, data, dt=None):
        if isinstance(data, Matrix):
            a = data.a.copy()
        else:
            a = np.array(data, dtype=object)
            flat = [v.item() if isinstance(v, np.generic) and not isinstance(v, np.floating) else v
                    for v in a.reshape(-1)]
            isf = (dt is not None and _kind(dt) == "f") or any(_isfloat(v) for v in flat)
            a = np.array(flat, dtype=cfg.fp if isf else np.int64).reshape(a.shape)
        self.a = a

    @classmethod
    def _of(cls, arr):
        m = cls.__new__(cls)
        m.a = arr
        return m

    # constructors
    @staticmethod
    def zero(dt, n, m=None):
        shape = (n,) if m is None else (n, m)
        return Matrix._of(np.zeros(shape, dtype=cfg.fp if _kind(dt) == "f" else np.int64))

    @staticmethod
    def identity(dt, n):
        return Matrix._of(np.eye(n, dtype=cfg.fp if _kind(dt) == "f" else np.int64))

    @staticmethod
    def field(n, m, dtype, shape=None, offset=None, **kw):
        return Field(dtype, (n, m), shape, offset)

    # element access
    def __getitem__(self, k):
        v = self.a[k]
        if isinstance(v, np.ndarray):
            return Matrix._of(v)
        return int(v) if self.a.dtype.kind == "i" else v

    def __setitem__(self, k, v):
        self.a[k] = v.a if isinstance(v, Matrix) else v

    def __len__(self):
        return self.a.shape[0]

    def __iter__(self):
        return (self[k] for k in range(self.a.shape[0]))

    @property
    def n(self):
        return self.a.shape[0]

    @property
    def m(self):
        return self.a.shape[1] if self.a.ndim == 2 else 1

    # arithmetic
    def __add__(self, o): return _binop(operator.add, self, o)
    def __radd__(self, o): return _binop(operator.add, o, self)
    def __sub__(self, o): return _binop(operator.sub, self, o)
    def __rsub__(self, o): return _binop(operator.sub, o, self)
    def __mul__(self, o): return _binop(operator.mul, self, o)
    def __rmul__(self, o): return _binop(operator.mul, o, self)
    def __truediv__(self, o): return _binop(operator.truediv, self, o)
    def __rtruediv__(self, o): return _binop(operator.truediv, o, self)
    def __floordiv__(self, o): return _binop(operator.floordiv, self, o)
    def __pow__(self, o): return _binop(operator.pow, self, o)
    def __neg__(self): return Matrix._of(-self.a)
    def __abs__(self): return Matrix._of(np.abs(self.a))

    def __matmul__(self, o):
        A, B = self.a, o.a
        if _isfloat(A) or _isfloat(B):
            A, B = _tofp(A), _tofp(B)
        # sequential sums of products, one rounding per operation
        if B.ndim == 1:
            r = A[:, 0] * B[0]
            for k in range(1, A.shape[1]):
                r = r + A[:, k] * B[k]
        else:
            r = A[:, 0:1] * B[0:1, :]
            for k in range(1, A.shape[1]):
                r = r + A[:, k:k + 1] * B[k:k + 1, :]
        return Matrix._of(r)

    def transpose(self):
        return Matrix._of(self.a.T.copy())

    def cast(self, dt):
        if _kind(dt) == "i":
            return Matrix._of(np.trunc(self.a).astype(np.int64))
        return Matrix._of(self.a.astype(cfg.fp))

    def outer_product(self, o):
        A, B = _tofp(self.a), _tofp(o.a)
        return Matrix._of(A[:, None] * B[None, :])

    def dot(self, o):
        A, B = self.a, o.a
        if _isfloat(A) or _isfloat(B):
            A, B = _tofp(A), _tofp(B)
        s = A[0] * B[0]
        for k in range(1, len(A)):
            s = s + A[k] * B[k]
        return _wrap(s)

    def sum(self):
        f = self.a.reshape(-1)
        s = f[0]
        for k in range(1, len(f)):
            s = s + f[k]
        return _wrap(s)

    def norm_sqr(self):
        return (self * self).sum()

    def norm(self, eps=0):
        return np.sqrt(_tofp(self.norm_sqr() + eps))

    def normalized(self, eps=0):
        invlen = 1 / (self.norm() + eps)
        return invlen * self

    def __repr__(self):
        return f"Matrix({self.a!r})"


class Vector(Matrix):
    __slots__ = ()

    @staticmethod
    def zero(dt, n):
        return Matrix.zero(dt, n)

    @staticmethod
    def field(n, dtype, shape=None, offset=None, **kw):
        return Field(dtype, (n,), shape, offset)


# ------------------------------------------------------------ math funcs --

def _ew(fn, x):
    if isinstance(x, Matrix):
        return Matrix._of(fn(_tofp(x.a)))
    return fn(cfg.fp(x))


def exp(x): return _ew(np.exp, x)
def log(x): return _ew(np.log, x)
def sqrt(x): return _ew(np.sqrt, x)
def sin(x): return _ew(np.sin, x)
def cos(x): return _ew(np.cos, x)
def atan2(y, x): return np.arctan2(_tofp(y), _tofp(x))


def floor(x):
    if isinstance(x, Matrix):
        return Matrix._of(np.floor(_tofp(x.a)))
    return np.floor(cfg.fp(x))


def _elem2(fn, a, b):
    A = a.a if isinstance(a, Matrix) else a
    B = b.a if isinstance(b, Matrix) else b
    if _isfloat(A) or _isfloat(B):
        A, B = _tofp(A), _tofp(B)
        if not isinstance(A, np.ndarray) and not isinstance(B, np.ndarray):
            A, B = cfg.fp(A), cfg.fp(B)
    return _wrap(fn(A, B))


def max(*args):  # noqa: A001  (Taichi's elementwise max)
    r = args[0]
    for b in args[1:]:
        r = _elem2(np.maximum, r, b)
    return r


def min(*args):  # noqa: A001
    r = args[0]
    for b in args[1:]:
        r = _elem2(np.minimum, r, b)
    return r


def abs(x):  # noqa: A001
    if isinstance(x, Matrix):
        return Matrix._of(np.abs(x.a))
    return np.abs(x) if isinstance(x, np.generic) else (x if x >= 0 else -x)


def _cast_int(x):
    if isinstance(x, Matrix):
        return x.cast(int)
    return int(x)


def _cast_float(x):
    if isinstance(x, Matrix):
        return x.cast(float)
    return cfg.fp(x)


def svd(A, dt=None):
    """3x3 SVD in the rotation convention (see the module docstring)."""
    M = np.asarray(A.a, dtype=np.float64)
    U, s, Vt = np.linalg.svd(M)
    V = Vt.T.copy()
    if np.linalg.det(U) < 0:
        U[:, -1] = -U[:, -1]
        s[-1] = -s[-1]
    if np.linalg.det(V) < 0:
        V[:, -1] = -V[:, -1]
        s[-1] = -s[-1]
    return (Matrix._of(U.astype(cfg.fp)), Matrix._of(np.diag(s).astype(cfg.fp)), Matrix._of(V.astype(cfg.fp)))


def random(dtype=None):
    return cfg.fp(np.random.random())


# --------------------------------------------------------------- misc API --

def static(x, *a):
    return x


def loop_config(**kw):
    pass


def no_activate(*a):
    pass


def block_local(*a):
    pass


def sync():
    pass


def assume_in_range(val, base, low, high):
    return val


def data_oriented(cls):
    return cls


class ndrange:
    def __init__(self, *dims):
        self.ranges = [range(d) if isinstance(d, int) else range(*d) for d in dims]

    def __iter__(self):
        import itertools
        return iter(itertools.product(*self.ranges))


def grouped(x):
    if isinstance(x, ndrange):
        return (Matrix._of(np.array(t, dtype=np.int64)) for t in x)
    if isinstance(x, Field):
        return x._grouped()
    raise TypeError(f"ti.grouped of {type(x)}")


def rescale_index(a, b, I):
    """Index I of field/SNode a rescaled to b (ratio of the cell sizes)."""
    ca, cb = _cell(a), _cell(b)
    k = np.asarray(I.a[:3], dtype=np.int64)
    if ca >= cb:
        return Matrix._of(k * (ca // cb))
    return Matrix._of(np.floor_divide(k, cb // ca))


def _cell(x):
    """Grid nodes per index of a field or SNode along one axis."""
    if isinstance(x, Field):
        return x.cell
    if x.kind == "dynamic_blocks" or (x.kind == "pointer" and x.parent_node.kind == "pointer"):
        return x.tree.leaf  # a leaf block
    raise TypeError(f"rescale_index through a {x.kind} SNode")


def atomic_max(a, b):
    raise RuntimeError("ti.atomic_max on a non-local target is not supported by the stand-in")


def atomic_add(a, b):
    raise RuntimeError("ti.atomic_add is not supported by the stand-in")


class _Profiler:
    def print_kernel_profiler_info(self):
        pass

    def print_memory_profiler_info(self):
        pass


profiler = _Profiler()


def init(*a, **k):
    pass


# ----------------------------------------------------------------- fields --

class _Comp:
    """A scalar component of a vector field (get_scalar_field)."""

    def __init__(self, f, idx):
        self.f, self.idx = f, idx


class Field:
    def __init__(self, dtype, elem=(), shape=None, offset=None):
        self.kind = _kind(dtype)
        self.elem = tuple(elem)
        self.store = None
        self.layout = None
        self.cell = 1
        self.snode = None
        if shape is not None:
            shape = () if shape == () else ((shape,) if isinstance(shape, int) else tuple(shape))
            self.layout = "dense"
            self.store = np.zeros(shape + self.elem, dtype=self._np())

    def _np(self):
        return cfg.fp if self.kind == "f" else np.int32

    def get_scalar_field(self, *idx):
        return _Comp(self, idx)

    def parent(self, k=1):
        s = self.snode
        for _ in range(k - 1):
            s = s.parent_node
        return s

    def loop_range(self):
        return self

    # value conversion
    def _out(self, v):
        if isinstance(v, np.ndarray):
            return Matrix._of(v)  # a view: writes through
        return int(v) if self.kind == "i" else v

    def _val(self, v):
        if isinstance(v, Matrix):
            return v.a
        if isinstance(v, (list, tuple)):
            return np.asarray([x.a if isinstance(x, Matrix) else x for x in v], dtype=object).astype(self._np())
        return v

    @staticmethod
    def _key(k):
        if k is None:
            return ()
        if isinstance(k, Matrix):
            return tuple(int(v) for v in k.a)
        if isinstance(k, tuple):
            out = []
            for v in k:
                if isinstance(v, Matrix):
                    out.extend(int(u) for u in v.a)
                else:
                    out.append(int(v))
            return tuple(out)
        return (int(k),)

    def __getitem__(self, k):
        key = self._key(k)
        if self.layout == "dense":
            return self._out(self.store[key])
        if self.layout == "particle":
            (p,) = key
            if p >= self.snode.length:
                return self._out(np.zeros(self.elem, self._np()).copy() if self.elem else self._np()(0))
            return self._out(self.store[p])
        if self.layout == "grid":
            return self.snode.tree.get(self, key)
        if self.layout == "pid":
            return self.snode.tree.pid_get(self, key)
        raise RuntimeError("field used before placement")

    def __setitem__(self, k, v):
        key = self._key(k)
        if self.layout == "dense":
            self.store[key] = self._val(v)
        elif self.layout == "particle":
            (p,) = key
            self.snode.activate(p)
            self.store[p] = self._val(v)
        elif self.layout == "grid":
            self.snode.tree.set(self, key, self._val(v))
        else:
            raise RuntimeError("field used before placement")

    def __iter__(self):
        if self.layout == "particle":
            return iter(range(self.snode.length))
        if self.layout == "dense":
            return iter(np.ndindex(self.store.shape[:self.store.ndim - len(self.elem)]))
        return (tuple(int(u) for u in I.a) for I in self._grouped())

    def _grouped(self):
        if self.layout == "particle":
            return (Matrix._of(np.array([p], dtype=np.int64)) for p in range(self.snode.length))
        if self.layout == "grid":
            return self.snode.tree.iter_nodes()
        if self.layout == "pid":
            return self.snode.tree.iter_pid(self)
        return (Matrix._of(np.array(t, dtype=np.int64)) for t in
                np.ndindex(self.store.shape[:self.store.ndim - len(self.elem)]))

    # numpy access for the golden generator
    def to_numpy(self):
        if self.layout == "particle":
            return self.store[:self.snode.length].copy()
        if self.layout == "dense":
            return self.store.copy()
        raise RuntimeError("use the tree accessors for sparse fields")

    def from_numpy(self, arr):
        if self.layout == "particle":
            n = len(arr)
            self.snode.activate(n - 1)
            self.store[:n] = arr
        else:
            self.store[...] = arr


# ----------------------------------------------------------------- SNodes --

PARTICLE_CAPACITY = 1 << 16


class SNode:
    def __init__(self, parent, kind, n, tree=None, cell=1):
        self.parent_node = parent
        self.kind = kind
        self.n = n
        self.tree = tree
        self.cell = cell
        self.length = 0
        self.fields = []

    def parent(self, k=1):
        s = self
        for _ in range(k):
            s = s.parent_node
        return s

    def pointer(self, axes_, n):
        if self.kind == "root":
            tree = GridTree()
            node = SNode(self, "pointer", n, tree)
            tree.top = node
            return node
        return SNode(self, "pointer", n, self.tree)

    def bitmasked(self, axes_, n):
        return self.pointer(axes_, n)

    def dense(self, axes_, n):
        if self.kind == "root":
            return SNode(self, "dense_root", n)
        node = SNode(self, "dense", n, self.tree, cell=1)
        self.tree.leaf = n
        return node

    def dynamic(self, axis, n, chunk_size=None):
        if self.kind == "root":
            return SNode(self, "dynamic_particles", n)
        node = SNode(self, "dynamic_blocks", n, self.tree)
        return node

    def place(self, *fields, offset=None, shared_exponent=False):
        for f in fields:
            if isinstance(f, _Comp):
                f = f.f
            if f.snode is not None:
                continue
            f.snode = self
            if self.kind == "dynamic_particles":
                f.layout = "particle"
                cap = int(builtins_min(self.n, PARTICLE_CAPACITY))
                f.store = np.zeros((cap,) + f.elem, dtype=f._np())
            elif self.kind == "dense":
                f.layout = "grid"
                f.cell = 1
                self.tree.add_field(f, offset)
            elif self.kind == "dynamic_blocks":
                f.layout = "pid"
                f.cell = self.tree.leaf
                self.tree.add_pid(f, offset)
            else:
                raise RuntimeError(f"placement under {self.kind} is not supported")
        return self

    def activate(self, p):
        if p >= self.length:
            self.length = p + 1

    def deactivate_all(self):
        if self.tree is not None:
            self.tree.clear()
        else:
            self.length = 0

    @property
    def cell_(self):
        return self.cell


class _Root(SNode):
    def __init__(self):
        super().__init__(None, "root", 1)

    def deactivate_all(self):
        pass


root = _Root()


class GridTree:
    """pointer -> pointer -> dense(leaf) grid with per-leaf-block activation;
    block particle lists (dynamic under the leaf pointer) share the blocks."""

    def __init__(self):
        self.top = None
        self.leaf = 4
        self.fields = []
        self.offsets = {}
        self.pid = None
        self.pid_offset = None
        self.blocks = {}  # block key -> {id(field): array}
        self.lists = {}   # block key -> list of particle ids

    def add_field(self, f, offset):
        self.fields.append(f)
        self.offsets[id(f)] = tuple(offset) if offset is not None else (0, 0, 0)

    def add_pid(self, f, offset):
        self.pid = f
        self.pid_offset = tuple(offset)[:3] if offset is not None else (0, 0, 0)

    def clear(self):
        self.blocks.clear()
        self.lists.clear()

    def _activate(self, bkey):
        b = self.blocks.get(bkey)
        if b is None:
            L = self.leaf
            b = {id(f): np.zeros((L, L, L) + f.elem, dtype=f._np()) for f in self.fields}
            self.blocks[bkey] = b
        return b

    def _split(self, key):
        L = self.leaf
        return tuple(k // L for k in key), tuple(k % L for k in key)

    def get(self, f, key):
        bkey, loc = self._split(key)
        b = self.blocks.get(bkey)
        if b is None:
            z = np.zeros(f.elem, dtype=f._np())
            return f._out(z if f.elem else z[()])
        return f._out(b[id(f)][loc])

    def set(self, f, key, val):
        bkey, loc = self._split(key)
        self._activate(bkey)[id(f)][loc] = val

    def iter_nodes(self):
        L = self.leaf
        for bkey in sorted(self.blocks):
            base = np.array(bkey, dtype=np.int64) * L
            for loc in np.ndindex(L, L, L):
                yield Matrix._of(base + np.array(loc, dtype=np.int64))

    def append(self, phys_block, p):
        bkey = tuple(int(a) + int(o) for a, o in zip(phys_block, self.pid_offset))
        self._activate(bkey)
        self.lists.setdefault(bkey, []).append(int(p))

    def pid_get(self, f, key):
        return self.lists[tuple(key[:3])][key[3]]

    def iter_pid(self, f):
        for bkey in sorted(self.lists):
            for k in range(len(self.lists[bkey])):
                yield Matrix._of(np.array(bkey + (k,), dtype=np.int64))

    # accessors for the golden generator
    def active_blocks(self):
        return sorted(self.blocks)

    def node_values(self, f):
        """(coords (K,3), values) of every node of the active blocks."""
        L = self.leaf
        coords, vals = [], []
        for bkey in sorted(self.blocks):
            base = np.array(bkey, dtype=np.int64) * L
            loc = np.array(list(np.ndindex(L, L, L)), dtype=np.int64)
            coords.append(base[None] + loc)
            vals.append(self.blocks[bkey][id(f)].reshape((L * L * L,) + f.elem))
        if not coords:
            return np.zeros((0, 3), np.int64), np.zeros((0,) + f.elem)
        return np.concatenate(coords), np.concatenate(vals)


def append(node, indices, val):
    """ti.append(dynamic SNode, physical indices of its parent, value)."""
    idx = indices.a if isinstance(indices, Matrix) else indices
    node.tree.append([int(v) for v in idx], val)


def field(dtype, shape=None, offset=None, **kw):
    return Field(dtype, (), shape, offset)


class BitpackedFields:
    def __init__(self, *a, **k):
        raise NotImplementedError("quantized fields are not supported by the stand-in")


# --------------------------------------------- kernel / func AST rewrite --

builtins_min = __builtins__["min"] if isinstance(__builtins__, dict) else __builtins__.min

_NUM = (int, float)


class _Fold(ast.NodeTransformer):
    """Folds arithmetic on numeric literals alone (Python-scope constants)."""

    @staticmethod
    def _const(node):
        return isinstance(node, ast.Constant) and type(node.value) in _NUM

    def visit_BinOp(self, node):
        self.generic_visit(node)
        if self._const(node.left) and self._const(node.right):
            v = eval(compile(ast.Expression(node), "<fold>", "eval"))
            return ast.copy_location(ast.Constant(v), node)
        return node

    def visit_UnaryOp(self, node):
        self.generic_visit(node)
        if self._const(node.operand) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = eval(compile(ast.Expression(node), "<fold>", "eval"))
            return ast.copy_location(ast.Constant(v), node)
        return node


class _Rewrite(ast.NodeTransformer):
    """Taichi kernel-scope semantics on a Python function body."""

    def visit_Constant(self, node):
        if type(node.value) is float:
            return ast.copy_location(
                ast.Call(func=ast.Name("__ti_const", ast.Load()), args=[node], keywords=[]), node)
        return node

    def visit_Call(self, node):
        self.generic_visit(node)
        if isinstance(node.func, ast.Name) and node.func.id in ("max", "min", "abs", "int", "float"):
            node.func = ast.copy_location(ast.Name(f"__ti_{node.func.id}", ast.Load()), node.func)
        return node

    def visit_Assign(self, node):
        self.generic_visit(node)
        if len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            node.value = ast.copy_location(
                ast.Call(func=ast.Name("__ti_copy", ast.Load()), args=[node.value], keywords=[]), node.value)
        return node

    def visit_Expr(self, node):
        c = node.value
        if (isinstance(c, ast.Call) and isinstance(c.func, ast.Attribute) and c.func.attr == "atomic_max"
                and isinstance(c.args[0], ast.Name)):
            tgt = c.args[0].id
            new = ast.Assign(targets=[ast.Name(tgt, ast.Store())],
                             value=ast.Call(func=ast.Name("__ti_max", ast.Load()),
                                            args=[ast.Name(tgt, ast.Load()), c.args[1]], keywords=[]))
            new = ast.copy_location(new, node)
            return self.generic_visit(new)
        self.generic_visit(node)
        return node


def _copy(v):
    if isinstance(v, Matrix):
        return Matrix._of(v.a.copy())
    return v


def _helpers():
    return {"__ti_const": lambda c: cfg.fp(c), "__ti_copy": _copy, "__ti_max": max, "__ti_min": min,
            "__ti_abs": abs, "__ti_int": _cast_int, "__ti_float": _cast_float}


def _rewrite(func):
    src = textwrap.dedent(inspect.getsource(func))
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    fdef = _Rewrite().visit(_Fold().visit(fdef))
    free = func.__code__.co_freevars
    if free:  # re-create the closure: an outer function binds the free names
        outer = ast.FunctionDef(name="__ti_outer", args=ast.arguments(
            posonlyargs=[], args=[ast.arg(n) for n in free], kwonlyargs=[], kw_defaults=[], defaults=[]),
            body=[fdef, ast.Return(ast.Name(fdef.name, ast.Load()))], decorator_list=[], returns=None,
            type_params=[])
        mod = ast.Module(body=[outer], type_ignores=[])
    else:
        mod = ast.Module(body=[fdef], type_ignores=[])
    ast.fix_missing_locations(mod)
    first = func.__code__.co_firstlineno
    ast.increment_lineno(mod, first - 1)
    code = compile(mod, inspect.getsourcefile(func) or "<kernel>", "exec")
    g = dict(func.__globals__)
    g.update(_helpers())
    ns = {}
    exec(code, g, ns)
    if free:
        return ns["__ti_outer"](*[c.cell_contents for c in func.__closure__])
    return ns[fdef.name]


def _convert_args(func, args, kwargs):
    sig = inspect.signature(func)
    ba = sig.bind(*args, **kwargs)
    for name, val in list(ba.arguments.items()):
        ann = sig.parameters[name].annotation
        if isinstance(ann, _DType):
            ba.arguments[name] = cfg.fp(val) if ann.kind == "f" else int(val)
    return ba.args, ba.kwargs


def kernel(func):
    state = {}

    def wrapper(*args, **kwargs):
        if "f" not in state:
            state["f"] = _rewrite(func)
        a, k = _convert_args(func, args, kwargs)
        return state["f"](*a, **k)

    wrapper.__wrapped__ = func
    wrapper.__name__ = func.__name__
    return wrapper


def func(fn):
    state = {}

    def wrapper(*args, **kwargs):
        if "f" not in state:
            state["f"] = _rewrite(fn)
        return state["f"](*args, **kwargs)

    wrapper.__wrapped__ = fn
    wrapper.__name__ = fn.__name__
    return wrapper
