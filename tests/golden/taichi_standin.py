"""A pure-Python stand-in for the subset of the Taichi DSL that Tina's triangle
rasteriser and deferred shading path use (test infrastructure only).

Taichi cannot be installed here, so tests/golden/make_golden.py installs this
module as `taichi` and executes the reference's own `tina` source with it to
produce golden vectors.  Semantics follow Taichi where they matter for the
numbers:

* kernels run serially in source order (the reference's `render_occup` then
  resolves `atomic_min(depth) > depth` in face order);
* Taichi's `float` is float32: field elements and kernel arithmetic are numpy
  float32 scalars (IEEE, no fused multiply-add); `int` is a Python int;
* Python-level constants fold in double precision at trace time and meet the
  float32 values as float32 literals (numpy's weak scalar promotion);
* @ti.kernel / @ti.func / @ti.pyfunc bodies are recompiled with an AST pass that
  maps int()/float()/min()/max()/`**` and ti.atomic_min(field[I], v) onto the
  element-wise helpers below, as Taichi's own AST transformer does; @ti.func
  arguments are passed by value;
* x ** n for an integer n is evaluated by repeated squaring, x ** y for a float y
  with powf; Vector.normalized() is v * (1 / sqrt(sum(v*v))) and
  Vector.sum() adds left to right, like Taichi's Matrix methods.
"""
import ast
import builtins
import functools
import inspect
import itertools
import math
import textwrap

import numpy as np

pi = math.pi
tau = math.tau
f32 = np.float32
i32 = int
cpu = 'cpu'
gpu = 'gpu'
opengl = 'opengl'


def init(*args, **kwargs):
    pass


# ---------------------------------------------------------------------------
# scalars
# ---------------------------------------------------------------------------
def _fix(x):
    """Kernel-side scalar: Python float results of f32 ops become float32."""
    if isinstance(x, (bool, np.bool_)):
        return int(x)
    if isinstance(x, np.floating) and not isinstance(x, np.float32):
        return np.float32(x)
    if isinstance(x, np.integer):
        return int(x)
    return x


def _is_float(x):
    return isinstance(x, (float, np.floating))


np.seterr(all='ignore')


def _binop(op, a, b):
    """One scalar op: float32 when either side is a kernel float32 value (a
    Python constant meets it as a float32 literal), Python arithmetic when both
    sides are trace-time constants."""
    if isinstance(a, Matrix) or isinstance(b, Matrix):
        return Matrix._elementwise(op, a, b)
    r = op(a, b)
    if isinstance(a, np.float32) or isinstance(b, np.float32):
        return np.float32(r)
    if isinstance(r, (bool, np.bool_)):
        return int(r)
    return r


def _pow_scalar(a, b):
    if isinstance(b, (int, np.integer)) and not isinstance(b, bool):
        n = int(b)
        if not (isinstance(a, np.float32)):
            return a ** n
        if n == 0:
            return np.float32(1.0)
        neg = n < 0
        n = abs(n)
        result, base, first = np.float32(1.0), a, True
        while n:
            if n & 1:
                result = base if first else np.float32(result * base)
                first = False
            n >>= 1
            if n:
                base = np.float32(base * base)
        return np.float32(np.float32(1.0) / result) if neg else result
    if isinstance(a, np.float32) or isinstance(b, np.float32):
        return np.float32(np.power(np.float32(a), np.float32(b)))
    return a ** b


def _ti_pow(a, b):
    if isinstance(a, Matrix) or isinstance(b, Matrix):
        return Matrix._elementwise(_pow_scalar, a, b)
    return _pow_scalar(a, b)


def _cast_int_scalar(x):
    if isinstance(x, (int, np.integer)):
        return int(x)
    x = float(x)
    if math.isnan(x):
        return -2**31
    if x >= 2**31:
        return 2**31 - 1
    if x < -2**31:
        return -2**31
    return int(x)  # truncation


def _ti_int(x):
    if isinstance(x, Matrix):
        return x._map(_cast_int_scalar)
    return _cast_int_scalar(x)


def _ti_float(x):
    if isinstance(x, Matrix):
        return x._map(lambda v: np.float32(v))
    return np.float32(x)


def _minmax_pair(fn, a, b):
    if isinstance(a, Matrix) or isinstance(b, Matrix):
        return Matrix._elementwise(lambda u, v: _minmax_pair(fn, u, v), a, b)
    if _is_float(a) or _is_float(b):
        if isinstance(a, np.float32) or isinstance(b, np.float32):
            return np.float32(fn(np.float32(a), np.float32(b)))
        return float(fn(a, b))
    return int(builtins.min(a, b) if fn is np.fmin else builtins.max(a, b))


def _ti_min(*args):
    if len(args) == 1:
        return builtins.min(args[0])
    r = args[0]
    for a in args[1:]:
        r = _minmax_pair(np.fmin, r, a)
    return r


def _ti_max(*args):
    if len(args) == 1:
        return builtins.max(args[0])
    r = args[0]
    for a in args[1:]:
        r = _minmax_pair(np.fmax, r, a)
    return r


def _unary(fn):
    def f(x):
        if isinstance(x, Matrix):
            return x._map(lambda v: np.float32(fn(np.float32(v))))
        if isinstance(x, np.float32):
            return np.float32(fn(x))
        return fn(x)
    return f


sqrt = _unary(np.sqrt)
floor = _unary(np.floor)
ceil = _unary(np.ceil)
sin = _unary(np.sin)
cos = _unary(np.cos)
exp = _unary(np.exp)
log = _unary(np.log)
tan = _unary(np.tan)
acos = _unary(np.arccos)
asin = _unary(np.arcsin)


def atan2(y, x):
    if isinstance(y, np.float32) or isinstance(x, np.float32):
        return np.float32(np.arctan2(np.float32(y), np.float32(x)))
    return math.atan2(y, x)


_rng = np.random.Generator(np.random.PCG64(12345))


def random(dtype=float):
    return np.float32(_rng.random())


def inside_kernel():
    return True


def static(x, *xs):
    return [x] + list(xs) if xs else x


def static_assert(cond, msg=None):
    assert cond, msg


def static_print(*args):
    pass


def smart(x):
    return x


def template():
    return None


def ext_arr():
    return None


def data_oriented(cls):
    return cls


def materialize_callback(f):
    f()
    return f


def get_runtime():
    class _R:
        materialized = True
    return _R()


def imread(path):
    raise RuntimeError('image decoding is not available in the Taichi stand-in')


class GUI:
    def __init__(self, *args, **kwargs):
        raise RuntimeError('no GUI in the Taichi stand-in')


# ---------------------------------------------------------------------------
# Matrix / Vector
# ---------------------------------------------------------------------------
class Matrix:
    """n x m matrix (m == 1: vector) of float32 or int entries."""

    __array_ufunc__ = None  # numpy scalars defer to Matrix's reflected operators

    def __init__(self, entries, _shape=None):
        if isinstance(entries, Matrix):
            entries = entries.to_list()
        entries = list(entries)
        if _shape is None:
            if entries and isinstance(entries[0], (list, tuple, Matrix)):
                rows = [list(r.entries if isinstance(r, Matrix) else r) for r in entries]
                _shape = (len(rows), len(rows[0]))
                entries = [x for r in rows for x in r]
            else:
                _shape = (len(entries), 1)
        self.n, self.m = _shape
        is_f = any(_is_float(e) for e in entries)
        if is_f:
            self.entries = [np.float32(e) for e in entries]
        else:
            self.entries = [int(e) for e in entries]

    # -- construction helpers ------------------------------------------------
    @classmethod
    def _from(cls, entries, shape):
        obj = cls.__new__(cls)
        obj.n, obj.m = shape
        obj.entries = [_fix(e) for e in entries]
        return obj

    def copy(self):
        return Matrix._from(list(self.entries), (self.n, self.m))

    @staticmethod
    def identity(dtype, n):
        z = [np.float32(0.0) if dtype in (float, f32) else 0 for _ in range(n * n)]
        for i in range(n):
            z[i * n + i] = np.float32(1.0) if dtype in (float, f32) else 1
        return Matrix._from(z, (n, n))

    @staticmethod
    def unit(n, i, dtype=float):
        z = [np.float32(0.0)] * n
        z[i] = np.float32(1.0)
        return Matrix._from(z, (n, 1))

    @staticmethod
    def cols(cols):
        n = cols[0].n
        m = len(cols)
        e = [None] * (n * m)
        for j, c in enumerate(cols):
            for i in range(n):
                e[i * m + j] = c.entries[i]
        return Matrix._from(e, (n, m))

    @staticmethod
    def rows(rows):
        n = len(rows)
        m = rows[0].n
        return Matrix._from([x for r in rows for x in r.entries], (n, m))

    @staticmethod
    def field(n, m, dtype=float, shape=(), **kwargs):
        return Field(shape, dtype, (n, m))

    # -- element access -----------------------------------------------------
    def _index(self, key):
        if isinstance(key, tuple):
            i, j = key
            return int(i) * self.m + int(j)
        return int(key)

    def __getitem__(self, key):
        return self.entries[self._index(key)]

    def __setitem__(self, key, value):
        idx = self._index(key)
        self.entries[idx] = self._coerce(value)
        self._writeback()

    def __call__(self, i, j=0):
        return self.entries[i * self.m + j]

    def _coerce(self, value):
        if self.entries and isinstance(self.entries[0], np.float32):
            return np.float32(value)
        return _fix(value)

    def _writeback(self):
        pass

    def _get(self, i):
        return self.entries[i]

    def _set(self, i, v):
        self.entries[i] = self._coerce(v)
        self._writeback()

    x = property(lambda s: s._get(0), lambda s, v: s._set(0, v))
    y = property(lambda s: s._get(1), lambda s, v: s._set(1, v))
    z = property(lambda s: s._get(2), lambda s, v: s._set(2, v))
    w = property(lambda s: s._get(3), lambda s, v: s._set(3, v))

    def __len__(self):
        return self.n

    def __iter__(self):
        if self.m == 1:
            return iter(self.entries)
        return iter([Matrix._from(self.entries[i * self.m:(i + 1) * self.m], (self.m, 1))
                     for i in range(self.n)])

    def to_list(self):
        if self.m == 1:
            return list(self.entries)
        return [self.entries[i * self.m:(i + 1) * self.m] for i in range(self.n)]

    def to_numpy(self):
        a = np.array(self.entries)
        return a if self.m == 1 else a.reshape(self.n, self.m)

    def __bool__(self):
        return all(bool(e) for e in self.entries)

    def __repr__(self):
        return f'Matrix({self.to_list()})'

    # -- arithmetic ------------------------------------------------------------
    def _map(self, fn):
        return Matrix._from([fn(e) for e in self.entries], (self.n, self.m))

    @staticmethod
    def _elementwise(op, a, b):
        if isinstance(a, Matrix) and isinstance(b, Matrix):
            assert (a.n, a.m) == (b.n, b.m), ((a.n, a.m), (b.n, b.m))
            return Matrix._from([_binop(op, x, y) for x, y in zip(a.entries, b.entries)], (a.n, a.m))
        if isinstance(a, Matrix):
            return Matrix._from([_binop(op, x, b) for x in a.entries], (a.n, a.m))
        return Matrix._from([_binop(op, a, y) for y in b.entries], (b.n, b.m))

    def __add__(self, o): return Matrix._elementwise(lambda a, b: a + b, self, o)
    def __radd__(self, o): return Matrix._elementwise(lambda a, b: a + b, o, self)
    def __sub__(self, o): return Matrix._elementwise(lambda a, b: a - b, self, o)
    def __rsub__(self, o): return Matrix._elementwise(lambda a, b: a - b, o, self)
    def __mul__(self, o): return Matrix._elementwise(lambda a, b: a * b, self, o)
    def __rmul__(self, o): return Matrix._elementwise(lambda a, b: a * b, o, self)
    def __truediv__(self, o): return Matrix._elementwise(_truediv, self, o)
    def __rtruediv__(self, o): return Matrix._elementwise(_truediv, o, self)
    def __floordiv__(self, o): return Matrix._elementwise(_floordiv, self, o)
    def __rfloordiv__(self, o): return Matrix._elementwise(_floordiv, o, self)
    def __mod__(self, o): return Matrix._elementwise(_mod, self, o)
    def __pow__(self, o): return _ti_pow(self, o)
    def __rpow__(self, o): return _ti_pow(o, self)
    def __neg__(self): return self._map(lambda v: -v)
    def __pos__(self): return self
    def __abs__(self): return self._map(lambda v: abs(v))
    def __lt__(self, o): return Matrix._elementwise(lambda a, b: int(a < b), self, o)
    def __le__(self, o): return Matrix._elementwise(lambda a, b: int(a <= b), self, o)
    def __gt__(self, o): return Matrix._elementwise(lambda a, b: int(a > b), self, o)
    def __ge__(self, o): return Matrix._elementwise(lambda a, b: int(a >= b), self, o)
    def __eq__(self, o): return Matrix._elementwise(lambda a, b: int(a == b), self, o)
    def __ne__(self, o): return Matrix._elementwise(lambda a, b: int(a != b), self, o)
    __hash__ = object.__hash__

    def __matmul__(self, o):
        assert self.m == o.n
        e = []
        for i in range(self.n):
            for j in range(o.m):
                acc = _binop(lambda a, b: a * b, self.entries[i * self.m], o.entries[j])
                for k in range(1, self.m):
                    acc = _binop(lambda a, b: a + b, acc,
                                 _binop(lambda a, b: a * b, self.entries[i * self.m + k],
                                        o.entries[k * o.m + j]))
                e.append(acc)
        return Matrix._from(e, (self.n, o.m))

    # -- Taichi Matrix methods -------------------------------------------------
    def sum(self):
        r = self.entries[0]
        for e in self.entries[1:]:
            r = _binop(lambda a, b: a + b, r, e)
        return r

    def dot(self, other):
        return (self * other).sum()

    def norm_sqr(self):
        return (self ** 2).sum()

    def norm(self, eps=0):
        return sqrt(_binop(lambda a, b: a + b, self.norm_sqr(), eps))

    def normalized(self, eps=0):
        invlen = _binop(_truediv, 1, _binop(lambda a, b: a + b, self.norm(), eps))
        return invlen * self

    def cross(self, other):
        a, b = self.entries, other.entries
        mul = lambda u, v: _binop(lambda p, q: p * q, u, v)
        subf = lambda u, v: _binop(lambda p, q: p - q, u, v)
        if self.n == 3:
            return Matrix._from([subf(mul(a[1], b[2]), mul(a[2], b[1])),
                                 subf(mul(a[2], b[0]), mul(a[0], b[2])),
                                 subf(mul(a[0], b[1]), mul(a[1], b[0]))], (3, 1))
        return subf(mul(a[0], b[1]), mul(a[1], b[0]))

    def all(self):
        return int(all(bool(e) for e in self.entries))

    def any(self):
        return int(any(bool(e) for e in self.entries))

    def max(self):
        return _ti_max(*self.entries) if len(self.entries) > 1 else self.entries[0]

    def min(self):
        return _ti_min(*self.entries) if len(self.entries) > 1 else self.entries[0]

    def transpose(self):
        return Matrix._from([self.entries[i * self.m + j] for j in range(self.m) for i in range(self.n)],
                            (self.m, self.n))

    def outer_product(self, other):
        return Matrix._from([_binop(lambda a, b: a * b, x, y) for x in self.entries for y in other.entries],
                            (self.n, other.n))


def _truediv(a, b):
    if isinstance(a, np.float32) or isinstance(b, np.float32):
        with np.errstate(all='ignore'):
            return np.float32(np.float32(a) / np.float32(b))
    if isinstance(a, int) and isinstance(b, int) and not isinstance(a, bool):
        # int / int in a kernel: both operands become float32, then an IEEE
        # float32 division (0 / 0 is NaN, x / 0 an infinity)
        with np.errstate(all='ignore'):
            return np.float32(np.float32(a) / np.float32(b))
    return a / b


def _ti_div(a, b):
    """`a / b` inside kernels and funcs (Taichi's truediv)."""
    if isinstance(a, Matrix) or isinstance(b, Matrix):
        return Matrix._elementwise(_truediv, a, b)
    return _truediv(a, b)


def _floordiv(a, b):
    if _is_float(a) or _is_float(b):
        return np.float32(np.floor(np.float32(a) / np.float32(b)))
    return a // b


def _mod(a, b):
    if _is_float(a) or _is_float(b):
        a, b = np.float32(a), np.float32(b)
        return np.float32(a - np.float32(np.floor(a / b)) * b)
    return a % b


class _VectorFactory:
    """ti.Vector(...) builds an n x 1 Matrix; ti.Vector.field etc."""

    def __call__(self, xs, dt=None):
        if isinstance(xs, Matrix):
            return xs.copy()
        return Matrix(list(xs))

    def __instancecheck__(self, obj):
        return isinstance(obj, Matrix)

    @staticmethod
    def field(n, dtype=float, shape=(), **kwargs):
        return Field(shape, dtype, (n, 1))

    @staticmethod
    def unit(n, i, dtype=float):
        return Matrix.unit(n, i, dtype)


Vector = _VectorFactory()


# ---------------------------------------------------------------------------
# Fields
# ---------------------------------------------------------------------------
class _FieldElement(Matrix):
    """A vector/matrix read from a field: element writes go back to the field."""

    def _writeback(self):
        self._field._store(self._key, self)


class Field:
    # Taichi leaves a read outside a field undefined; with clamp_reads set, an
    # out-of-range index reads the nearest element (the convention the build
    # under test documents for its post-processing passes)
    clamp_reads = False

    def __init__(self, shape, dtype, elem=None):
        if isinstance(shape, int):
            shape = (shape,)
        self.shape = tuple(int(s) for s in shape)
        self.dtype = dtype
        self.elem = elem  # (n, m) or None for scalars
        npdt = np.float32 if dtype in (float, f32) else np.int32
        full = self.shape + ((elem[0] * elem[1],) if elem else ())
        self.data = np.zeros(full, dtype=npdt)
        self.n = elem[0] if elem else None
        self.m = elem[1] if elem else None

    def _key(self, key):
        if key is None:
            return ()
        if isinstance(key, Matrix):
            return tuple(int(k) for k in key.entries)
        if isinstance(key, tuple):
            out = []
            for k in key:
                if isinstance(k, Matrix):
                    out.extend(int(v) for v in k.entries)
                else:
                    out.append(int(k))
            return tuple(out)
        return (int(key),)

    def __getitem__(self, key):
        k = self._key(key)
        if Field.clamp_reads and len(k) == len(self.shape):
            k = tuple(min(max(i, 0), n - 1) for i, n in zip(k, self.shape))
        if self.elem is None:
            v = self.data[k]
            return np.float32(v) if self.data.dtype == np.float32 else int(v)
        row = self.data[k]
        conv = np.float32 if self.data.dtype == np.float32 else int
        obj = _FieldElement._from([conv(v) for v in row], self.elem)
        obj._field = self
        obj._key = k
        return obj

    def _store(self, k, value):
        if self.elem is None:
            self.data[k] = value
        else:
            if isinstance(value, Matrix):
                vals = value.entries
            else:
                vals = np.asarray(value, dtype=np.float64).ravel().tolist()
                if len(vals) > self.elem[0] * self.elem[1]:  # e.g. a 4x4 list into a 3x3 field
                    arr = np.asarray(value, dtype=np.float64)
                    vals = arr[:self.elem[0], :self.elem[1]].ravel().tolist()
            self.data[k] = np.asarray(vals, dtype=self.data.dtype)

    def __setitem__(self, key, value):
        self._store(self._key(key), value)

    def __iter__(self):
        for idx in itertools.product(*[range(s) for s in self.shape]):
            yield idx[0] if len(idx) == 1 else idx

    def fill(self, v):
        if isinstance(v, Matrix):
            self.data[...] = np.asarray(v.entries, dtype=self.data.dtype)
        else:
            self.data[...] = v

    def from_numpy(self, arr):
        arr = np.asarray(arr)
        self.data[...] = arr.reshape(self.data.shape).astype(self.data.dtype)

    def to_numpy(self):
        if self.elem and self.elem[1] != 1:
            return self.data.reshape(self.shape + self.elem).copy()
        return self.data.copy()

    def copy_from(self, other):
        self.data[...] = other.data


def field(dtype, shape=(), **kwargs):
    return Field(shape, dtype, None)


# ---------------------------------------------------------------------------
# loops
# ---------------------------------------------------------------------------
def ndrange(*ranges):
    rs = []
    for r in ranges:
        if isinstance(r, (tuple, list)):
            rs.append(range(int(r[0]), int(r[1])))
        else:
            rs.append(range(int(r)))
    return itertools.product(*rs)


def grouped(x):
    if isinstance(x, Field):
        it = itertools.product(*[range(s) for s in x.shape])
    else:
        it = x
    for idx in it:
        if not isinstance(idx, tuple):
            idx = (idx,)
        yield Matrix._from(list(idx), (len(idx), 1))


def atomic_min_ref(fld, key, value):
    old = fld[key]
    if value < old:
        fld[key] = value
    return old


def atomic_add_ref(fld, key, value):
    old = fld[key]
    fld[key] = old + value
    return old


# ---------------------------------------------------------------------------
# kernel / func decorators: recompile the body with Taichi's source rewrites
# ---------------------------------------------------------------------------
class _Rewrite(ast.NodeTransformer):
    def visit_Call(self, node):
        self.generic_visit(node)
        f = node.func
        if isinstance(f, ast.Name) and f.id in ('int', 'float', 'min', 'max'):
            node.func = ast.Name(id={'int': '_ti_int', 'float': '_ti_float', 'min': '_ti_min',
                                     'max': '_ti_max'}[f.id], ctx=ast.Load())
        elif (isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) and f.value.id == 'ti'
              and f.attr in ('atomic_min', 'atomic_add') and node.args
              and isinstance(node.args[0], ast.Subscript)):
            sub = node.args[0]
            node = ast.Call(func=ast.Attribute(value=ast.Name(id='ti', ctx=ast.Load()),
                                               attr=f.attr + '_ref', ctx=ast.Load()),
                            args=[sub.value, sub.slice, node.args[1]], keywords=[])
        return node

    def visit_BinOp(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.Pow):
            return ast.Call(func=ast.Name(id='_ti_pow', ctx=ast.Load()), args=[node.left, node.right],
                            keywords=[])
        if isinstance(node.op, ast.Div):
            return ast.Call(func=ast.Name(id='_ti_div', ctx=ast.Load()), args=[node.left, node.right],
                            keywords=[])
        return node

    def visit_AugAssign(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.Pow):
            return ast.Assign(targets=[node.target],
                              value=ast.Call(func=ast.Name(id='_ti_pow', ctx=ast.Load()),
                                             args=[_load(node.target), node.value], keywords=[]))
        return node


def _load(target):
    t = ast.parse(ast.unparse(target), mode='eval').body
    return t


class _Env(dict):
    def __init__(self, base):
        super().__init__()
        self._base = base
        self['__builtins__'] = base.get('__builtins__', builtins)

    def __missing__(self, key):
        return self._base[key]


_HELPERS = {'_ti_int': _ti_int, '_ti_float': _ti_float, '_ti_min': _ti_min, '_ti_max': _ti_max,
            '_ti_pow': _ti_pow, '_ti_div': _ti_div}


def _recompile(fn):
    try:
        src = textwrap.dedent(inspect.getsource(fn))
    except (OSError, TypeError):
        return fn
    tree = ast.parse(src)
    fdef = tree.body[0]
    if not isinstance(fdef, (ast.FunctionDef, ast.AsyncFunctionDef)):
        return fn
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_Rewrite().visit(tree))
    ast.increment_lineno(tree, fn.__code__.co_firstlineno - 1)  # keep the file's line numbers
    glb = fn.__globals__
    for k, v in _HELPERS.items():
        glb.setdefault(k, v)
    env = glb
    if fn.__closure__:
        # free variables of a nested kernel become globals of the recompiled one;
        # everything else still resolves late through the module's globals
        env = _Env(glb)
        for name, cell in zip(fn.__code__.co_freevars, fn.__closure__):
            try:
                env[name] = cell.cell_contents
            except ValueError:
                pass
    code = compile(tree, inspect.getsourcefile(fn) or '<ti>', 'exec')
    ns = {}
    exec(code, env, ns)
    new = ns[fdef.name]
    new = functools.update_wrapper(new, fn)
    return new


def _copy_arg(a):
    return a.copy() if isinstance(a, Matrix) else a


def func(fn):
    new = _recompile(fn)

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        args = [_copy_arg(a) for a in args]
        return new(*args, **kwargs)
    return wrapper


def pyfunc(fn):
    return func(fn)


def kernel(fn):
    new = _recompile(fn)

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        return new(*args, **kwargs)
    return wrapper


class _Lang:
    pass


lang = _Lang()
