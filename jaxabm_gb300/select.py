"""Host side of K6 (stable compaction) and K7 (reductions) over SoA agent states.

``compact_states`` is ``AgentCollection.filter`` / ``AgentList.select``
(jaxabm/agent.py:213-243, jaxabm/agentpy.py:316-345): the mask is compacted into ascending
indices by the warp-ballot kernel, the count is read back once (the reference's
``int(jnp.sum(mask))`` host sync), and every attribute is gathered by row.

``select_where`` is the same for a condition that ``compile_condition`` can turn into a
predicate program (comparisons of single float32 / int32 / int8 / bool attributes with
numbers, combined with ``&``, ``|`` and ``~``): the program runs inside the compaction
kernels (``abm_select_where``), so no mask array is built; other conditions are evaluated
eagerly into a mask.
"""

import numbers

import numpy as np
import torch

from . import _dev
from . import _lib

REDUCE_SUM, REDUCE_MEAN, REDUCE_MIN, REDUCE_MAX = 0, 1, 2, 3


def _as_mask(mask, n):
    if not isinstance(mask, torch.Tensor):
        mask = torch.as_tensor(mask)
    if mask.device.type != "cuda":
        mask = mask.to(_dev.device())
    mask = mask.reshape(-1)
    if mask.numel() != n:
        raise ValueError(f"mask has {mask.numel()} entries for {n} agents")
    if mask.dtype == torch.bool:
        mask = mask.view(torch.uint8)
    elif mask.dtype != torch.uint8:
        mask = (mask != 0).view(torch.uint8)
    return mask.contiguous()


def select_indices(mask, n=None):
    """Ascending int32 indices of the true entries and their count (one host sync)."""
    if n is None:
        n = mask.numel()
    m = _as_mask(mask, n)
    idx = _dev.empty((max(n, 1),), torch.int32)
    count = _dev.empty((1,), torch.int64)
    ws = _dev.workspace(_lib.load().abm_select_workspace_bytes(n))
    _lib.call("abm_select_indices", _dev.ptr(m), n, _dev.ptr(idx), _dev.ptr(count), _dev.ptr(ws),
              ws.numel(), _dev.stream_handle())
    c = int(count.item())
    return idx[:c], c


def gather_rows(t, idx):
    """``t[idx]`` along dim 0 via the library's row gather."""
    t = t.contiguous()
    count = idx.numel()
    out = torch.empty((count,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)
    if count == 0:
        return out
    row_bytes = t.element_size() * (t[0].numel() if t.dim() > 1 else 1)
    _lib.call("abm_gather_rows", _dev.ptr(t), t.shape[0], row_bytes, _dev.ptr(idx), count,
              _dev.ptr(out), _dev.stream_handle())
    return out


def compact_states(states, mask):
    """(``{k: v[mask]}``, count) with ascending order preserved."""
    n = next(iter(states.values())).shape[0]
    idx, count = select_indices(mask, n)
    out = {}
    for k, v in states.items():
        if isinstance(v, torch.Tensor) and v.dim() >= 1 and v.shape[0] == n:
            out[k] = gather_rows(v, idx)
        else:
            out[k] = v
    return out, count


def reduce(x, op=REDUCE_MEAN):
    """Device float32 scalar: sum/mean/min/max of a float tensor (float64 accumulation)."""
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise ValueError("reduce expects a CUDA tensor")
    x32 = x.reshape(-1).to(torch.float32).contiguous()
    n = x32.numel()
    out = _dev.empty((), torch.float32)
    if n == 0:
        out.fill_(float("nan"))
        return out
    ws = _dev.workspace(_lib.load().abm_reduce_workspace_bytes(n))
    _lib.call("abm_reduce_f32", _dev.ptr(x32), n, int(op), _dev.ptr(out), _dev.ptr(ws),
              ws.numel(), _dev.stream_handle())
    return out


def mean(x):
    return reduce(x, REDUCE_MEAN)


# ---- conditions compiled into predicate programs ---------------------------------------

SELECT_LT, SELECT_LE, SELECT_GT, SELECT_GE, SELECT_EQ, SELECT_NE = 1, 2, 3, 4, 5, 6
SELECT_AND, SELECT_OR, SELECT_NOT = 7, 8, 9
_DTYPES = {torch.float32: 0, torch.int32: 1, torch.int8: 2, torch.uint8: 3, torch.bool: 3}
_MAX_ATTRS, _MAX_OPS = 4, 16

OP_DTYPE = np.dtype([("code", "<i4"), ("attr", "<i4"), ("value", "<f8")])
ATTR_DTYPE = np.dtype([("data", "<u8"), ("dtype", "<i4"), ("reserved", "<i4")])


class _NotCompilable(Exception):
    pass


class _Expr:
    """A traced condition: comparison leaves combined with &, | and ~."""

    def __and__(self, other):
        return _Node(SELECT_AND, self, _lift(other))

    def __rand__(self, other):
        return _Node(SELECT_AND, _lift(other), self)

    def __or__(self, other):
        return _Node(SELECT_OR, self, _lift(other))

    def __ror__(self, other):
        return _Node(SELECT_OR, _lift(other), self)

    def __invert__(self):
        return _Node(SELECT_NOT, self)

    def __bool__(self):
        raise _NotCompilable("a traced condition has no truth value")


def _lift(x):
    if not isinstance(x, _Expr):
        raise _NotCompilable(f"cannot combine a condition with {type(x).__name__}")
    return x


class _Node(_Expr):
    def __init__(self, code, *args):
        self.code, self.args = code, args


class _Cmp(_Expr):
    def __init__(self, attr, code, value):
        self.attr, self.code, self.value = attr, code, value


def _number(v):
    if isinstance(v, bool) or isinstance(v, numbers.Real) or isinstance(v, np.generic):
        return float(v)
    if isinstance(v, torch.Tensor) and v.numel() == 1 and not v.is_cuda:
        return float(v.item())
    raise _NotCompilable(f"cannot compare an attribute with {type(v).__name__}")


class _Attr:
    """An attribute of the traced states; comparing it with a number makes a leaf."""

    def __init__(self, name):
        self.name = name

    def _cmp(self, code, other):
        try:
            return _Cmp(self.name, code, _number(other))
        except _NotCompilable:
            return NotImplemented

    def __lt__(self, o):
        return self._cmp(SELECT_LT, o)

    def __le__(self, o):
        return self._cmp(SELECT_LE, o)

    def __gt__(self, o):
        return self._cmp(SELECT_GT, o)

    def __ge__(self, o):
        return self._cmp(SELECT_GE, o)

    def __eq__(self, o):
        return self._cmp(SELECT_EQ, o)

    def __ne__(self, o):
        return self._cmp(SELECT_NE, o)

    __hash__ = object.__hash__

    def __bool__(self):
        raise _NotCompilable("an attribute has no truth value")


class _BoolAttr(_Attr, _Expr):
    """A bool attribute: compared like any attribute, or used as a flag itself
    (``attr != 0``) in a combination."""


class _TracedStates:
    """Stands in for the states dict while tracing: indexing gives an ``_Attr`` for every
    1-D attribute of a supported dtype, and only that."""

    def __init__(self, states):
        self._states = states

    def __getitem__(self, name):
        v = self._states[name]
        if not isinstance(v, torch.Tensor) or v.dim() != 1 or v.dtype not in _DTYPES:
            raise _NotCompilable(f"attribute {name!r} is not a 1-D float32/int32/int8/bool array")
        return _BoolAttr(name) if v.dtype == torch.bool else _Attr(name)

    def __contains__(self, name):
        return name in self._states


def compile_condition(condition, states):
    """``(program, attribute names)`` of ``condition`` traced on stand-ins for ``states``, or
    None when the condition does anything but compare single attributes with numbers and
    combine the results with &, | and ~ (it is then evaluated eagerly).  The program is a
    list of (code, attribute index, value) in postfix order (``abm_select_where``)."""
    try:
        expr = condition(_TracedStates(states))
    except Exception:
        return None
    if not isinstance(expr, _Expr):
        return None
    names, prog = [], []

    def emit(e):
        if isinstance(e, _BoolAttr):
            e = _Cmp(e.name, SELECT_NE, 0.0)
        if isinstance(e, _Cmp):
            if e.attr not in names:
                names.append(e.attr)
            prog.append((e.code, names.index(e.attr), e.value))
        else:
            for a in e.args:
                emit(a)
            prog.append((e.code, 0, 0.0))
    emit(expr)
    if len(names) > _MAX_ATTRS or len(prog) > _MAX_OPS:
        return None
    return prog, names


# which path the last select_where took ("predicate" or "mask"), for inspection
last_path = None


def select_where(states, condition):
    """Ascending int32 indices of the agents satisfying ``condition(states)`` and their
    count: through a compiled predicate program when the condition allows it, else through
    the eager mask."""
    global last_path
    n = next(iter(states.values())).shape[0]
    compiled = compile_condition(condition, states)
    if compiled is None:
        last_path = "mask"
        return select_indices(condition(states), n)
    prog, names = compiled
    attrs = np.zeros(len(names), dtype=ATTR_DTYPE)
    keep = []
    for a, name in enumerate(names):
        v = states[name]
        if not v.is_cuda or v.shape[0] != n:
            last_path = "mask"
            return select_indices(condition(states), n)
        v = v.contiguous()
        keep.append(v)
        attrs[a] = (v.data_ptr(), _DTYPES[v.dtype], 0)
    ops = np.array(prog, dtype=OP_DTYPE)
    idx = _dev.empty((max(n, 1),), torch.int32)
    count = _dev.empty((1,), torch.int64)
    ws = _dev.workspace(_lib.load().abm_select_workspace_bytes(max(n, 1)))
    _lib.call("abm_select_where", attrs.ctypes.data, len(names), ops.ctypes.data, len(prog), n,
              _dev.ptr(idx), _dev.ptr(count), _dev.ptr(ws), ws.numel(), _dev.stream_handle())
    c = int(count.item())
    last_path = "predicate"
    del keep
    return idx[:c], c


def compact_where(states, condition):
    """(``{k: v[condition(states)]}``, count): ``select_where`` then the row gathers."""
    n = next(iter(states.values())).shape[0]
    idx, count = select_where(states, condition)
    out = {}
    for k, v in states.items():
        if isinstance(v, torch.Tensor) and v.dim() >= 1 and v.shape[0] == n:
            out[k] = gather_rows(v, idx)
        else:
            out[k] = v
    return out, count
