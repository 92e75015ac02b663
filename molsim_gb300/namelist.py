"""Fortran namelist input, the format of the reference's `<project>.in` files.

A file is a sequence of groups `&nmlName var = values, ... /`.  This parser
reads the forms those files use: scalars and value lists, repeat counts
(`3*100.0`, `2*` for null values), element and section assignments of arrays
(`npptct(1,2) = 20`, `zat(2) = -1.0, 1.0`), derived-type values given as a
list (`bond = 2.5, 2, 5.0`) or by component (`bond%k = 2.5`), strings in
single or double quotes, logicals (`.t.`, `.false.`, `T`), integers and reals
(`1.0d-5`), and `!` comments.  Names are case-insensitive and stored in lower
case.

Each variable maps to a `Var`: the values of a whole-variable assignment in
order (`Var.values`) and the element assignments by 1-based index tuple
(`Var.items`).  `array()` expands a variable to a full Fortran array with a
default, column-major for more than one dimension, as a namelist read into a
preset array would.
"""
from dataclasses import dataclass, field
import re
from typing import Dict, List, Optional, Tuple

import numpy as np

__all__ = ["Var", "BadGroup", "NamelistError", "parse_namelists", "read_namelists", "scalar", "array"]


class NamelistError(ValueError):
    pass


@dataclass
class Var:
    values: Optional[List] = None                           # name = v1, v2, ...
    items: Dict[Tuple[int, ...], List] = field(default_factory=dict)   # name(i[,j]) = v1, ...


_NULL = object()   # a null value (r* or an empty slot): keeps the preset value


def _strip_comments(text):
    out, quote = [], None
    for line in text.splitlines():
        buf = []
        for ch in line:
            if quote:
                buf.append(ch)
                if ch == quote:
                    quote = None
            elif ch in "'\"":
                quote = ch
                buf.append(ch)
            elif ch == "!":
                break
            else:
                buf.append(ch)
        out.append("".join(buf))
    return "\n".join(out)


_TOKEN = re.compile(r"""
    (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
  | (?P<group>[&$][A-Za-z_]\w*)
  | (?P<end>/|[&$]end\b)
  | (?P<lhs>[A-Za-z_]\w*(?:\s*\([^()=]*\)|%\w+)*\s*=)
  | (?P<sep>,)
  | (?P<word>[^\s,/'"=]+)
""", re.VERBOSE | re.IGNORECASE)


def _value(word):
    w = word.strip()
    lw = w.lower()
    if re.fullmatch(r"[+-]?\d+", w):
        return int(w)
    if re.fullmatch(r"[+-]?(\d+\.?\d*|\.\d+)([edq][+-]?\d+)?", lw):
        return float(re.sub(r"[dq]", "e", lw))
    if lw in (".t.", ".true.", "t", "true"):
        return True
    if lw in (".f.", ".false.", "f", "false"):
        return False
    if lw.startswith(".t"):
        return True
    if lw.startswith(".f"):
        return False
    raise NamelistError(f"cannot read value {word!r}")


def _values(tokens):
    """(kind, text) tokens of one right-hand side -> a list of values with
    repeat counts expanded (null values as _NULL)."""
    vals, pending, last_sep = [], None, True
    for kind, text in tokens:
        if kind == "sep":
            if last_sep:
                vals.append(_NULL)     # empty slot: a null value
            last_sep = True
            continue
        if kind == "str":
            q = text[0]
            v = text[1:-1].replace(q + q, q)
            vals.append(v)
            last_sep = False
            continue
        m = re.fullmatch(r"(\d+)\*(.*)", text)
        if m:
            n, rest = int(m.group(1)), m.group(2)
            vals.extend([_NULL if rest == "" else _value(rest)] * n)
        else:
            vals.append(_value(text))
        last_sep = False
    return vals


def _lhs(text):
    """(name, index tuple or None) of an assignment's left side; a section
    (a(1:3)) or a component of an element (v(2)%l) gives (text, 'raw')."""
    t = text.strip()[:-1].strip()
    m = re.fullmatch(r"([A-Za-z_][\w%]*)\s*(?:\(([^)]*)\))?", t)
    if m is None:
        return t.lower(), "raw"
    name = m.group(1).lower()
    if m.group(2) is None:
        return name, None
    parts = [p.strip() for p in m.group(2).split(",")]
    if any(not re.fullmatch(r"[+-]?\d+", p) for p in parts):
        return t.lower(), "raw"
    return name, tuple(int(p) for p in parts)


class BadGroup:
    """A group that does not parse.  The reference reads a group only when
    its routine needs it, so a malformed group it never reads is harmless;
    here the error is raised when the group is used."""

    def __init__(self, name, err):
        self.name, self.err = name, err

    def __getattr__(self, attr):
        raise NamelistError(f"&{self.name}: {self.err}")

    def get(self, *a, **k):
        raise NamelistError(f"&{self.name}: {self.err}")

    def __contains__(self, key):
        raise NamelistError(f"&{self.name}: {self.err}")


def _parse_group(name, tokens):
    group: Dict[str, Var] = {}
    var = idx = None
    rhs: List[Tuple[str, str]] = []

    def flush():
        nonlocal var, idx, rhs
        if var is None:
            return
        vals = _values(rhs)
        if idx == "raw":   # sections and element components: kept as text, values as read
            group.setdefault("__raw__", Var(items={})).items[(var,)] = vals
        else:
            v = group.setdefault(var, Var())
            if idx is None:
                v.values = vals
            else:
                v.items[idx] = vals
        var, idx, rhs = None, None, []

    for kind, tok in tokens:
        if kind == "lhs":
            flush()
            var, idx = _lhs(tok)
        elif var is None:
            if kind != "sep":
                raise NamelistError(f"value {tok!r} without a variable in &{name}")
        else:
            rhs.append((kind, tok))
    flush()
    return group


def parse_namelists(text) -> Dict[str, Dict[str, Var]]:
    """All groups of a namelist file: {group: {variable: Var}} (lower case).
    A group runs to its '/' (or '&end'), or to the next group when its '/'
    is missing; a group that does not parse is kept as a BadGroup."""
    text = _strip_comments(text)
    groups: Dict[str, Dict[str, Var]] = {}
    cur, toks, closed = None, [], False

    def finish():
        nonlocal cur, toks
        if cur is None:
            return
        try:
            groups[cur] = _parse_group(cur, toks)
            if not closed:
                raise NamelistError("not closed by /")
        except NamelistError as e:
            groups[cur] = BadGroup(cur, str(e))
        cur, toks = None, []

    for m in _TOKEN.finditer(text):
        kind = m.lastgroup
        tok = m.group(kind)
        if kind == "group":
            finish()
            cur, closed = tok[1:].lower(), False
            continue
        if cur is None:
            continue   # text between groups is ignored
        if kind == "end":
            closed = True
            finish()
        else:
            toks.append((kind, tok))
    finish()
    return groups


def read_namelists(path):
    with open(path) as f:
        return parse_namelists(f.read())


def scalar(group: Dict[str, Var], name, default=None):
    """The value of a scalar variable (its first value), or default."""
    v = group.get(name.lower())
    if v is None or not v.values or v.values[0] is _NULL:
        return default
    return v.values[0]


def array(group: Dict[str, Var], name, shape, default, dtype=float):
    """A Fortran array of the given shape (1-based indices in the file),
    preset to default and overwritten by the assignments in file order:
    whole-variable values fill it in column-major order, an element
    assignment name(i,j) = v1, v2, ... fills from (i,j) onwards."""
    shape = (shape,) if np.isscalar(shape) else tuple(shape)
    flat = np.full(int(np.prod(shape)), default, dtype=object)
    v = group.get(name.lower())

    def put(start, vals):
        for k, x in enumerate(vals):
            if start + k >= flat.size:
                raise NamelistError(f"{name}: more values than elements")
            if x is not _NULL:
                flat[start + k] = x

    if v is not None:
        if v.values is not None:
            put(0, v.values)
        for idx, vals in v.items.items():
            if len(idx) != len(shape):
                raise NamelistError(f"{name}{idx}: rank differs from {shape}")
            off, stride = 0, 1
            for i, n in zip(idx, shape):
                if not 1 <= i <= n:
                    raise NamelistError(f"{name}{idx} outside {shape}")
                off += (i - 1) * stride
                stride *= n
            put(off, vals)
    out = np.array(flat.tolist(), dtype=dtype)
    return out.reshape(shape, order="F")
