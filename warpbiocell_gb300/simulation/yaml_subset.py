"""The YAML subset of experiment and sweep files, for machines without PyYAML.

``safe_load`` uses PyYAML when it is importable and otherwise parses block mappings and block
sequences (``key: value``, ``- item``, items that are mappings), flow sequences and mappings
(``[1, 2]``, ``{a: 1}``), quoted and plain scalars, and ``#`` comments. Plain scalars resolve as
YAML 1.1 does for the values these files hold: ``true/false/yes/no/on/off``, ``null``/``~``,
integers, and floats written with a decimal point or an exponent (``7.2e6`` included; PyYAML
leaves that one a string, which the configuration loader converts anyway). Anchors, tags,
multi-document streams and block scalars (``|``, ``>``) are not supported and raise ValueError.
"""

from __future__ import annotations

import re

try:  # pragma: no cover - depends on the machine
    import yaml as _pyyaml
except ImportError:  # pragma: no cover
    _pyyaml = None

_INT = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9][0-9_]*(\.[0-9_]*)?)([eE][-+]?[0-9]+)?$")
_BOOL = {"true": True, "yes": True, "on": True, "false": False, "no": False, "off": False}


def safe_load(text: str):
    if _pyyaml is not None:
        return _pyyaml.safe_load(text)
    return _Parser(text).document()


def safe_dump(value, default_flow_style: bool = False) -> str:
    """Enough of YAML's emitter for configuration dicts (block style) and override values (flow)."""
    if _pyyaml is not None:
        return _pyyaml.safe_dump(value, default_flow_style=default_flow_style, sort_keys=False)
    if default_flow_style or not isinstance(value, dict):
        return _flow(value) + "\n"
    return "".join(_block(value, 0))


def scalar(text: str):
    """A plain or quoted scalar, or a flow collection, as in an override ``key=value``."""
    text = text.strip()
    if _pyyaml is not None:
        return _pyyaml.safe_load(text)
    if not text:
        return None
    value, rest = _Flow(text).value()
    if rest.strip():
        raise ValueError(f"unexpected text after a value: {rest!r}")
    return value


# ---- emitter ------------------------------------------------------------------------------------

def _flow(v) -> str:
    if v is None:
        return "null"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, float)):
        return repr(v)
    if isinstance(v, str):
        plain = v and not re.search(r"[:#\[\]{},'\"]|^\s|\s$", v) and _plain(v) == v
        return v if plain else "'" + v.replace("'", "''") + "'"
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_flow(x) for x in v) + "]"
    if isinstance(v, dict):
        return "{" + ", ".join(f"{_flow(k)}: {_flow(x)}" for k, x in v.items()) + "}"
    return _flow(str(v))


def _block(d: dict, indent: int):
    pad = " " * indent
    for k, v in d.items():
        if isinstance(v, dict) and v:
            yield f"{pad}{_flow(k)}:\n"
            yield from _block(v, indent + 2)
        elif isinstance(v, (list, tuple)) and v and any(isinstance(x, dict) for x in v):
            yield f"{pad}{_flow(k)}:\n"
            for item in v:
                if isinstance(item, dict) and item:
                    lines = list(_block(item, indent + 4))
                    lines[0] = f"{pad}  - " + lines[0].lstrip()
                    yield from lines
                else:
                    yield f"{pad}  - {_flow(item)}\n"
        else:
            yield f"{pad}{_flow(k)}: {_flow(v)}\n"


# ---- parser -------------------------------------------------------------------------------------

def _plain(token: str):
    t = token.strip()
    low = t.lower()
    if low in ("null", "~", ""):
        return None
    if low in _BOOL:
        return _BOOL[low]
    if _INT.match(t):
        return int(t.replace("_", ""))
    if _FLOAT.match(t) and any(c.isdigit() for c in t):
        return float(t.replace("_", ""))
    if low in (".inf", "+.inf"):
        return float("inf")
    if low == "-.inf":
        return float("-inf")
    if low == ".nan":
        return float("nan")
    return t


def _strip_comment(line: str) -> str:
    quote = None
    for i, c in enumerate(line):
        if quote:
            if c == quote:
                quote = None
        elif c in "'\"":
            quote = c
        elif c == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i].rstrip()
    return line.rstrip()


class _Flow:
    """Flow values: [..], {..}, quoted strings, plain scalars (ending at , ] } in a collection)."""

    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def _ws(self):
        while self.i < len(self.s) and self.s[self.i] in " \t":
            self.i += 1

    def value(self, in_collection: bool = False):
        self._ws()
        if self.i >= len(self.s):
            return None, ""
        c = self.s[self.i]
        if c == "[":
            self.i += 1
            out = []
            while True:
                self._ws()
                if self.s[self.i:self.i + 1] == "]":
                    self.i += 1
                    break
                v, _ = self.value(True)
                out.append(v)
                self._ws()
                if self.s[self.i:self.i + 1] == ",":
                    self.i += 1
                elif self.s[self.i:self.i + 1] != "]":
                    raise ValueError(f"bad flow sequence: {self.s!r}")
            return out, self.s[self.i:]
        if c == "{":
            self.i += 1
            out = {}
            while True:
                self._ws()
                if self.s[self.i:self.i + 1] == "}":
                    self.i += 1
                    break
                k, _ = self.value(True)
                self._ws()
                if self.s[self.i:self.i + 1] != ":":
                    raise ValueError(f"bad flow mapping: {self.s!r}")
                self.i += 1
                v, _ = self.value(True)
                out[k] = v
                self._ws()
                if self.s[self.i:self.i + 1] == ",":
                    self.i += 1
                elif self.s[self.i:self.i + 1] != "}":
                    raise ValueError(f"bad flow mapping: {self.s!r}")
            return out, self.s[self.i:]
        if c in "'\"":
            j = self.i + 1
            buf = []
            while j < len(self.s):
                if self.s[j] == c:
                    if c == "'" and self.s[j + 1:j + 2] == "'":
                        buf.append("'")
                        j += 2
                        continue
                    break
                if c == '"' and self.s[j] == "\\" and j + 1 < len(self.s):
                    buf.append({"n": "\n", "t": "\t"}.get(self.s[j + 1], self.s[j + 1]))
                    j += 2
                    continue
                buf.append(self.s[j])
                j += 1
            else:
                raise ValueError(f"unterminated string: {self.s!r}")
            self.i = j + 1
            return "".join(buf), self.s[self.i:]
        j = self.i
        stops = ",]}" if in_collection else ""
        while j < len(self.s) and self.s[j] not in stops:
            if in_collection and self.s[j] == ":" and (j + 1 == len(self.s) or self.s[j + 1] in " \t"):
                break
            j += 1
        token = self.s[self.i:j]
        self.i = j
        return _plain(token), self.s[self.i:]


class _Parser:
    def __init__(self, text: str):
        self.lines = []
        for raw in text.splitlines():
            if raw.strip() in ("---", "...") or raw.lstrip().startswith("%"):
                continue
            line = _strip_comment(raw.replace("\t", "    "))
            if line.strip():
                self.lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
        self.k = 0

    def document(self):
        if not self.lines:
            return None
        value = self.node(self.lines[0][0])
        if self.k != len(self.lines):
            raise ValueError(f"unexpected indentation at {self.lines[self.k][1]!r}")
        return value

    def node(self, indent: int):
        _, text = self.lines[self.k]
        if text.startswith("- ") or text == "-":
            return self.sequence(indent)
        if _key_split(text) is not None:
            return self.mapping(indent)
        self.k += 1
        return scalar(text)

    def mapping(self, indent: int) -> dict:
        out = {}
        while self.k < len(self.lines):
            ind, text = self.lines[self.k]
            if ind < indent:
                break
            if ind > indent:
                raise ValueError(f"unexpected indentation at {text!r}")
            split = _key_split(text)
            if split is None:
                break
            key, rest = split
            self.k += 1
            out[key] = self.after_key(rest, ind)
        return out

    def after_key(self, rest: str, ind: int):
        if rest and rest[0] in "|>&!*":
            raise ValueError(f"unsupported YAML construct: {rest!r}")
        if rest:
            return scalar(rest)
        if self.k < len(self.lines):
            nind, ntext = self.lines[self.k]
            if nind > ind or (nind == ind and ntext.startswith("-")):
                return self.node(nind)
        return None

    def sequence(self, indent: int) -> list:
        out = []
        while self.k < len(self.lines):
            ind, text = self.lines[self.k]
            if ind != indent or not (text.startswith("- ") or text == "-"):
                break
            item = text[1:].strip()
            if not item:
                self.k += 1
                out.append(self.node(self.lines[self.k][0]) if self.k < len(self.lines) and
                           self.lines[self.k][0] > indent else None)
                continue
            if _key_split(item) is not None and item[0] not in "[{'\"":
                # a mapping whose first key sits on the dash line: re-read it at its own column
                column = ind + 1 + (len(text) - 1 - len(text[1:].lstrip(" ")))
                self.lines[self.k] = (column, item)
                out.append(self.mapping(column))
            else:
                self.k += 1
                out.append(scalar(item))
        return out


def _key_split(text: str):
    """(key, rest) when ``text`` is ``key: rest`` / ``key:``, else None."""
    if text[0] in "[{":
        return None
    if text[0] in "'\"":
        f = _Flow(text)
        key, rest = f.value()
        rest = rest.lstrip()
        if rest.startswith(":") and (len(rest) == 1 or rest[1] in " \t"):
            return key, rest[1:].strip()
        return None
    m = re.match(r"^([^:#]+?)\s*:(\s+|$)(.*)$", text)
    if not m:
        return None
    return m.group(1).strip(), m.group(3).strip()
