"""Boolean network model: nodes, logic programs, MaBoSS rates, initial states, and the MaBoSS
(.bnd/.cfg) and BoolNet (.bnet) readers (reference: network/model.py:27-251).

Update semantics implemented by the kernels: asynchronous (uniform random single-node picks),
synchronous (all non-input nodes at once) and MaBoSS (Gillespie over ``rate_up``/``rate_down``,
each the pair (value when the logic is true, value when false)). Input nodes — no logic, or
all rates zero — never change on their own; the simulation clamps them.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from warpbiocell_gb300.network import expression as ex

MAX_WORDS = 4  # kernels hold up to 4 x 64 = 256 nodes per cell


class NetworkError(ValueError):
    pass


@dataclass
class Node:
    name: str
    logic: object | None = None
    rate_up: tuple[float, float] = (1.0, 0.0)
    rate_down: tuple[float, float] = (0.0, 1.0)
    p_on: float = 0.0

    @property
    def is_input(self) -> bool:
        return self.logic is None or (max(self.rate_up) == 0.0 and max(self.rate_down) == 0.0)


@dataclass
class BooleanNetwork:
    nodes: list[Node]
    source: str = ""
    variables: dict = field(default_factory=dict)

    def __post_init__(self):
        names = [n.name for n in self.nodes]
        if len(set(names)) != len(names):
            raise NetworkError("duplicate node names")
        if len(names) > 64 * MAX_WORDS:
            raise NetworkError(f"at most {64 * MAX_WORDS} nodes are supported, got {len(names)}")
        self.index = {name: i for i, name in enumerate(names)}
        for node in self.nodes:
            if node.logic is None:
                continue
            missing = ex.variables(node.logic) - set(self.index)
            if missing:
                raise NetworkError(f"node {node.name!r} references unknown nodes {sorted(missing)}")
            if ex.depth(node.logic) > 64:
                raise NetworkError(f"node {node.name!r}: expression nests deeper than 64")

    @property
    def names(self) -> list[str]:
        return [n.name for n in self.nodes]

    @property
    def n_nodes(self) -> int:
        return len(self.nodes)

    @property
    def n_words(self) -> int:
        return (self.n_nodes + 63) // 64

    @property
    def input_names(self) -> list[str]:
        return [n.name for n in self.nodes if n.is_input]

    def __getitem__(self, name: str) -> Node:
        return self.nodes[self.index[name]]

    def programs(self) -> dict[str, np.ndarray]:
        """Flattened postfix programs and per-node metadata (the kernels' arrays)."""
        ops: list[int] = []
        args: list[int] = []
        start: list[int] = []
        length: list[int] = []
        for node in self.nodes:
            start.append(len(ops))
            if node.logic is None:
                length.append(0)
                continue
            o, a = ex.compile_postfix(node.logic, self.index)
            ops += o
            args += a
            length.append(len(o))
        f32 = np.float32
        return {
            "ops": np.array(ops or [0], dtype=np.int32),
            "args": np.array(args or [0], dtype=np.int32),
            "start": np.array(start, dtype=np.int32),
            "length": np.array(length, dtype=np.int32),
            "updatable": np.array([i for i, n in enumerate(self.nodes) if not n.is_input], dtype=np.int32),
            "rate_up_true": np.array([n.rate_up[0] for n in self.nodes], dtype=f32),
            "rate_up_false": np.array([n.rate_up[1] for n in self.nodes], dtype=f32),
            "rate_down_true": np.array([n.rate_down[0] for n in self.nodes], dtype=f32),
            "rate_down_false": np.array([n.rate_down[1] for n in self.nodes], dtype=f32),
            "p_on": np.array([n.p_on for n in self.nodes], dtype=f32),
        }

    def truth_tables(self, programs: dict[str, np.ndarray] | None = None, max_inputs: int = 6) -> dict[str, np.ndarray]:
        """The truth tables of this network's programs (see :func:`truth_tables`)."""
        arrays = programs if programs is not None else self.programs()
        return truth_tables(arrays["ops"], arrays["args"], arrays["start"], arrays["length"], arrays["updatable"],
                            self.n_nodes, max_inputs)

    def targets(self, state: np.ndarray) -> np.ndarray:
        """Logic value of every node for a boolean state vector (inputs keep their state)."""
        mapping = {name: bool(state[i]) for name, i in self.index.items()}
        out = np.array(state, dtype=bool).copy()
        for i, node in enumerate(self.nodes):
            if not node.is_input:
                out[i] = ex.evaluate(node.logic, mapping)
        return out

    def synchronous_step(self, state: np.ndarray) -> np.ndarray:
        return self.targets(state)

    def pack(self, state: np.ndarray) -> np.ndarray:
        """Bool vector -> uint64 words (node i -> word i // 64, bit i % 64)."""
        bits = np.zeros(self.n_words * 64, dtype=np.uint8)
        bits[: self.n_nodes] = np.asarray(state, dtype=bool)
        return np.packbits(bits.reshape(self.n_words, 64), axis=1, bitorder="little").view("<u8").reshape(self.n_words)

    def unpack(self, words: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(np.asarray(words, dtype="<u8").reshape(self.n_words))
        bits = np.unpackbits(w.view(np.uint8), bitorder="little")
        return bits[: self.n_nodes].astype(bool)


# ---- readers ------------------------------------------------------------------------------------


def _strip_comments(text: str) -> str:
    """Remove // line comments and /* block */ comments."""
    out = []
    i = 0
    while i < len(text):
        if text.startswith("//", i):
            j = text.find("\n", i)
            i = len(text) if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = len(text) if j < 0 else j + 2
        else:
            out.append(text[i])
            i += 1
    return "".join(out)


def _is_word(s: str) -> bool:
    return bool(s) and all(c.isascii() and (c.isalnum() or c == "_") for c in s)


def _is_number(s: str) -> bool:
    return bool(s) and all(c in "+-0123456789.eE" for c in s)


def read_cfg(path: str | Path) -> tuple[dict[str, float], dict[str, float]]:
    """MaBoSS .cfg: ``$var = value;`` and ``NODE.istate = ...;`` / ``[NODE].istate = p0 [0], p1 [1];``
    statements -> (variables, p_on per node). Other statements (simulation settings) are ignored."""
    variables: dict[str, float] = {}
    p_on: dict[str, float] = {}
    for statement in _strip_comments(Path(path).read_text()).split(";"):
        s = statement.strip()
        if not s:
            continue
        lhs, eq, rhs = s.partition("=")
        if not eq:
            continue
        lhs, rhs = lhs.strip(), rhs.strip()
        if lhs.startswith("$") and _is_word(lhs[1:]) and _is_number(rhs):
            variables[lhs[1:]] = float(rhs)
            continue
        if lhs.endswith(".istate"):
            name = lhs[: -len(".istate")].strip()
            if name.startswith("["):
                name = name[1:]
            if name.endswith("]"):
                name = name[:-1]
            name = name.strip()
            if not _is_word(name):
                continue
            if rhs in ("0", "1"):
                p_on[name] = float(rhs)
                continue
            probs: dict[int, float] = {}
            for part in rhs.split(","):
                part = part.strip()
                if "[" not in part or not part.endswith("]"):
                    continue
                p, _, v = part[:-1].partition("[")
                v, p = v.strip(), p.strip()
                if v in ("0", "1") and _is_number(p):
                    probs[int(v)] = float(p)
            total = sum(probs.values()) or 1.0
            p_on[name] = probs.get(1, 0.0) / total
    return variables, p_on


def _number(token: str, variables: dict[str, float]) -> float:
    token = token.strip()
    if token.startswith("$"):
        if token[1:] not in variables:
            raise NetworkError(f"undefined variable {token} (is the .cfg file missing?)")
        return float(variables[token[1:]])
    try:
        return float(token)
    except ValueError as exc:
        raise NetworkError(f"cannot read rate {token!r}") from exc


def _rate(text: str, variables: dict[str, float], has_logic: bool) -> tuple[float, float]:
    """``@logic ? a : b`` -> (a, b); a plain number or $var -> (v, v)."""
    text = text.strip()
    if text.startswith("@logic"):
        rest = text[len("@logic"):].strip()
        if rest.startswith("?") and ":" in rest:
            a, _, b = rest[1:].partition(":")
            a, b = a.strip(), b.strip()
            if a and b and " " not in a and " " not in b:
                if not has_logic:
                    raise NetworkError(f"rate {text!r} refers to @logic on a node without logic")
                return _number(a, variables), _number(b, variables)
    v = _number(text, variables)
    return v, v


def _node_blocks(text: str):
    """Yield (name, body) for each ``node NAME { body }`` block (body up to the first '}')."""
    pos = 0
    while True:
        k = text.find("node", pos)
        if k < 0:
            return
        after = k + 4
        if (k > 0 and (text[k - 1].isalnum() or text[k - 1] == "_")) or after >= len(text) or not text[after].isspace():
            pos = k + 4
            continue
        j = after
        while j < len(text) and text[j].isspace():
            j += 1
        e = j
        while e < len(text) and (text[e].isalnum() or text[e] == "_"):
            e += 1
        name = text[j:e]
        b = e
        while b < len(text) and text[b].isspace():
            b += 1
        if not name or b >= len(text) or text[b] != "{":
            pos = k + 4
            continue
        close = text.find("}", b + 1)
        if close < 0:
            return
        yield name, text[b + 1:close]
        pos = close + 1


def read_bnd(path: str | Path, cfg: str | Path | None = None) -> BooleanNetwork:
    """MaBoSS .bnd with ``node NAME { logic = ...; rate_up = ...; rate_down = ...; }`` blocks."""
    text = _strip_comments(Path(path).read_text())
    variables, p_on = read_cfg(cfg) if cfg else ({}, {})
    nodes = []
    for name, body in _node_blocks(text):
        fields: dict[str, str] = {}
        for statement in body.split(";"):
            s = statement.strip()
            if s:
                key, _, value = s.partition("=")
                fields[key.strip()] = value.strip()
        logic = ex.parse(fields["logic"]) if "logic" in fields else None
        up_default = "@logic ? 1 : 0" if logic is not None else "0"
        down_default = "@logic ? 0 : 1" if logic is not None else "0"
        rate_up = _rate(fields.get("rate_up", up_default), variables, logic is not None)
        rate_down = _rate(fields.get("rate_down", down_default), variables, logic is not None)
        nodes.append(Node(name=name, logic=logic, rate_up=rate_up, rate_down=rate_down, p_on=p_on.get(name, 0.0)))
    if not nodes:
        raise NetworkError(f"no node blocks found in {path}")
    return BooleanNetwork(nodes, source=str(path), variables=variables)


def read_bnet(path: str | Path) -> BooleanNetwork:
    """BoolNet .bnet: ``target, factors`` lines; ``A, A`` (or a missing rule) marks an input."""
    nodes: dict[str, Node] = {}
    for raw in Path(path).read_text().splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line or line.lower().replace(" ", "").startswith("targets,factors"):
            continue
        name, _, rule = line.partition(",")
        name, rule = name.strip(), rule.strip()
        if not name or not rule:
            raise NetworkError(f"cannot read line {raw!r}")
        logic = None if rule == name else ex.parse(rule)
        active = logic is not None
        nodes[name] = Node(name=name, logic=logic, rate_up=(1.0, 0.0) if active else (0.0, 0.0),
                           rate_down=(0.0, 1.0) if active else (0.0, 0.0))
    if not nodes:
        raise NetworkError(f"no rules found in {path}")
    return BooleanNetwork(list(nodes.values()), source=str(path))


def load_network(path: str | Path, cfg: str | Path | None = None) -> BooleanNetwork:
    path = Path(path)
    if path.suffix == ".bnet":
        return read_bnet(path)
    if path.suffix == ".bnd":
        return read_bnd(path, cfg)
    raise NetworkError(f"unknown network format {path.suffix!r} (use .bnd or .bnet)")


_MASK64 = (1 << 64) - 1


def run_postfix(ops: list[int], args: list[int], value: dict[int, int]) -> int:
    """One program on one state, with the kernels' stack semantics (kernels/network_kernels.py:50-78
    as restated in csrc/wbc_network.cu): a 64-bit stack word, top = bit 0; VAR and CONST push (a
    CONST pushes its argument as a 64-bit two's-complement word), NOT flips the top, AND / OR pop
    the top and combine it into the new top; unknown opcodes do nothing."""
    stack = 0
    for op, a in zip(ops, args):
        if op == 0:
            stack = ((stack << 1) | value[a]) & _MASK64
        elif op == 4:
            stack = ((stack << 1) | (a & _MASK64)) & _MASK64
        elif op == 1:
            stack ^= 1
        elif op == 2:
            top = stack & 1
            stack >>= 1
            stack = (stack & ~1 & _MASK64) | ((stack & 1) & top)
        elif op == 3:
            top = stack & 1
            stack >>= 1
            stack = (stack & ~1 & _MASK64) | ((stack & 1) | top)
    return stack & 1


def truth_tables(ops, args, start, length, updatable, n_nodes: int, max_inputs: int = 6) -> dict[str, np.ndarray]:
    """Per node, the truth table of its postfix program when the node is updatable and its program
    reads at most ``max_inputs`` (<= 6) distinct nodes: ``arity`` (-1 = no table), ``inputs`` (6
    node ids per node, unused ones 0) and ``bits`` (bit b = the program's value when input j holds
    bit j of b). Every entry comes from running the program with the kernels' postfix semantics
    (:func:`run_postfix`), so a table and its program agree on every state."""
    if not 0 <= max_inputs <= 6:
        raise ValueError("max_inputs must be within [0, 6]")
    arity = np.full(n_nodes, -1, dtype=np.int32)
    inputs = np.zeros((n_nodes, 6), dtype=np.int32)
    bits = np.zeros(n_nodes, dtype=np.uint64)
    for node in sorted({int(u) for u in np.asarray(updatable).tolist()}):
        if length[node] == 0:
            continue
        o = [int(v) for v in ops[start[node]:start[node] + length[node]]]
        a = [int(v) for v in args[start[node]:start[node] + length[node]]]
        reads = sorted({arg for op, arg in zip(o, a) if op == 0})
        if len(reads) > max_inputs or any(not 0 <= r < n_nodes for r in reads):
            continue
        table = 0
        for pattern in range(1 << len(reads)):
            value = {r: (pattern >> j) & 1 for j, r in enumerate(reads)}
            table |= run_postfix(o, a, value) << pattern
        arity[node] = len(reads)
        inputs[node, :len(reads)] = reads
        bits[node] = table
    return {"arity": arity, "inputs": inputs.reshape(-1), "bits": bits}
