"""Boolean expressions -> postfix programs (reference: network/expression.py:1-184).

Grammar, loosest binding first: OR (``|``, ``||``, ``OR``), AND (``&``, ``&&``, ``AND``), NOT
(``!``, ``NOT``), atoms (identifier, ``0``/``1``/``true``/``false`` in any case, parenthesised
expression). Binary operators associate to the left. Programs are two int32 lists, ops and
args: VAR a pushes node a, CONST a pushes a (0/1), NOT negates the top, AND/OR pop the top
two and push the result. The evaluator keeps the stack in one uint64, so depth <= 64.
"""

from __future__ import annotations

from dataclasses import dataclass

OP_VAR, OP_NOT, OP_AND, OP_OR, OP_CONST = 0, 1, 2, 3, 4

_SYMBOLS = {"||": "|", "&&": "&", "(": "(", ")": ")", "&": "&", "|": "|", "!": "!"}
_WORDS = {"and": "&", "or": "|", "not": "!"}


class ExpressionError(ValueError):
    pass


@dataclass(frozen=True)
class Var:
    name: str


@dataclass(frozen=True)
class Const:
    value: bool


@dataclass(frozen=True)
class Not:
    child: object


@dataclass(frozen=True)
class And:
    left: object
    right: object


@dataclass(frozen=True)
class Or:
    left: object
    right: object


def _is_ident_start(ch: str) -> bool:
    return ch.isascii() and (ch.isalpha() or ch == "_")


def _is_ident_char(ch: str) -> bool:
    return ch.isascii() and (ch.isalnum() or ch == "_")


def tokenize(text: str) -> list[str]:
    """Split into operator symbols, identifiers and digit runs (word operators normalised)."""
    tokens: list[str] = []
    s = text.strip()
    pos = 0
    while pos < len(s):
        ch = s[pos]
        if ch.isspace():
            pos += 1
            continue
        two = s[pos:pos + 2]
        if two in ("||", "&&"):
            tokens.append(_SYMBOLS[two])
            pos += 2
            continue
        if ch in _SYMBOLS:
            tokens.append(_SYMBOLS[ch])
            pos += 1
            continue
        if _is_ident_start(ch):
            end = pos + 1
            while end < len(s) and _is_ident_char(s[end]):
                end += 1
            word = s[pos:end]
            tokens.append(_WORDS.get(word.lower(), word))
            pos = end
            continue
        if ch.isdigit():
            end = pos + 1
            while end < len(s) and s[end].isdigit():
                end += 1
            tokens.append(s[pos:end])
            pos = end
            continue
        raise ExpressionError(f"cannot tokenize {s[pos:pos + 20]!r} in {text!r}")
    return tokens


class _Parser:
    def __init__(self, text: str):
        self.text = text
        self.tokens = tokenize(text)
        self.pos = 0

    def peek(self):
        return self.tokens[self.pos] if self.pos < len(self.tokens) else None

    def take(self, expected=None):
        tok = self.peek()
        if tok is None or (expected is not None and tok != expected):
            raise ExpressionError(f"expected {expected!r}, got {tok!r} in {self.text!r}")
        self.pos += 1
        return tok

    def expr_or(self):
        node = self.expr_and()
        while self.peek() == "|":
            self.take()
            node = Or(node, self.expr_and())
        return node

    def expr_and(self):
        node = self.expr_not()
        while self.peek() == "&":
            self.take()
            node = And(node, self.expr_not())
        return node

    def expr_not(self):
        if self.peek() == "!":
            self.take()
            return Not(self.expr_not())
        return self.atom()

    def atom(self):
        tok = self.take()
        if tok == "(":
            node = self.expr_or()
            self.take(")")
            return node
        if tok in ("0", "1"):
            return Const(tok == "1")
        if tok.lower() in ("true", "false"):
            return Const(tok.lower() == "true")
        if tok.isdigit():
            raise ExpressionError(f"unexpected number {tok!r} in {self.text!r}")
        if tok in ("|", "&", "!", ")"):
            raise ExpressionError(f"unexpected {tok!r} in {self.text!r}")
        return Var(tok)


def parse(text: str):
    """Expression text -> AST."""
    p = _Parser(text)
    node = p.expr_or()
    if p.peek() is not None:
        raise ExpressionError(f"trailing tokens {p.tokens[p.pos:]} in {text!r}")
    return node


def variables(node) -> set[str]:
    if isinstance(node, Var):
        return {node.name}
    if isinstance(node, Const):
        return set()
    if isinstance(node, Not):
        return variables(node.child)
    return variables(node.left) | variables(node.right)


def evaluate(node, state: dict) -> bool:
    """Reference evaluation with a name -> bool mapping."""
    if isinstance(node, Var):
        return bool(state[node.name])
    if isinstance(node, Const):
        return node.value
    if isinstance(node, Not):
        return not evaluate(node.child, state)
    if isinstance(node, And):
        return evaluate(node.left, state) and evaluate(node.right, state)
    return evaluate(node.left, state) or evaluate(node.right, state)


def compile_postfix(node, index: dict) -> tuple[list[int], list[int]]:
    """AST -> (ops, args) in post-order, node names resolved through ``index``."""
    ops: list[int] = []
    args: list[int] = []

    def walk(n):
        if isinstance(n, Var):
            if n.name not in index:
                raise ExpressionError(f"unknown node {n.name!r}")
            ops.append(OP_VAR)
            args.append(index[n.name])
        elif isinstance(n, Const):
            ops.append(OP_CONST)
            args.append(1 if n.value else 0)
        elif isinstance(n, Not):
            walk(n.child)
            ops.append(OP_NOT)
            args.append(0)
        else:
            walk(n.left)
            walk(n.right)
            ops.append(OP_AND if isinstance(n, And) else OP_OR)
            args.append(0)

    walk(node)
    return ops, args


def depth(node) -> int:
    """Stack depth the postfix evaluation needs (must stay <= 64)."""
    if isinstance(node, (Var, Const)):
        return 1
    if isinstance(node, Not):
        return depth(node.child)
    return max(depth(node.left), depth(node.right) + 1)
