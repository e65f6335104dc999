"""Seeded random Boolean networks written as logic expressions.

The metabolic + gene-network workload gives every non-input node a random truth table over 2-4
distinct other nodes. To stay within the reference's model format, each table is written as a
disjunctive normal form (the OR of the minterms whose output is 1) and parsed by the same
expression compiler as a MaBoSS or BoolNet file (``network/expression.py``), so the kernels
evaluate ordinary postfix programs. Constant tables become ``0`` / ``1``.
"""

from __future__ import annotations

import numpy as np

from warpbiocell_gb300.network import expression as ex
from warpbiocell_gb300.network.model import BooleanNetwork, Node

FATE_NAMES = ("Proliferation", "Apoptosis", "Growth_Arrest", "Necrosis")


def dnf(inputs: list[str], table: np.ndarray) -> str:
    """Expression text of a truth table: row r of ``table`` is the output for the assignment whose
    bit b (of r) is the value of ``inputs[b]``."""
    rows = [r for r in range(len(table)) if table[r]]
    if not rows:
        return "0"
    if len(rows) == len(table):
        return "1"
    terms = []
    for r in rows:
        lits = [name if (r >> b) & 1 else f"!{name}" for b, name in enumerate(inputs)]
        terms.append("(" + " & ".join(lits) + ")")
    return " | ".join(terms)


def random_truth_table_network(n_nodes: int = 106, input_names: tuple[str, ...] = ("Oxygen_supply", "Glucose_supply"),
                               seed: int = 0, min_inputs: int = 2, max_inputs: int = 4,
                               p_on: float = 0.5) -> BooleanNetwork:
    """``n_nodes`` nodes: the named inputs (no logic), four fate nodes, the rest generic genes;
    every non-input node reads ``min_inputs``..``max_inputs`` distinct other nodes through a random
    truth table. Non-input nodes start ON with probability ``p_on``, inputs OFF."""
    rng = np.random.default_rng(seed)
    n_inputs = len(input_names)
    if n_nodes < n_inputs + len(FATE_NAMES) + 1:
        raise ValueError("too few nodes")
    names = list(input_names) + list(FATE_NAMES) + [f"G{k:03d}" for k in range(n_nodes - n_inputs - len(FATE_NAMES))]
    nodes = [Node(name) for name in input_names]
    for idx in range(n_inputs, n_nodes):
        k = int(rng.integers(min_inputs, max_inputs + 1))
        others = [j for j in range(n_nodes) if j != idx]
        chosen = [names[j] for j in rng.choice(others, size=k, replace=False)]
        table = rng.random(1 << k) < 0.5
        nodes.append(Node(names[idx], ex.parse(dnf(chosen, table)), p_on=p_on))
    return BooleanNetwork(nodes, source=f"random truth tables (seed {seed})")
