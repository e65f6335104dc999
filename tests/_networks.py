"""Shared test helper: a BooleanNetwork whose postfix programs are exactly the reference's
MicroC programs (from the golden fixture network_microc.npz), with the fixture's MaBoSS rates."""

import numpy as np

from warpbiocell_gb300.network import expression as ex
from warpbiocell_gb300.network.model import BooleanNetwork, Node


def microc_network(golden, rates: bool = False) -> BooleanNetwork:
    """A BooleanNetwork whose programs are exactly the reference's MicroC programs."""
    g = golden("network_microc")
    names = [str(x) for x in g["names"]]
    ops, args, start, length = g["prog_ops"], g["prog_args"], g["prog_start"], g["prog_length"]
    updatable = set(g["prog_updatable"].tolist())
    p_on = g["prog_p_on"]

    def to_ast(node):
        stack = []
        for op, a in zip(ops[start[node]:start[node] + length[node]], args[start[node]:start[node] + length[node]]):
            if op == ex.OP_VAR:
                stack.append(ex.Var(names[a]))
            elif op == ex.OP_CONST:
                stack.append(ex.Const(bool(a)))
            elif op == ex.OP_NOT:
                stack.append(ex.Not(stack.pop()))
            else:
                b, a2 = stack.pop(), stack.pop()
                stack.append(ex.And(a2, b) if op == ex.OP_AND else ex.Or(a2, b))
        return stack[0]

    nodes = []
    for i, name in enumerate(names):
        if i in updatable and rates:
            nodes.append(Node(name, to_ast(i), rate_up=(float(g["prog_rate_up_true"][i]), float(g["prog_rate_up_false"][i])),
                              rate_down=(float(g["prog_rate_down_true"][i]), float(g["prog_rate_down_false"][i])),
                              p_on=float(p_on[i])))
        elif i in updatable:
            nodes.append(Node(name, to_ast(i), p_on=float(p_on[i])))
        else:
            logic = to_ast(i) if length[i] > 0 else None
            nodes.append(Node(name, logic, rate_up=(0.0, 0.0), rate_down=(0.0, 0.0), p_on=float(p_on[i])))
    net = BooleanNetwork(nodes)
    for key in ("ops", "args", "start", "length", "updatable"):
        np.testing.assert_array_equal(net.programs()[key], g[f"prog_{key}"])
    return net


