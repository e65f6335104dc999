"""Generate the golden fixtures in this folder from the reference's own Python code.

The reference (Gennappio/WarpBioCell) needs NVIDIA Warp to run its kernels, which is not
installable here; its numpy references (src/warpbiocell/reference/fields.py, mechanics.py), its
network readers and compiler (network/model.py, network/expression.py) and its initial-condition
helper (cells/initialization.py) only touch Warp through decorators and constants at import
time. This script therefore installs a minimal stand-in module named ``warp`` (decorators return
the function, ``constant`` returns its value) and imports those modules from the reference tree.

Run from the repository root:  python tests/golden/make_golden.py [/path/to/reference]
Outputs (committed): tests/golden/*.npz. The tests never import the reference.
"""

from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# The reference project's checkout: the first argument, else $WBC_REFERENCE_ROOT.
_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WBC_REFERENCE_ROOT")
if not _root:
    sys.exit(f"usage: {Path(__file__).name} <reference checkout> (or set WBC_REFERENCE_ROOT)")
REFERENCE = Path(_root)


class _Anything:
    def __call__(self, *args, **kwargs):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __getitem__(self, key):
        return _Anything()


def _install_warp_stand_in() -> None:
    stub = types.ModuleType("warp")
    stub.constant = lambda value: value
    stub.kernel = lambda fn=None, **kw: fn if fn is not None else (lambda f: f)
    stub.func = lambda fn=None, **kw: fn if fn is not None else (lambda f: f)
    stub.__getattr__ = lambda name: _Anything()
    sys.modules["warp"] = stub


def main() -> None:
    _install_warp_stand_in()
    sys.path.insert(0, str(REFERENCE / "src"))
    from warpbiocell.cells.initialization import spherical_cluster
    from warpbiocell.fields.scalar_field import Boundary
    from warpbiocell.network import expression as ex
    from warpbiocell.network.model import load_network, read_bnd
    from warpbiocell.reference import fields as rf
    from warpbiocell.reference import mechanics as rm

    # 1. initial conditions
    clusters = {}
    for k, (n, r, sp, jit, seed) in enumerate([(600, 8.0, 0.85, 0.3, 11), (400, 8.0, 1.0, 0.2, 5), (1000, 8.0, 0.9, 0.1, 0),
                                               (300, 8.0, 1.0, 0.3, 4), (257, 6.5, 0.95, 0.15, 3)]):
        clusters[f"c{k}"] = spherical_cluster(n, r, spacing_factor=sp, jitter=jit, seed=seed)
        clusters[f"c{k}_args"] = np.array([n, r, sp, jit, seed], dtype=np.float64)
    np.savez_compressed(HERE / "spherical_cluster.npz", **clusters)

    # 2. deposit: per-state densities of a mixed population (300 cells, 20 um voxels)
    rng = np.random.default_rng(4)
    pos = spherical_cluster(300, 8.0, spacing_factor=1.0, jitter=0.3, seed=4)
    pos = np.vstack([pos, np.array([[500.0, 0.0, 0.0], [0.0, -149.0, 0.0], [149.9, 149.9, 149.9]], np.float32)])
    states = rng.integers(0, 4, size=pos.shape[0]).astype(np.int32)
    origin, dx, shape = (-150.0, -150.0, -150.0), 20.0, (16, 16, 16)
    dens = np.stack([rf.deposit_reference(pos, states == s, origin, dx, shape) for s in range(4)])
    np.savez_compressed(HERE / "deposit.npz", positions=pos, states=states, origin=np.array(origin), dx=dx,
                        shape=np.array(shape), density=dens)

    # 3. sampling: random field, positions inside and outside the grid
    rng = np.random.default_rng(1)
    field = rng.uniform(0.0, 40.0, size=(9, 8, 7))
    spos = np.vstack([rng.uniform(-100.0, 120.0, size=(300, 3)), [[1000.0, 0.0, 0.0], [0.0, -1000.0, 5.0]]]).astype(np.float32)
    origin_s, dx_s = (-60.0, -50.0, -40.0), 25.0
    np.savez_compressed(HERE / "sample.npz", field=field.astype(np.float32), positions=spos, origin=np.array(origin_s),
                        dx=dx_s, expected=rf.sample_reference(field.astype(np.float32), spos, origin_s, dx_s))

    # 4. exact discrete steady states (dense solve + Picard)
    mixed = (Boundary.DIRICHLET, Boundary.NEUMANN, Boundary.DIRICHLET)
    rng = np.random.default_rng(3)
    d1 = rng.uniform(0.0, 2.0e-3, size=(8, 7, 6)).astype(np.float32)
    exact1 = rf.steady_state_reference(np.full((8, 7, 6), 20.0), d1, 2.0e3, 5.0e4, 3.0, 10.0, mixed)
    rng = np.random.default_rng(8)
    d2 = rng.uniform(0.0, 1.5e-3, size=(9, 9, 9)).astype(np.float32)
    prod2 = rng.uniform(0.0, 50.0, size=(9, 9, 9)).astype(np.float32)
    src2 = rng.uniform(0.0, 5.0, size=(9, 9, 9)).astype(np.float32)
    exact2 = rf.steady_state_reference(np.full((9, 9, 9), 1.0), d2, 2.4e5, 3.0e4, 1.0, 15.0, (Boundary.DIRICHLET,) * 3,
                                       production=prod2, source=src2, source_k=0.04)
    rng = np.random.default_rng(2)
    v3 = rng.uniform(5.0, 20.0, size=(7, 6, 5))
    d3 = rng.uniform(0.0, 1.0e-3, size=(7, 6, 5))
    dt3 = 0.9 * 10.0**2 / (6.0 * 2.0e3)
    ftcs = [v3.astype(np.float32).astype(np.float64)]
    for _ in range(5):
        ftcs.append(rf.ftcs_step_reference(ftcs[-1], d3.astype(np.float32), 2.0e3, 5.0e4, 3.0, 10.0, dt3, mixed))
    np.savez_compressed(HERE / "steady_state.npz", density1=d1, exact1=exact1, density2=d2, production2=prod2,
                        source2=src2, exact2=exact2, ftcs_values=v3.astype(np.float32), ftcs_density=d3.astype(np.float32),
                        ftcs_dt=dt3, ftcs_steps=np.stack(ftcs))

    # 5. contact velocities and neighbour counts (O(N^2))
    rng = np.random.default_rng(9)
    cpos = spherical_cluster(400, 8.0, spacing_factor=0.85, jitter=0.3, seed=9)
    cr = rng.uniform(6.0, 9.0, size=400).astype(np.float32)
    vel, counts = rm.contact_velocities_reference(cpos, cr, 10.0, 2 * 9.0 + 0.5)
    steps = [cpos.astype(np.float64)]
    for _ in range(20):
        steps.append(rm.contact_substep_reference(steps[-1], cr, 10.0, 2 * 9.0 + 0.5, 0.01))
    np.savez_compressed(HERE / "contact.npz", positions=cpos, radii=cr, rate=10.0, query_radius=18.5, velocities=vel,
                        counts=counts, dt=0.01, trajectory=np.stack(steps))

    # 6. Boolean networks: the MicroC network's programs and synchronous steps on random states
    net_dir = REFERENCE / "configs" / "networks"
    net = load_network(net_dir / "microc_jaya.bnd", net_dir / "microc_jaya.cfg")
    prog = net.programs()
    rng = np.random.default_rng(5)
    states = rng.random((256, net.n_nodes)) < 0.5
    words = np.stack([net.pack(row) for row in states])
    step1 = np.stack([net.synchronous_step(row) for row in states])
    step2 = np.stack([net.synchronous_step(row) for row in step1])
    np.savez_compressed(HERE / "network_microc.npz", names=np.array(net.names), input_names=np.array(net.input_names),
                        words=words, states=states, step1=step1, step2=step2,
                        step1_words=np.stack([net.pack(r) for r in step1]),
                        step2_words=np.stack([net.pack(r) for r in step2]), **{f"prog_{k}": v for k, v in prog.items()})

    # 7. readers and compiler on synthetic model text (written for these fixtures)
    bnd = HERE / "toy_network.bnd"
    cfg = HERE / "toy_network.cfg"
    bnd_text = bnd.read_text()
    toy = read_bnd(bnd, cfg)
    tp = toy.programs()
    exprs = ["A & !B", "!(A | B) | C", "A && B || !C", "A AND NOT B", "!!A", "1", "A | 0",
             "(A & !B) | (C & (B | !A)) & !(C & A)", "true & (false | A)", "a_1 | B2 & !(C)"]
    index = {"A": 0, "B": 1, "C": 2, "a_1": 3, "B2": 4}
    compiled = {}
    for k, text in enumerate(exprs):
        o, a = ex.compile_postfix(ex.parse(text), index)
        compiled[f"e{k}_ops"] = np.array(o, dtype=np.int32)
        compiled[f"e{k}_args"] = np.array(a, dtype=np.int32)
        compiled[f"e{k}_depth"] = np.array(ex.depth(ex.parse(text)))
    np.savez_compressed(HERE / "network_readers.npz", bnd_text=np.array(bnd_text), names=np.array(toy.names),
                        p_on=np.array([n.p_on for n in toy.nodes]), inputs=np.array(toy.input_names),
                        exprs=np.array(exprs), **{f"prog_{k}": v for k, v in tp.items()}, **compiled)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
