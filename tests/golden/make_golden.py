"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources are present (they are built into
oracle/_ref/libgtref.so by oracle/Makefile.ref):

    make -f oracle/Makefile.ref REF=<the reference tree>
    python tests/golden/make_golden.py

Each fixture holds seeded inputs and the reference's outputs for them:
tree (serial layout) and tree order, grouped lists for several group sizes
and packings, the CPU evaluation of those lists, the group solver's forces,
FP64 and FP32 direct sums, and a small benchmark galaxy. The CPU tests check
the oracle against these files bit for bit.
"""

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from native import NO_PARALLEL, Ref, coincident_system, lopsided_sphere  # noqa: E402

CASES = {
    "lopsided_3000": lambda: lopsided_sphere(3000, 11),
    "lopsided_613": lambda: lopsided_sphere(613, 3),
    "coincident_150": coincident_system,
}
LIST_VARIANTS = [(0.7, 7, False), (0.7, 32, False), (0.7, 32, True), (1.0, 32, True)]
EPS = 0.01


def main():
    ref = Ref()
    for name, make in CASES.items():
        pos, mass = make()
        out = {"pos": pos, "mass": mass}
        for leaf in (1, 8):
            nodes, order, depth = ref.tree(pos, mass, leaf, NO_PARALLEL)
            out[f"tree_leaf{leaf}_nodes"] = nodes
            out[f"tree_leaf{leaf}_order"] = order
            out[f"tree_leaf{leaf}_depth"] = np.int64(depth)
        for theta, gs, pack in LIST_VARIANTS:
            key = f"lists_t{theta}_gs{gs}_p{int(pack)}"
            _, _, L, ev = ref.lists(pos, mass, theta=theta, group_size=gs, leaf_size=8, pack=pack,
                                    eps=EPS, evaluate=True)
            out[key + "_groups"] = L.groups
            out[key + "_cell_list"] = L.cell_list
            out[key + "_body_list"] = L.body_list
            out[key + "_cells"] = L.cells
            out[key + "_bodies"] = L.bodies
            out[key + "_eval"] = ev
            out[key + "_stats"] = np.array([L.stats.cell_interactions, L.stats.body_interactions,
                                            L.stats.max_list, L.stats.max_group], np.uint64)
        acc, pot, _ = ref.group_force(pos, mass, theta=0.6, eps=EPS, pack=False)
        out["group_acc"], out["group_pot"] = acc, pot
        acc, pot, st = ref.tree_force(pos, mass, theta=0.6, eps=EPS)
        out["tree_acc"], out["tree_pot"] = acc, pot
        out["tree_stats"] = np.array(st, np.uint64)
        acc, pot = ref.direct_fp64(pos, mass, eps=EPS)
        out["direct64_acc"], out["direct64_pot"] = acc, pot
        bodies, d32 = ref.direct_fp32(pos, mass, [1.0, 1.0, 1.0], eps=EPS)
        out["direct32_bodies"], out["direct32_out"] = bodies, d32
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, {k: getattr(v, "shape", ()) for k, v in out.items() if k.endswith("nodes")})
    # the benchmark galaxy model at small n: positions, masses, types
    gp, gv, gm, gt = ref.galaxy(n=6000, seed=1)
    np.savez_compressed(HERE / "galaxy_6000.npz", pos=gp, vel=gv, mass=gm, type=gt)
    print("galaxy_6000", gp.shape)


if __name__ == "__main__":
    main()
