"""Comparisons between the device build and the oracle / reference.

Node numbering differs by design (the device numbers nodes in walk order,
the reference appends children blocks as it splits, and its parallel build
depends on the thread count), so nodes are compared by identity: a node is
fixed by its first body and its depth, since a node and its only child share
a range but not a depth.
"""

import numpy as np


def ref_depths(nodes):
    """Depth of every node of a reference-layout tree (children after parents)."""
    depth = np.zeros(len(nodes), np.int64)
    fc = nodes["first_child"].astype(np.int64)
    nc = nodes["n_children"].astype(np.int64)
    for i in range(len(nodes)):
        if nc[i] > 0:
            depth[fc[i]:fc[i] + nc[i]] = depth[i] + 1
    return depth


def node_keys(begin, depth):
    return (np.asarray(begin, np.int64) << 7) | np.asarray(depth, np.int64)


def compare_trees(dev_nodes, ref_nodes):
    """Returns a list of mismatch descriptions (empty when identical)."""
    bad = []
    if len(dev_nodes) != len(ref_nodes):
        return [f"node count {len(dev_nodes)} != {len(ref_nodes)}"]
    rd = ref_depths(ref_nodes)
    dk = node_keys(dev_nodes["begin"], dev_nodes["depth"])
    rk = node_keys(ref_nodes["begin"], rd)
    di, ri = np.argsort(dk), np.argsort(rk)
    if not np.array_equal(dk[di], rk[ri]):
        return ["node sets differ"]
    d, r = dev_nodes[di], ref_nodes[ri]
    for f in ("end", "half", "center", "com", "mass", "quad", "delta"):
        if not np.array_equal(d[f], r[f]):
            k = np.nonzero(np.any((d[f] != r[f]).reshape(len(d), -1), axis=1))[0]
            bad.append(f"{f}: {len(k)} nodes differ, first at begin={d['begin'][k[0]]}")
    leaf_d = d["n_children"] == 0
    leaf_r = r["n_children"] == 0
    if not np.array_equal(leaf_d, leaf_r) or not np.array_equal(d["n_children"], r["n_children"]):
        bad.append("children counts differ")
    return bad


def sorted_per_group(values, starts, ends):
    """Each group's entries sorted, groups in turn (a group's multiset)."""
    counts = (np.asarray(ends, np.int64) - np.asarray(starts, np.int64))
    gid = np.repeat(np.arange(len(counts)), counts)
    v = np.asarray(values)[np.concatenate([np.arange(s, e) for s, e in zip(starts, ends)])
                           if len(counts) else np.zeros(0, np.int64)]
    return v[np.lexsort((v, gid))]


def compare_lists(dev, dev_nodes, ref_lists, ref_nodes, body_order=False):
    """Groups, every group's cell list in order, and every group's bodies:
    as a multiset, or in order with body_order. The device's walk by warps
    writes a group's bodies in the order its steps reach them (its exports
    give them sorted); the reference's order -- siblings last octant first,
    the bodies of a node in tree order -- is pinned through the walk by
    threads (option walk_warps 0), which keeps it."""
    bad = []
    g_d, g_r = dev["groups"], ref_lists.groups
    if g_d.shape != g_r.shape:
        return [f"group count {len(g_d)} != {len(g_r)}"]
    if not np.array_equal(g_d[:, :6], g_r[:, :6]):
        k = np.nonzero(np.any(g_d[:, :6] != g_r[:, :6], axis=1))[0]
        bad.append(f"{len(k)} group records differ, first {k[0]}: {g_d[k[0]]} vs {g_r[k[0]]}")
        return bad
    if body_order:
        same = np.array_equal(dev["body_list"], ref_lists.body_list)
    else:
        same = np.array_equal(sorted_per_group(dev["body_list"], g_d[:, 4], g_d[:, 5]),
                              sorted_per_group(ref_lists.body_list, g_r[:, 4], g_r[:, 5]))
    if not same:
        bad.append("body lists differ")
    dkey = node_keys(dev_nodes["begin"], dev_nodes["depth"])
    rkey = node_keys(ref_nodes["begin"], ref_depths(ref_nodes))
    if len(dev["cell_list"]) != len(ref_lists.cell_list) or not np.array_equal(
            dkey[dev["cell_list"]], rkey[ref_lists.cell_list]):
        bad.append("cell lists differ")
    return bad


def rel_errors(acc, ref):
    return np.linalg.norm(acc - ref, axis=1) / np.linalg.norm(ref, axis=1)


def scatter(tree_order_vals, order):
    out = np.zeros_like(tree_order_vals)
    out[np.asarray(order, np.int64)] = tree_order_vals
    return out


# ---- the reference's list invariants (tests/test_gpu_kernels.cpp:109-168) ----

def check_lists(node_begin, node_end, groups, cell_list, body_list, n, group_size):
    """Groups tile [0, n) in order and have 1..group_size targets; every body is
    covered exactly once by each group's list (a cell covers all its bodies);
    no accepted cell contains one of the group's targets. Returns the number
    of violations."""
    bad = 0
    nxt = 0
    for g in groups:
        if g[0] != nxt or g[1] <= g[0] or g[1] - g[0] > group_size:
            bad += 1
        nxt = g[1]
    bad += int(nxt != n)
    nb = np.asarray(node_begin, np.int64)
    ne = np.asarray(node_end, np.int64)
    for g in groups:
        cov = np.zeros(n + 1, np.int64)
        cells = np.asarray(cell_list[g[2]:g[3]], np.int64)
        b, e = nb[cells], ne[cells]
        bad += int(np.count_nonzero((b < g[1]) & (g[0] < e)))
        np.add.at(cov, b, 1)
        np.add.at(cov, e, -1)
        cov = np.cumsum(cov)[:n]
        np.add.at(cov, np.asarray(body_list[g[4]:g[5]], np.int64), 1)
        bad += int(np.count_nonzero(cov != 1))
    return bad


def check_packing(node_begin, node_end, children, groups):
    """Packing only merges siblings: every group is a whole node, a chunk of a
    leaf, or a run of consecutive children of the deepest node containing it.
    `children(p)` lists p's children. Returns the number of violations."""
    bad = 0
    for g in groups:
        p = 0
        while True:
            for c in children(p):
                if node_begin[c] <= g[0] and g[1] <= node_end[c]:
                    p = c
                    break
            else:
                break
        if node_begin[p] == g[0] and node_end[p] == g[1]:
            continue
        ch = children(p)
        if not ch:
            continue
        starts = any(node_begin[c] == g[0] for c in ch)
        ends = any(node_end[c] == g[1] for c in ch)
        bad += int(not (starts and ends))
    return bad


def ref_children(nodes):
    fc, nc = nodes["first_child"], nodes["n_children"]
    return lambda p: list(range(int(fc[p]), int(fc[p]) + int(nc[p]))) if nc[p] > 0 else []


def dev_children(nodes):
    skip = nodes["skip"]
    nch = nodes["n_children"]

    def children(p):
        if nch[p] == 0:
            return []
        out, c = [], p + 1
        while c < skip[p]:
            out.append(c)
            c = int(skip[c])
        return out[::-1]
    return children
