"""Write the synthetic Gmsh meshes (format 4.0.8) used by the GmshCloud tests.

    python tests/golden/make_msh.py

``dshape.msh``: the unit square whose top side is the arc y = 1 + 0.25 sin(pi x); four curves
Bottom, Right, Top, Left (physical tags 1-4) and the surface (tag 5); boundary nodes at uneven
spacings and jittered interior nodes (seeded), so that no nearest-neighbour query has a tie.
Only what a 4.0.8 reader takes from the file is written: physical names, point and curve entities,
node blocks by entity, and 2-node line elements along every curve.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def top(x):
    return 1.0 + 0.25 * np.sin(np.pi * x)


def dshape(nb=9, ni=12, seed=3):
    rng = np.random.default_rng(seed)
    corners = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])

    def params(k):  # k interior points of a side, uneven
        t = (np.arange(1, k + 1) + rng.uniform(-0.3, 0.3, k)) / (k + 1)
        return np.sort(t)
    tb, tr, tt, tl = params(nb), params(nb - 2), params(nb + 2), params(nb - 1)
    curves = {
        1: ("Bottom", np.stack([tb, 0 * tb], 1), (1, 2)),
        2: ("Right", np.stack([0 * tr + 1.0, tr], 1), (2, 3)),
        3: ("Top", np.stack([1.0 - tt, top(1.0 - tt)], 1), (3, 4)),
        4: ("Left", np.stack([0 * tl, 1.0 - tl], 1), (4, 1)),
    }
    gx, gy = np.meshgrid((np.arange(1, ni) + 0.0) / ni, (np.arange(1, ni) + 0.0) / ni, indexing="ij")
    x = gx.ravel() + rng.uniform(-0.25, 0.25, gx.size) / ni
    y = gy.ravel() * top(gx.ravel()) + rng.uniform(-0.25, 0.25, gx.size) / ni
    inside = (x > 0.02) & (x < 0.98) & (y > 0.02) & (y < top(x) - 0.02)
    interior = np.stack([x[inside], y[inside]], 1)
    return corners, curves, interior


def write(path, corners, curves, interior):
    out = ["$MeshFormat", "4 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(curves) + 1)]
    for tag, (name, _, _) in curves.items():
        out.append(f'1 {tag} "{name}"')
    out.append(f'2 {len(curves) + 1} "Domain"')
    out += ["$EndPhysicalNames", "$Entities", f"{len(corners)} {len(curves)} 1 0"]
    for i, (cx, cy) in enumerate(corners):
        out.append(f"{i + 1} {cx} {cy} 0 {cx} {cy} 0 0")
    for tag, (name, pts, (a, b)) in curves.items():
        lo, hi = np.minimum(corners[a - 1], corners[b - 1]), np.maximum(corners[a - 1], corners[b - 1])
        out.append(f"{tag} {lo[0]} {lo[1]} 0 {hi[0]} {hi[1]} 0 1 {tag} 2 {a} {-b}")
    out.append(f"1 0 0 0 1 1.25 0 1 {len(curves) + 1} {len(curves)} " + " ".join(str(t) for t in curves))
    out.append("$EndEntities")
    n_nodes = len(corners) + sum(len(c[1]) for c in curves.values()) + len(interior)
    out += ["$Nodes", f"{len(corners) + len(curves) + 1} {n_nodes}"]
    tag = 1
    corner_tag = {}
    for i, (cx, cy) in enumerate(corners):
        out += [f"{i + 1} 0 0 1", f"{tag} {float(cx)!r} {float(cy)!r} 0"]
        corner_tag[i + 1] = tag
        tag += 1
    curve_tags = {}
    for ctag, (name, pts, _) in curves.items():
        out.append(f"{ctag} 1 0 {len(pts)}")
        curve_tags[ctag] = []
        for px, py in pts:
            out.append(f"{tag} {float(px)!r} {float(py)!r} 0")
            curve_tags[ctag].append(tag)
            tag += 1
    out.append(f"1 2 0 {len(interior)}")
    for px, py in interior:
        out.append(f"{tag} {float(px)!r} {float(py)!r} 0")
        tag += 1
    out.append("$EndNodes")
    n_el = sum(len(v) + 1 for v in curve_tags.values())
    out += ["$Elements", f"{len(curves)} {n_el}"]
    el = 1
    for ctag, (_, _, (a, b)) in curves.items():
        chain = [corner_tag[a]] + curve_tags[ctag] + [corner_tag[b]]
        out.append(f"{ctag} 1 1 {len(chain) - 1}")
        for u, v in zip(chain[:-1], chain[1:]):
            out.append(f"{el} {u} {v}")
            el += 1
    out.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


if __name__ == "__main__":
    write(os.path.join(HERE, "dshape.msh"), *dshape())
    print("wrote", os.path.join(HERE, "dshape.msh"))
