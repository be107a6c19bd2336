"""Point clouds with the reference's node ordering (host side, NumPy).

``SquareCloud`` reproduces updes/cloud.py:382-510 (global ids, facet typing,
normals) and the renumbering of updes/cloud.py:115-172 (internal, Dirichlet,
Neumann, Robin, periodic), vectorised.  With support_size="max" every node's
support is "all other nodes" (updes/cloud.py:97-112), so the N x (N-1)
support table is never materialised.
"""
from __future__ import annotations

import numpy as np


class Cloud:
    """Common attributes of a meshfree cloud (updes/cloud.py:10-49)."""

    def __init__(self, facet_types, support_size="max"):
        if support_size not in ("max", None):
            raise NotImplementedError("only support_size='max' (global collocation) is implemented")
        self.support_size = "max"
        self.dim = 2
        self.N = self.Ni = self.Nd = self.Nn = self.Nr = 0
        self.Np = []
        # periodic facet types get their position appended (updes/cloud.py:42-49)
        self.facet_types = {k: (v + str(i) if v[0] == "p" else v) for i, (k, v) in enumerate(facet_types.items())}


class SquareCloud(Cloud):
    """Unit-square cloud of Nx x Ny nodes (updes/cloud.py:378-510).

    ``coords``: optional (Nx*Ny, 2) coordinates by ORIGINAL id (id = i*Ny + j).
    ``jitter``: optional ``(frac, seed)``: nodes of type other than d/n/r move by
    U(-frac*h, frac*h) per coordinate (h = smaller spacing), drawn as one
    (N, 2) block from ``numpy.random.default_rng(seed)``.  The reference's
    ``noise_key`` uses jax.random, which is not reproduced here.
    """

    def __init__(self, Nx=7, Ny=5, noise_key=None, coords=None, jitter=None, **kwargs):
        super().__init__(**kwargs)
        if noise_key is not None:
            raise NotImplementedError("jax noise keys are not reproduced: pass coords= or jitter=(frac, seed)")
        self.Nx, self.Ny = int(Nx), int(Ny)
        self.N = self.Nx * self.Ny
        Nx, Ny, N = self.Nx, self.Ny, self.N
        gid = np.arange(N)
        ii, jj = gid // Ny, gid % Ny                         # id = i*Ny + j (cloud.py:418-422)
        self.global_indices = gid.reshape(Nx, Ny).copy()
        ft = self.facet_types
        for f in ("North", "South", "East", "West"):
            if f not in ft:
                raise ValueError(f"facet_types must define {f}")
        # corner precedence North > South > East > West (cloud.py:457-470)
        facet = np.where(jj == Ny - 1, "North", np.where(jj == 0, "South", np.where(
            ii == Nx - 1, "East", np.where(ii == 0, "West", ""))))
        ntype = np.array([ft[f] if f else "i" for f in facet], dtype=object)
        xs, ys = np.linspace(0.0, 1.0, Nx), np.linspace(0.0, 1.0, Ny)
        if coords is None:
            coords = np.stack([xs[ii], ys[jj]], axis=-1)
            if jitter is not None:
                frac, seed = jitter
                h = min(xs[1] - xs[0], ys[1] - ys[0])
                noise = np.random.default_rng(seed).uniform(-frac * h, frac * h, size=(N, 2))
                move = np.array([t not in ("d", "n", "r") for t in ntype])
                coords[move] += noise[move]
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        if coords.shape != (N, 2):
            raise ValueError(f"coords must be ({N}, 2)")
        # renumbering: i, d, n, r, then periodic groups by sorted type key (cloud.py:124-150)
        first = np.array([t[0] for t in ntype])
        order = [gid[first == c] for c in ("i", "d", "n", "r")]
        for key in sorted({t for t in ntype if t[0] == "p"}):
            order.append(gid[ntype == key])
        order = np.concatenate(order)
        new = np.empty(N, dtype=np.int64)
        new[order] = np.arange(N)
        self.renumbering_map = {int(g): int(new[g]) for g in range(N)}
        self.sorted_nodes = coords[order]
        self.node_types = {int(new[g]): ntype[g] for g in range(N)}
        self.facet_nodes = {f: new[facet == f].tolist() for f in ft}
        self.Nd = int(sum(len(self.facet_nodes[f]) for f, t in ft.items() if t == "d"))
        self.Nn = int(sum(len(self.facet_nodes[f]) for f, t in ft.items() if t == "n"))
        self.Nr = int(sum(len(self.facet_nodes[f]) for f, t in ft.items() if t == "r"))
        npd = {}
        for f, t in ft.items():
            if t[0] == "p":
                npd[t[:-1]] = npd.get(t[:-1], 0) + len(self.facet_nodes[f])
        self.Np = [npd[k] for k in sorted(npd)]
        self.Ni = N - self.Nd - self.Nn - self.Nr - sum(self.Np)
        # outward normals of n, r, p nodes (cloud.py:493-510), by renumbered id
        nvec = {"North": (0.0, 1.0), "South": (0.0, -1.0), "East": (1.0, 0.0), "West": (-1.0, 0.0)}
        has = np.isin(first, ["n", "r", "p"])
        normals = np.zeros((N, 2))
        for f, v in nvec.items():
            normals[facet == f] = v
        self.normals_by_node = np.zeros((N, 2))
        self.normals_by_node[new[has]] = normals[has]
        self.has_normal = np.zeros(N, dtype=bool)
        self.has_normal[new[has]] = True
        self.outward_normals = {int(i): self.normals_by_node[i] for i in np.flatnonzero(self.has_normal)}
        self.sorted_outward_normals = self.normals_by_node[self.has_normal]

    @property
    def nodes(self):
        return {i: self.sorted_nodes[i] for i in range(self.N)}
