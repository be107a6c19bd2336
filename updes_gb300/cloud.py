"""Point clouds with the reference's node ordering (host side, NumPy).

``SquareCloud`` reproduces updes/cloud.py:382-510 (global ids, facet typing,
normals) and the renumbering of updes/cloud.py:115-172 (internal, Dirichlet,
Neumann, Robin, periodic), vectorised.  With support_size="max" every node's
support is "all other nodes" (updes/cloud.py:97-112), so the N x (N-1)
support table is never materialised.  With an integer support_size every
node's support is its support_size - 1 nearest other nodes
(``sorted_local_supports``, updes/cloud.py:83-112), found with SciPy's
KD-tree instead of the reference's BallTree: the same sets wherever no two
candidates are equally far at the edge of a support (the order inside a
support does not matter to any matrix built from it).
"""
from __future__ import annotations

import numpy as np


class Cloud:
    """Common attributes of a meshfree cloud (updes/cloud.py:10-49)."""

    def __init__(self, facet_types, support_size="max"):
        if support_size is None:
            support_size = "max"
        if support_size != "max" and (isinstance(support_size, bool) or not isinstance(support_size, (int, np.integer))):
            raise ValueError(f"support_size must be 'max' or an int, not {support_size!r}")
        self.support_size = support_size if support_size == "max" else int(support_size)
        self.sorted_local_supports = None
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
        self.sorted_local_supports = _define_local_supports(self)

    @property
    def nodes(self):
        return {i: self.sorted_nodes[i] for i in range(self.N)}


def _define_local_supports(cloud):
    """(N, support_size - 1) int32 supports in sorted node order, or None for "max" (updes/cloud.py:83-112:
    the support_size nearest nodes of each node, the first of them, the node itself, dropped)."""
    k = cloud.support_size
    if k == "max" or k == cloud.N:  # every other node (support_size = N is the same as "max")
        return None
    if not 0 < k <= cloud.N:
        raise AssertionError("Support size must be strictly greater than 0 and at most the number of nodes")
    if k == 1:
        raise ValueError("support_size 1 leaves every support empty: the collocation matrix would be singular")
    from scipy.spatial import cKDTree
    _, nb = cKDTree(cloud.sorted_nodes).query(cloud.sorted_nodes, k=k)
    nb = np.asarray(nb, dtype=np.int64).reshape(cloud.N, k)
    return np.ascontiguousarray(nb[:, 1:], dtype=np.int32)


class GmshCloud(Cloud):
    """Cloud read from a Gmsh mesh file, format 4.0.8 (updes/cloud.py:520-734).

    ``filename``: a ``.msh`` file, or a ``.py`` script that writes ``mesh.msh`` with the gmsh Python
    package (run as the reference does, ``python <script> <mesh_save_location> --nopopup``).
    The reading follows the reference line by line in what it takes from the file:
      - facet names: the first ``count - 1`` entries of ``$PhysicalNames`` (the last one names the
        surface), and each curve entity's physical tag, the 4th token from the end of its
        ``$Entities`` line;
      - nodes from ``$Nodes`` blocks: dimension 0 are corners, 1 take their curve's facet type, 2 are
        interior; node ids are the file's tags minus one;
      - a corner belongs to the facet of lowest precedence (order in ``facet_types``) among the curves
        whose 2-node elements in ``$Elements`` contain it, and is appended to that facet's node list.
    Outward normals of Neumann, Robin and periodic nodes (updes/cloud.py:698-734): the tangent runs to
    the nearest other node of the same curve, the inward vector to the second-nearest interior node,
    and the normal (-t_y, t_x) is flipped to point away from the interior.  Nodes are renumbered
    interior, Dirichlet, Neumann, Robin, periodic, each in file order (updes/cloud.py:124-172).
    Periodic facets are not counted into ``Np`` by the reference's reader and are rejected here.
    """

    def __init__(self, filename, mesh_save_location=None, facet_types=None, support_size="max"):
        if facet_types is None:
            raise ValueError("facet_types is required")
        super().__init__(facet_types=facet_types, support_size=support_size)
        if any(v[0] == "p" for v in facet_types.values()):
            raise NotImplementedError("periodic facets on a Gmsh cloud are not counted by the reference reader")
        self.facet_precedence = {k: i for i, k in enumerate(facet_types)}
        self.filename = self._meshfile(filename, mesh_save_location)
        self._read()
        self._normals()
        self._renumber()
        self.sorted_local_supports = _define_local_supports(self)

    @staticmethod
    def _meshfile(filename, mesh_save_location):
        import os
        import subprocess
        import sys
        if mesh_save_location is None:
            mesh_save_location = os.path.dirname(filename) + "/"
        ext = filename.rsplit(".", maxsplit=1)[-1]
        if ext == "msh":
            return filename
        if ext == "py":
            subprocess.run([sys.executable, filename, mesh_save_location, "--nopopup"], check=True)
            return mesh_save_location + "mesh.msh"
        raise ValueError(f"unsupported mesh file {filename!r} (.msh or .py)")

    def _read(self):
        with open(self.filename) as fh:
            lines = fh.read().splitlines()
        pos = 0

        def seek(tag):
            nonlocal pos
            while tag not in lines[pos]:
                pos += 1
            pos += 1

        seek("$PhysicalNames")
        count = int(lines[pos].split()[0])
        pos += 1
        phys = {}
        for _ in range(count - 1):
            t = lines[pos].split()
            phys[int(t[1])] = t[2][1:-1]
            pos += 1
        seek("$Entities")
        t = lines[pos].split()
        n_vertices, n_curves = int(t[0]), int(t[1])
        pos += 1 + n_vertices
        self.facet_names = {}
        for _ in range(n_curves):
            t = lines[pos].split()
            self.facet_names[int(t[0])] = phys[int(t[-4])]
            pos += 1
        seek("$Nodes")
        self.N = int(lines[pos].split()[1])
        pos += 1
        coords = np.zeros((self.N, 2))
        ntype = np.empty(self.N, dtype=object)
        self.facet_nodes = {v: [] for v in self.facet_names.values()}
        self.facet_tag_nodes = {k: [] for k in self.facet_names}
        corners = []  # in file order
        while "$EndNodes" not in lines[pos]:
            t = lines[pos].split()
            entity, dim, nb = int(t[0]), int(t[1]), int(t[-1])
            pos += 1
            block = np.array([lines[pos + i].split()[:3] for i in range(nb)], dtype=np.float64).reshape(nb, 3)
            pos += nb
            ids = block[:, 0].astype(np.int64) - 1
            coords[ids] = block[:, 1:3]
            if dim == 0:
                corners.extend(ids.tolist())
            elif dim == 1:
                ntype[ids] = self.facet_types[self.facet_names[entity]]
                self.facet_nodes[self.facet_names[entity]] += ids.tolist()
                self.facet_tag_nodes[entity] += ids.tolist()
            elif dim == 2:
                ntype[ids] = "i"
        membership = {c: [] for c in corners}
        seek("$Elements")
        pos += 1  # the block and element counts
        corner_set = set(corners)
        while "$EndElements" not in lines[pos]:
            t = lines[pos].split()
            entity, dim, nb = int(t[0]), int(t[1]), int(t[-1])
            pos += 1
            if dim == 1:
                for i in range(nb):
                    nodes = [int(v) - 1 for v in lines[pos + i].split()[1:]]
                    for c in corner_set.intersection(nodes):
                        if any(v != c for v in nodes):
                            membership[c].append(entity)
            pos += nb
        for c in corners:  # file order, as the reference's dict
            tags = sorted(membership[c], key=lambda tag: self.facet_precedence[self.facet_names[tag]])
            if not tags:
                raise ValueError(f"corner node {c + 1} lies on no boundary element")
            name = self.facet_names[tags[0]]
            ntype[c] = self.facet_types[name]
            self.facet_nodes[name].append(c)
            self.facet_tag_nodes[tags[0]].append(c)
        if any(v is None for v in ntype):
            raise ValueError("every node must belong to a point, curve or surface entity")
        self._coords, self._ntype = coords, ntype

    def _normals(self):
        from scipy.spatial import cKDTree
        coords, ntype = self._coords, self._ntype
        interior = np.flatnonzero(np.array([t == "i" for t in ntype]))
        in_tree = cKDTree(coords[interior])
        self._normal = {}
        for tag, fnodes in self.facet_tag_nodes.items():
            if self.facet_types[self.facet_names[tag]][0] not in ("n", "r", "p"):
                continue
            if len(fnodes) < 2:
                raise AssertionError("Mesh not fine enough for normal computation")
            fc = coords[fnodes]
            _, nb_f = cKDTree(fc).query(fc, k=2)
            _, nb_i = in_tree.query(fc, k=2)
            tangent = fc[nb_f[:, 1]] - fc
            inward = coords[interior[nb_i[:, 1]]] - fc
            normal = np.stack([-tangent[:, 1], tangent[:, 0]], axis=-1)
            normal /= np.linalg.norm(normal, axis=1, keepdims=True)
            flip = np.einsum("ij,ij->i", normal, inward) > 0
            normal[flip] = -normal[flip]
            for k, node in enumerate(fnodes):
                self._normal[node] = normal[k]

    def _renumber(self):
        coords, ntype, N = self._coords, self._ntype, self.N
        first = np.array([t[0] for t in ntype])
        gid = np.arange(N)
        order = np.concatenate([gid[first == c] for c in ("i", "d", "n", "r")])
        new = np.empty(N, dtype=np.int64)
        new[order] = np.arange(N)
        self.renumbering_map = {int(g): int(new[g]) for g in range(N)}
        self.sorted_nodes = np.ascontiguousarray(coords[order])
        self.node_types = {int(new[g]): ntype[g] for g in range(N)}
        self.facet_nodes = {f: [int(new[i]) for i in v] for f, v in self.facet_nodes.items()}
        self.facet_tag_nodes = {k: [int(new[i]) for i in v] for k, v in self.facet_tag_nodes.items()}
        self.Ni, self.Nd, self.Nn, self.Nr = (int(np.sum(first == c)) for c in ("i", "d", "n", "r"))
        self.Np = []
        self.normals_by_node = np.zeros((N, 2))
        self.has_normal = np.zeros(N, dtype=bool)
        for g, v in self._normal.items():
            self.normals_by_node[new[g]] = v
            self.has_normal[new[g]] = True
        self.outward_normals = {int(i): self.normals_by_node[i] for i in np.flatnonzero(self.has_normal)}
        self.sorted_outward_normals = self.normals_by_node[self.has_normal]

    @property
    def nodes(self):
        return {i: self.sorted_nodes[i] for i in range(self.N)}
