"""Turn a golden case description into oracle inputs (test helper)."""
from __future__ import annotations

import json
import os

import numpy as np

import cases as C
from oracle import updes_np as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False))


def oracle_problem(case, compat=True):
    """Cloud, rows, operator weights, q for a case, computed by the oracle alone."""
    cloud = O.square_cloud(case["Nx"], case["Ny"], case["facets"], coords=C.grid_coords(case))
    X = cloud.sorted_nodes
    kind, param = case["rbf"]
    fields = C.make_fields(case, X)
    Ni = cloud.Ni
    W = C.op_weights(case["op"], X[:Ni, 0], X[:Ni, 1], None if fields is None else fields[:, :Ni])
    betas = {}
    bcv = {}
    for f, spec in case["bc"].items():
        ids = np.array(cloud.facet_nodes[f], dtype=np.int64)
        if isinstance(spec, tuple):
            bcv[f] = C.FUNCS[spec[0]](np, X[ids, 0], X[ids, 1])
            betas[f] = C.FUNCS[spec[1]](np, X[ids, 0], X[ids, 1])
        else:
            bcv[f] = C.FUNCS[spec](np, X[ids, 0], X[ids, 1])
    robin = O.robin_betas(cloud, betas, compat=compat)
    rows = O.boundary_rows(cloud, robin, compat=compat)
    if case["rhs"] == "value_over_dt":
        u0 = C.make_rhs_field(case, X)
        cu = O.field_coefficients(cloud, kind, param, case["max_degree"], u0)
        f_int = O.value(X[:Ni], cu, X, kind, param) / C.ADV_DT
    else:
        f_int = C.FUNCS[case["rhs"]](np, X[:Ni, 0], X[:Ni, 1])
    q = O.assemble_q(cloud, f_int, bcv)
    supports = O.local_supports(X, case["support"]) if case.get("support") is not None else None
    return dict(cloud=cloud, rows=rows, W=W, q=q, kind=kind, param=param, deg=case["max_degree"],
                fields=fields, robin=robin, bcv=bcv, supports=supports)


def case_of(g):
    c = json.loads(str(g["case"]))
    c["facets"] = dict(c["facets"])
    c["bc"] = {k: tuple(v) if isinstance(v, list) else v for k, v in c["bc"].items()}
    if c.get("jitter") is not None:
        c["jitter"] = tuple(c["jitter"])
    return c
