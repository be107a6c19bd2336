"""Radial basis functions with the reference's names and signatures.

``polyharmonic(x, center, a=1)`` etc. mirror updes/utils.py:30-69 and can be
called directly (NumPy, one pair of points).  The solver does not call them:
it identifies the kernel and its parameter (``rbf_spec``) and evaluates the
kernel and its closed-form derivatives inside the CUDA assembly kernel.
"""
from __future__ import annotations

import functools
import math

import numpy as np

from . import _lib


def distance(node1, node2):
    """Euclidean distance (updes/utils.py:19-22)."""
    d = np.asarray(node1, dtype=np.float64) - np.asarray(node2, dtype=np.float64)
    return np.sqrt(d @ d)


def multiquadric(x, center, eps=1.0):
    """Hardy's multiquadric sqrt(1 + (eps r)^2) (updes/utils.py:30-35)."""
    return np.sqrt(1.0 + (eps * distance(x, center)) ** 2)


def inverse_multiquadric(x, center, eps=1.0):
    """1 / sqrt(1 + (eps r)^2) (updes/utils.py:37-42)."""
    return 1.0 / np.sqrt(1.0 + (eps * distance(x, center)) ** 2)


def gaussian(x, center, eps=1.0):
    """exp(-(eps r)^2) (updes/utils.py:44-48)."""
    return np.exp(-(eps * distance(x, center)) ** 2)


def polyharmonic(x, center, a=1):
    """Polyharmonic spline r^(2a+1) (updes/utils.py:50-55)."""
    return distance(x, center) ** (2 * a + 1)


def thin_plate(x, center, a=1):
    """Thin plate spline log(r) r^(2a), 0 at r = 0 (updes/utils.py:63-69)."""
    r = distance(x, center)
    return 0.0 if r == 0.0 else math.log(r) * r ** (2 * a)


_KINDS = {
    "polyharmonic": (_lib.RBF_POLYHARMONIC, "a", 1),
    "gaussian": (_lib.RBF_GAUSSIAN, "eps", 1.0),
    "multiquadric": (_lib.RBF_MULTIQUADRIC, "eps", 1.0),
    "inverse_multiquadric": (_lib.RBF_INVERSE_MULTIQUADRIC, "eps", 1.0),
    "thin_plate": (_lib.RBF_THIN_PLATE, "a", 1),
}
KIND_NAMES = {v[0]: k for k, v in _KINDS.items()}


def rbf_spec(rbf) -> tuple[int, float]:
    """(kernel id, parameter) of an RBF callable.

    Accepts this module's functions, the reference's functions of the same
    names (``updes.polyharmonic`` ...), and ``functools.partial`` /
    ``jax.tree_util.Partial`` wrappers that set ``a`` or ``eps`` — the forms the
    reference's demos pass (e.g. ``partial(polyharmonic, a=2)``).
    Any other callable is rejected: the GPU assembly needs closed forms.
    """
    if rbf is None:
        rbf = polyharmonic  # updes/utils.py:85-86 default
    kw = {}
    f = rbf
    while isinstance(f, functools.partial) or (hasattr(f, "func") and hasattr(f, "keywords")):
        if getattr(f, "args", ()):
            raise ValueError("RBF partials must set parameters by keyword (a=..., eps=...)")
        kw = {**(f.keywords or {}), **kw}
        f = f.func
    name = getattr(f, "__name__", None)
    if name not in _KINDS:
        raise ValueError(f"unsupported RBF {rbf!r}: use polyharmonic, gaussian, multiquadric, "
                         "inverse_multiquadric or thin_plate (optionally through functools.partial)")
    kid, pname, default = _KINDS[name]
    extra = set(kw) - {pname}
    if extra:
        raise ValueError(f"unexpected RBF parameters {sorted(extra)} for {name}")
    param = float(kw.get(pname, default))
    if pname == "a" and (param != int(param) or param < 1 or param > 8):
        raise ValueError(f"{name}: a must be an integer in [1, 8], got {param}")
    return kid, param
