"""The reference's assembly functions by name (updes/assembly.py:10-485), as host calls that return NumPy
arrays: every matrix is assembled on the GPU by ``updes_assemble`` (the same kernel the solve uses) and the
requested block is read back.  Plus the reference's scalar kernel forms of r (updes/utils.py:30-88).

The solve itself never forms these blocks (it factors the Kansa matrix K once); they are for code that
calls the reference's assembly directly.  M (``nb_monomials``) is 1, 3, 6, 10 or 15 (degree 0 to 4).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .operators import (DEFAULT_OPTIONS, DeviceProblem, _interp_problem, _torch, boundary_rows, capture_operator,
                        materialize_B, nodal_value, prepare)
from .rbf import distance, polyharmonic

_DEGREE = {1: 0, 3: 1, 6: 2, 10: 3, 15: 4}


def _degree(nb_monomials):
    if nb_monomials not in _DEGREE:
        raise ValueError(f"nb_monomials must be one of {sorted(_DEGREE)} (degree 0 to 4), not {nb_monomials}")
    return _DEGREE[nb_monomials]


def _assemble(dp):
    """The full n x n matrix of a device problem, FP64, on the host."""
    torch = _torch()
    lib = _lib.load()
    n = dp.n
    ld = int(lib.updes_matrix_ld(n, 8))
    K = torch.zeros((n, ld), dtype=torch.float64, device=dp.device)
    _lib.check(lib.updes_assemble(ctypes.byref(dp.c), K.data_ptr(), ld, None, 0, dp.stream()), "updes_assemble")
    return K[:, :n].cpu().numpy()


def _kansa_problem(operator, cloud, rbf, nb_monomials, args=None, robin_coeffs=None):
    """The device problem of K with the captured operator on the interior rows and the cloud's boundary rows
    (Robin coefficients per node from ``robin_coeffs``)."""
    deg = _degree(nb_monomials)
    Ni = cloud.Ni
    fields = None
    if args:
        fields = np.stack([np.asarray(a, dtype=np.float64) for a in args])[:, :Ni]
    if operator is not None and Ni:
        W = capture_operator(operator, cloud.sorted_nodes[:Ni], rbf, fields)
    else:
        W = np.zeros((Ni, 5))
    kind, bnodes, geom = boundary_rows(cloud, dict(robin_coeffs or {}), DEFAULT_OPTIONS.compat_reference_quirks)
    return DeviceProblem(cloud, rbf, deg, W, kind, bnodes, geom, DEFAULT_OPTIONS.self_term), deg


def assemble_Phi(cloud, rbf):
    """Φ (N x N): the kernel between every node and every other, 0 on the diagonal as in the reference
    (updes/assembly.py:10-36)."""
    N = cloud.N
    return _assemble(_interp_problem(cloud, rbf, 0))[:N, :N]


def assemble_P(cloud, nb_monomials):
    """P (N x M): the monomials at the nodes (updes/assembly.py:39-59)."""
    N = cloud.N
    A = _assemble(_interp_problem(cloud, polyharmonic, _degree(nb_monomials)))
    return A[:N, N:]


def assemble_A(cloud, rbf, nb_monomials=2):
    """A = [[Φ, P], [Pᵀ, 0]] (updes/assembly.py:62-85)."""
    return _assemble(_interp_problem(cloud, rbf, _degree(nb_monomials)))


def assemble_invert_A(cloud, rbf, nb_monomials):
    """inv(A), by an FP64 LU of A on the GPU and solves with the identity (updes/assembly.py:87-90)."""
    torch = _torch()
    lib = _lib.load()
    dp = _interp_problem(cloud, rbf, _degree(nb_monomials))
    n = dp.n
    ld = int(lib.updes_matrix_ld(n, 8))
    A = torch.zeros((n, ld), dtype=torch.float64, device=dp.device)
    _lib.check(lib.updes_assemble(ctypes.byref(dp.c), A.data_ptr(), ld, None, 0, dp.stream()), "updes_assemble")
    piv = torch.empty(2 * n, dtype=torch.int32, device=dp.device)
    nbytes = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, _lib.PREC_FP64, ctypes.byref(nbytes)), "updes_lu_workspace")
    ws = torch.empty(nbytes.value + 8 * n + 512, dtype=torch.uint8, device=dp.device)
    info = ctypes.c_int32()
    _lib.check(lib.updes_lu_factor(n, A.data_ptr(), ld, _lib.PREC_FP64, None, 0, piv.data_ptr(), ws.data_ptr(),
                                   ws.numel(), ctypes.byref(info), dp.stream()), "updes_lu_factor")
    if info.value != 0:
        raise _lib.UpdesError(_lib.ERR_SINGULAR, f"assemble_invert_A (zero pivot at column {info.value})")
    Y = torch.eye(n, dtype=torch.float64, device=dp.device)
    _lib.check(lib.updes_lu_solve(n, A.data_ptr(), ld, _lib.PREC_FP64, piv.data_ptr(), Y.data_ptr(), n, n, 0,
                                  ws.data_ptr(), ws.numel(), dp.stream()), "updes_lu_solve")
    return Y.cpu().numpy()


def assemble_op_Phi_P(operator, cloud, rbf, nb_monomials, args):
    """(opΦ (Ni x N), opP (Ni x M)): the linear operator applied to the kernel and the monomials at the
    interior nodes, with per-node ``args`` fields (updes/assembly.py:93-137)."""
    dp, _ = _kansa_problem(operator, cloud, rbf, nb_monomials, args)
    K = _assemble(dp)
    N, Ni = cloud.N, cloud.Ni
    return K[:Ni, :N], K[:Ni, N:]


def assemble_bd_Phi_P(cloud, rbf, nb_monomials, robin_coeffs=None):
    """(bdΦ (Nb x N), bdP (Nb x M)): the boundary rows, Dirichlet, Neumann, Robin (β per node from
    ``robin_coeffs``) and periodic, in the reference's order and with its quirks (updes/assembly.py:141-362)."""
    dp, _ = _kansa_problem(None, cloud, rbf, nb_monomials, None, robin_coeffs)
    K = _assemble(dp)
    N, Ni = cloud.N, cloud.Ni
    return K[Ni:N, :N], K[Ni:N, N:]


def assemble_B(operator, cloud, rbf, nb_monomials, diff_args, robin_coeffs):
    """B = [opΦ opP; bdΦ bdP] · inv(A)[:, :N] (N x N) (updes/assembly.py:366-401), in FP64 on the GPU."""
    dp, deg = _kansa_problem(operator, cloud, rbf, nb_monomials, diff_args, robin_coeffs)
    return materialize_B(dp, cloud, rbf, deg)


def assemble_q(operator, boundary_conditions, cloud, rbf, nb_monomials, rhs_args):
    """q (N): the rhs operator at the interior nodes and the boundary values on the facets, periodic facets
    zeroed (updes/assembly.py:434-485)."""
    deg = _degree(nb_monomials)
    op = lambda x, center, rbf_, monomial, fields: nodal_value(x, center, rbf_, monomial)
    *_, q = prepare(op, operator, cloud, boundary_conditions, rbf, deg, None, rhs_args, DEFAULT_OPTIONS)
    return q


# The reference's kernels as functions of the distance r (updes/utils.py:30-71).
def polyharmonic_func(r, a):
    return np.asarray(r, dtype=np.float64) ** (2 * a + 1)


def gaussian_func(r, eps):
    return np.exp(-(eps * np.asarray(r, dtype=np.float64)) ** 2)


def multiquadric_func(r, eps):
    return np.sqrt(1 + (eps * np.asarray(r, dtype=np.float64)) ** 2)


def inv_multiquadric_func(r, eps):
    return 1.0 / np.sqrt(1 + (eps * np.asarray(r, dtype=np.float64)) ** 2)


def thin_plate_func(r, a):
    """log(r) r^(2a), 0 where that is not finite (r = 0), as the reference's nan_to_num."""
    r = np.asarray(r, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.log(r) * r ** (2 * a)
    return np.nan_to_num(v, nan=0.0, neginf=0.0, posinf=0.0)


def make_nodal_rbf(x, node, rbf):
    """``rbf`` (a function of the distance r; the polyharmonic spline when None) at |x - node|
    (updes/utils.py:73-88)."""
    return (rbf if rbf is not None else polyharmonic)(distance(x, node))
