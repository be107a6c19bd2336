"""Reverse-mode differentiation through the GPU solve (torch.autograd).

The reference differentiates ``pde_solver`` with ``jax.grad`` through
``inv`` / GEMM / lineax QR (demos/Laplace/10_laplace_with_diff_phys.py:89-104),
or runs a second full solve for a hand-written adjoint
(demos/Laplace/03_laplace_with_adjoint.py:88-143).  Here the backward pass
reuses the forward LU factors:

    K c = [q; 0],  vals = [Φ P] c
    g      = dJ/dc + [Φ P]ᵀ dJ/dvals            (updes_eval_values_t)
    λ      = K⁻ᵀ g                              (updes_solve_transpose, same factors + FP64 GMRES)
    dJ/dq  = λ[:N]                              (boundary values and interior rhs)
    dJ/dWᵢ = -λᵢ (D c)ᵢ                         (updes_coeff_grad, entries regenerated on the fly)

W are the per-node operator weights captured from ``diff_operator``; their
dependence on the ``diff_args`` fields is linearised at the forward point by
central differences of the (cheap, vectorised) capture, so gradients with
respect to the fields follow by the chain rule.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .operators import DeviceProblem, SolverOptions, boundary_conditions_func_to_arr, capture_operator, prepare


def _torch():
    import torch
    return torch


class _SolveState:
    """One factorised system kept alive for its backward pass."""

    def __init__(self, dp: DeviceProblem, opts: SolverOptions):
        torch = _torch()
        self.dp = dp
        self.opts = opts
        lib = _lib.load()
        self.co = opts.c_opts()
        nbytes = ctypes.c_size_t()
        _lib.check(lib.updes_solve_workspace(ctypes.byref(dp.c), ctypes.byref(self.co), ctypes.byref(nbytes)),
                   "updes_solve_workspace")
        self.ws = torch.empty(nbytes.value, dtype=torch.uint8, device=dp.device)
        self.info = None


class RBFSolve:
    """``vals, coeffs = RBFSolve.apply(q, W, state)``: differentiable in q (N,) and W (Ni, 5)."""

    _fn = None

    @classmethod
    def apply(cls, q, W, state):
        if cls._fn is None:
            cls._fn = _make_function()
        return cls._fn.apply(q, W, state)


def _make_function():
    torch = _torch()

    class _Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, q, W, state):
            dp = state.dp
            lib = _lib.load()
            Wd = W.detach().to(dtype=torch.float64, device=dp.device).contiguous()
            if dp.Ni:
                dp.W = Wd
                dp.c.op_weights = Wd.data_ptr()
            qd = q.detach().to(dtype=torch.float64, device=dp.device).contiguous()
            coeffs = torch.empty(dp.n, dtype=torch.float64, device=dp.device)
            vals = torch.empty(dp.N, dtype=torch.float64, device=dp.device)
            info = _lib.SolveInfo()
            st = lib.updes_solve(ctypes.byref(dp.c), qd.data_ptr(), coeffs.data_ptr(), vals.data_ptr(),
                                 ctypes.byref(state.co), ctypes.byref(info), state.ws.data_ptr(), state.ws.numel(),
                                 dp.stream())
            state.info = info.as_dict()
            _lib.check(st, "updes_solve")
            ctx.state = state
            ctx.save_for_backward(coeffs)
            ctx.w_grad = W.requires_grad
            return vals, coeffs

        @staticmethod
        def backward(ctx, g_vals, g_coeffs):
            state = ctx.state
            dp = state.dp
            (coeffs,) = ctx.saved_tensors
            lib = _lib.load()
            s = dp.stream()
            g = torch.zeros(dp.n, dtype=torch.float64, device=dp.device)
            if g_vals is not None:
                gv = g_vals.detach().to(torch.float64).contiguous()
                _lib.check(lib.updes_eval_values_t(ctypes.byref(dp.c), gv.data_ptr(), g.data_ptr(), s),
                           "updes_eval_values_t")
            if g_coeffs is not None:
                g = g + g_coeffs.detach().to(torch.float64)
            g = g.contiguous()
            lam = torch.empty(dp.n, dtype=torch.float64, device=dp.device)
            info = _lib.SolveInfo()
            st = lib.updes_solve_transpose(ctypes.byref(dp.c), g.data_ptr(), lam.data_ptr(), ctypes.byref(state.co),
                                           ctypes.byref(info), state.ws.data_ptr(), state.ws.numel(), s)
            state.adjoint_info = info.as_dict()
            _lib.check(st, "updes_solve_transpose")
            grad_q = lam[:dp.N].clone()
            grad_W = None
            if ctx.w_grad and dp.Ni:
                grad_W = torch.empty((dp.Ni, 5), dtype=torch.float64, device=dp.device)
                _lib.check(lib.updes_coeff_grad(ctypes.byref(dp.c), coeffs.data_ptr(), lam.data_ptr(),
                                                grad_W.data_ptr(), s), "updes_coeff_grad")
            return grad_q, grad_W, None

    return _Fn


def _field_jacobians(diff_operator, X, rbf, fields, which):
    """dW/dfields[f] per interior node (Ni, 5) for f in ``which``, by central differences of the capture."""
    jac = {}
    for f in which:
        h = 1e-5 * (1.0 + np.abs(fields[f]))
        fp, fm = fields.copy(), fields.copy()
        fp[f] += h
        fm[f] -= h
        Wp = capture_operator(diff_operator, X, rbf, fp)
        Wm = capture_operator(diff_operator, X, rbf, fm)
        jac[f] = (Wp - Wm) / (2.0 * h)[:, None]
    return jac


def pde_solver_torch(diff_operator, rhs_operator, cloud, boundary_conditions, rbf, max_degree, diff_args=None,
                     rhs_args=None, options=None):
    """Differentiable ``pde_solver``: returns ``(vals, coeffs)`` as float64 CUDA tensors.

    Boundary-condition arrays (per facet, in ``cloud.facet_nodes`` order) and
    ``diff_args`` fields (per node) may be torch tensors with
    ``requires_grad``; ``loss.backward()`` then fills their ``.grad`` through
    the adjoint described in the module docstring.
    """
    torch = _torch()
    opts = options or SolverOptions()
    dev = torch.device("cuda", torch.cuda.current_device())

    def as_np(v):
        return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v

    bc_np = {}
    for f, v in boundary_conditions.items():
        bc_np[f] = tuple(as_np(t) for t in v) if isinstance(v, tuple) else as_np(v)
    fields_np = None if diff_args is None else [np.asarray(as_np(a), dtype=np.float64) for a in diff_args]
    W0, kind, bnodes, geom, q0 = prepare(diff_operator, rhs_operator, cloud, bc_np, rbf, max_degree,
                                         diff_args=fields_np, rhs_args=rhs_args, options=opts)
    dp = DeviceProblem(cloud, rbf, max_degree, W0, kind, bnodes, geom, opts.self_term)
    state = _SolveState(dp, opts)
    # q as a function of the boundary tensors
    q = torch.as_tensor(q0, dtype=torch.float64, device=dev)
    for f, v in boundary_conditions.items():
        vv = v[0] if isinstance(v, tuple) else v
        if isinstance(vv, torch.Tensor) and vv.requires_grad and cloud.facet_types[f][0] != "p":
            ids = torch.as_tensor(np.asarray(cloud.facet_nodes[f], dtype=np.int64), device=dev)
            q = q.index_put((ids,), vv.to(device=dev, dtype=torch.float64).expand(ids.shape[0]))
    # W as a function of the field tensors (linearised at the forward point)
    W = torch.as_tensor(W0, dtype=torch.float64, device=dev)
    if diff_args is not None and cloud.Ni:
        which = [i for i, a in enumerate(diff_args) if isinstance(a, torch.Tensor) and a.requires_grad]
        if which:
            F = np.stack(fields_np)[:, :cloud.Ni]
            jac = _field_jacobians(diff_operator, cloud.sorted_nodes[:cloud.Ni], rbf, F, which)
            for i in which:
                d = diff_args[i].to(device=dev, dtype=torch.float64)[:cloud.Ni] - torch.as_tensor(F[i], device=dev)
                W = W + torch.as_tensor(jac[i], device=dev) * d[:, None]
    vals, coeffs = RBFSolve.apply(q, W, state)
    return vals, coeffs
