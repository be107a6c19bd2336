"""``pde_solver`` as a JAX function with a custom VJP (eager mode), over DLPack.

The reference is differentiated with ``jax.grad`` through its own solve
(demos/Laplace/10_laplace_with_diff_phys.py:89-104).  This bridge gives a JAX
caller the same ``jax.grad``/``jax.vjp`` interface on top of the GPU solve and
its adjoint (``updes_gb300.adjoint``): arrays cross between JAX and PyTorch by
DLPack, without copies when both live on the same GPU, and the backward pass
reuses the forward factors through torch autograd.

The forward pass captures the operator on the host (it needs concrete values),
so the bridge is for eager use: ``jax.grad(loss)(control)`` works, ``jax.jit``
around it does not.  JAX is imported lazily; without it ``pde_solver_jax``
raises ``ImportError``.
"""
from __future__ import annotations

import itertools
import threading

_TAPES: dict = {}          # handle -> (torch inputs, torch outputs) kept for the backward pass
_LOCK = threading.Lock()
_NEXT = itertools.count(1)


def _to_torch(x):
    import torch
    return torch.from_dlpack(x)


def _to_jax(t):
    import jax.dlpack
    return jax.dlpack.from_dlpack(t.contiguous())


def pde_solver_jax(diff_operator, rhs_operator, cloud, rbf, max_degree, bc_template, diff_operator_fields=False,
                   options=None):
    """Return ``f(bc_values, fields) -> (vals, coeffs)`` as a JAX function with a custom VJP.

    ``bc_template``: dict facet -> boundary values (arrays, or callables evaluated once); the facets
    listed in ``bc_values`` (a dict of JAX arrays, one value per facet node) override them and are
    differentiable.  ``fields``: a tuple of JAX arrays passed as ``diff_args`` (differentiable when
    ``diff_operator_fields`` is true, else ignored by the VJP).
    """
    import jax
    import torch

    from .adjoint import pde_solver_torch

    def run_torch(bc_values, fields, requires_grad):
        bcs = dict(bc_template)
        tin = []
        for f, v in bc_values.items():
            t = _to_torch(v).to(torch.float64).requires_grad_(requires_grad)
            bcs[f] = t
            tin.append(t)
        targs = None
        if fields:
            targs = []
            for v in fields:
                t = _to_torch(v).to(torch.float64).requires_grad_(requires_grad and diff_operator_fields)
                targs.append(t)
                tin.append(t)
        vals, coeffs = pde_solver_torch(diff_operator, rhs_operator, cloud, bcs, rbf, max_degree, diff_args=targs,
                                        options=options)
        return tin, (vals, coeffs)

    @jax.custom_vjp
    def solve(bc_values, fields):
        _, (vals, coeffs) = run_torch(bc_values, fields, False)
        return _to_jax(vals.detach()), _to_jax(coeffs.detach())

    def fwd(bc_values, fields):
        tin, (vals, coeffs) = run_torch(bc_values, fields, True)
        handle = next(_NEXT)
        with _LOCK:
            _TAPES[handle] = (tin, (vals, coeffs))
        return (_to_jax(vals.detach()), _to_jax(coeffs.detach())), (handle, bc_values, fields)

    def bwd(res, cot):
        handle, bc_values, fields = res
        with _LOCK:
            tin, outs = _TAPES.pop(handle)
        g_vals, g_coeffs = (_to_torch(c).to(torch.float64) for c in cot)
        needs = [t for t in tin if t.requires_grad]
        grads = torch.autograd.grad(outs, needs, grad_outputs=(g_vals, g_coeffs), allow_unused=True)
        it = iter(grads)
        out_bc = {}
        for f, v in bc_values.items():
            g = next(it)
            out_bc[f] = _to_jax(g) if g is not None else jax.numpy.zeros_like(v)
        out_fields = fields
        if fields:
            gf = []
            for v in fields:
                g = next(it) if diff_operator_fields else None
                gf.append(_to_jax(g) if g is not None else jax.numpy.zeros_like(v))
            out_fields = tuple(gf)
        return out_bc, out_fields

    solve.defvjp(fwd, bwd)
    return solve
