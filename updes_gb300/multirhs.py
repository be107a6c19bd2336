"""Many right-hand sides against one collocation system, and implicit time stepping on the GPU.

The reference advances time-dependent problems by calling ``pde_solver_jit`` once
per step and per initial condition, rebuilding and refactoring the same matrix
each time (demos/Advection/00_advection_with_rbf.py:83-93, with the rhs
``u_prev / dt`` of its ``my_rhs_operator``).  Here the system is assembled and
factored once (``updes_factor``, FP64 by default: the factorisation is paid once,
while every step applies the factors, so their accuracy is what matters); each
call then solves R <= 64 right-hand sides together (``updes_solve_batch``: the
factors applied in double-float arithmetic on the FP32 pipes, a fixed number of
refinement sweeps with a double-float residual) and evaluates
``vals = [Phi P] C`` for all of them (``updes_eval_values_batch``).
Nothing in a step reads back to the host, so ``implicit_steps`` records one step
into a CUDA graph and replays it.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .operators import (DEFAULT_OPTIONS, DeviceProblem, SolverOptions, _system_key, compute_nb_monomials,
                        prepare)

MAX_RHS = 64


class MultiRHSSolver:
    """One system ``K c = q`` (the operator and boundary rows of ``pde_solver``), factored once.

    ``boundary_conditions`` fixes the boundary values used by ``implicit_steps``
    (the same for every column); ``solve`` takes complete right-hand sides.
    ``sweeps`` is the number of refinement sweeps after the first solve.  With the default FP64
    factors one sweep brings every column to FP64 accuracy; FP32 factors (``precision="fp32"``)
    contract only as fast as their conditioning allows and need more.
    """

    def __init__(self, diff_operator, cloud, boundary_conditions, rbf, max_degree, diff_args=None, options=None,
                 sweeps=1):
        self.opts = options or SolverOptions(precision="fp64")
        from .operators import _torch
        torch = _torch()
        self.torch = torch
        zero_rhs = lambda x, centers, rbf, fields: 0.0 * x[0]
        W, kind, bnodes, geom, q = prepare(diff_operator, zero_rhs, cloud, boundary_conditions, rbf, max_degree,
                                           diff_args, None, self.opts)
        self.cloud = cloud
        self.dp = DeviceProblem(cloud, rbf, max_degree, W, kind, bnodes, geom, self.opts.self_term)
        self.N, self.Ni, self.n = self.dp.N, self.dp.Ni, self.dp.n
        self.q_boundary = torch.as_tensor(q[self.Ni:], dtype=torch.float64, device=self.dp.device)
        self.sweeps = int(sweeps)
        self.key = _system_key(cloud, rbf, max_degree, W, kind, bnodes, geom, self.opts)
        lib = _lib.load()
        co = self.opts.c_opts()
        nbytes = ctypes.c_size_t()
        _lib.check(lib.updes_solve_workspace(ctypes.byref(self.dp.c), ctypes.byref(co), ctypes.byref(nbytes)),
                   "updes_solve_workspace")
        self.ws = torch.empty(nbytes.value, dtype=torch.uint8, device=self.dp.device)
        bbytes = ctypes.c_size_t()
        _lib.check(lib.updes_batch_workspace(self.n, ctypes.byref(bbytes)), "updes_batch_workspace")
        self.bws = torch.empty(bbytes.value, dtype=torch.uint8, device=self.dp.device)
        fi = _lib.SolveInfo()
        _lib.check(lib.updes_factor(ctypes.byref(self.dp.c), ctypes.byref(co), ctypes.byref(fi), self.ws.data_ptr(),
                                    self.ws.numel(), self.dp.stream()), "updes_factor")
        self.factor_info = fi.as_dict()
        _lib.check(lib.updes_batch_prepare(ctypes.byref(self.dp.c), self.ws.data_ptr(), self.ws.numel(),
                                           self.bws.data_ptr(), self.bws.numel(), self.dp.stream()),
                   "updes_batch_prepare")

    # -- device calls (stream-ordered, no host reads) -------------------------------------------------
    def _solve_into(self, Q, C, stream):
        lib = _lib.load()
        R = Q.shape[1]
        st = lib.updes_solve_batch(ctypes.byref(self.dp.c), R, Q.data_ptr(), Q.stride(0), C.data_ptr(), C.stride(0),
                                   self.sweeps, self.ws.data_ptr(), self.ws.numel(), self.bws.data_ptr(),
                                   self.bws.numel(), stream)
        _lib.check(st, "updes_solve_batch")

    def _eval_into(self, C, V, stream):
        lib = _lib.load()
        st = lib.updes_eval_values_batch(ctypes.byref(self.dp.c), C.shape[1], C.data_ptr(), C.stride(0),
                                         V.data_ptr(), V.stride(0), stream)
        _lib.check(st, "updes_eval_values_batch")

    def check_status(self):
        """Raise if a device-side wait or the factor check of an earlier batched call failed (syncs)."""
        lib = _lib.load()
        err = ctypes.c_int32(0)
        _lib.check(lib.updes_workspace_status(ctypes.byref(self.dp.c), self.ws.data_ptr(), self.ws.numel(),
                                              ctypes.byref(err), self.dp.stream()), "updes_workspace_status")
        _lib.check(err.value, "batched solve (device status)")

    def _as_block(self, Q):
        torch = self.torch
        Q = torch.as_tensor(Q, dtype=torch.float64, device=self.dp.device)
        if Q.dim() == 1:
            Q = Q[:, None]
        if Q.shape[0] != self.N or not 1 <= Q.shape[1] <= MAX_RHS:
            raise ValueError(f"right-hand sides must be ({self.N}, R) with 1 <= R <= {MAX_RHS}")
        return Q.contiguous()

    # -- public --------------------------------------------------------------------------------------
    def solve(self, Q, want_vals=True):
        """coeffs (n, R) and vals (N, R) for the right-hand-side columns Q (N, R); device tensors."""
        torch = self.torch
        Q = self._as_block(Q)
        R = Q.shape[1]
        C = torch.empty((self.n, R), dtype=torch.float64, device=self.dp.device)
        s = self.dp.stream()
        self._solve_into(Q, C, s)
        V = None
        if want_vals:
            V = torch.empty((self.N, R), dtype=torch.float64, device=self.dp.device)
            self._eval_into(C, V, s)
        self.check_status()
        return C, V

    def implicit_steps(self, U0, steps, rhs_scale, rhs_const=None, graph=True):
        """Advance ``steps`` implicit steps of  (operator) u_new = rhs_scale * u_old + rhs_const  (interior)
        with the boundary values of ``boundary_conditions``; U0 (N, R) nodal values.  Returns U (N, R).

        For implicit Euler on  u_t + L u = f  the operator is ``u/dt + L u`` and rhs_scale = 1/dt.
        With ``graph=True`` one step is captured in a CUDA graph and replayed.
        """
        torch = self.torch
        U = self._as_block(U0).clone()
        R = U.shape[1]
        Ni = self.Ni
        Q = torch.empty((self.N, R), dtype=torch.float64, device=self.dp.device)
        Q[Ni:] = self.q_boundary[:, None]
        C = torch.empty((self.n, R), dtype=torch.float64, device=self.dp.device)
        F = None
        if rhs_const is not None:
            F = torch.as_tensor(rhs_const, dtype=torch.float64, device=self.dp.device)
            F = (F[:, None] if F.dim() == 1 else F)[:Ni].expand(Ni, R).contiguous()

        def step():
            torch.mul(U[:Ni], float(rhs_scale), out=Q[:Ni])
            if F is not None:
                Q[:Ni].add_(F)
            s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            self._solve_into(Q, C, s)
            self._eval_into(C, U, s)

        if steps <= 0:
            return U
        if not graph:
            for _ in range(steps):
                step()
            self.check_status()
            return U
        # warm up on a side stream (loads modules, sets kernel attributes), then capture one step
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        U_init = U.clone()
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        U.copy_(U_init)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step()
        for _ in range(steps):
            g.replay()
        self.check_status()
        self.last_graph = g
        return U

    def make_graph(self, U, steps_per_graph=1, rhs_scale=1.0):
        """A CUDA graph of ``steps_per_graph`` steps on the static block U (N, R) in place: replay advances U."""
        torch = self.torch
        R = U.shape[1]
        Ni = self.Ni
        Q = torch.empty((self.N, R), dtype=torch.float64, device=self.dp.device)
        Q[Ni:] = self.q_boundary[:, None]
        C = torch.empty((self.n, R), dtype=torch.float64, device=self.dp.device)

        def step():
            torch.mul(U[:Ni], float(rhs_scale), out=Q[:Ni])
            s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            self._solve_into(Q, C, s)
            self._eval_into(C, U, s)

        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        keep = U.clone()
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        U.copy_(keep)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(steps_per_graph):
                step()
        g._updes_buffers = (Q, C)   # keep the captured buffers alive with the graph
        return g
