"""GPU: the mixed solve's preconditioner with 128-row triangular blocks (two 64-row halves inside a
block) on sizes whose last block is full, has a partial second half, or a single partial half."""
import numpy as np
import pytest

import updes_gb300 as U
from updes_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx", [32, 35, 45])   # n = 1030, 1231, 2031: the last block has 6, 79, 111 rows
def test_mixed_solve_block_shapes(nx):
    sysd = WL.poisson_manufactured(nx)
    s32 = U.pde_solver_jit(options=U.SolverOptions(precision="fp32", reuse_factorization=False), **sysd)
    info = dict(U.LAST_INFO)
    s64 = U.pde_solver_jit(options=U.SolverOptions(precision="fp64", reuse_factorization=False), **sysd)
    assert info["fell_back"] == 0 and info["converged"] == 1, info
    assert np.linalg.norm(s32.vals - s64.vals) <= 1e-8 * np.linalg.norm(s64.vals)
