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


def test_tagged_hand_off_gives_bitwise_the_counted_one():
    """The 128-row solves hand each solved block to the next through tagged words by default; with
    UPDES_TRSV_TAGS=0 (a fresh process: the switch is read once) they use the finished-block count and
    separate x planes.  Same arithmetic on the same values, so the solves are bitwise equal, GMRES
    iterations included."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, json; sys.path.insert(0, %r)\n"
            "import updes_gb300 as U\nfrom updes_gb300 import workloads as WL\n"
            "s = U.pde_solver_jit(options=U.SolverOptions(precision='fp32', reuse_factorization=False), "
            "**WL.poisson_manufactured(45))\n"
            "print(json.dumps({'vals': s.vals.tolist(), 'iters': U.LAST_INFO['iters']}))\n") % root
    out = {}
    for tags in ("1", "0"):
        env = dict(os.environ, UPDES_TRSV_TAGS=tags)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[tags] = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert out["1"]["iters"] == out["0"]["iters"]
    assert np.array_equal(np.array(out["1"]["vals"]), np.array(out["0"]["vals"]))
