"""updes_lu_solve_noalloc: the triangular solves for callers that may not allocate.

Some callers cannot allocate device memory where they solve (a handler run by
another framework's executor only gets the buffers that framework planned; a
time-stepping loop may have to stay off the allocator).  This entry point takes
the same factors and right-hand sides as updes_lu_solve but keeps its scratch in
a fixed array inside the library.  The test calls it twice in a row through the
C ABI and checks each result against the workspace-based updes_lu_solve.
"""
import ctypes

import numpy as np
import pytest

from gpu_helpers import lu_factor_random as _factor
from updes_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_noalloc_solve_matches_workspace_solve(precision, nrhs):
    import torch
    lib = _lib.load()
    n = 700
    A, F, ld, piv, ws, s = _factor(n, precision, 11 + precision)
    B = np.random.default_rng(5).standard_normal((n, nrhs))
    for trans in (0, 1):
        Bref = torch.as_tensor(B.copy(), device="cuda")
        _lib.check(lib.updes_lu_solve(n, F.data_ptr(), ld, precision, piv.data_ptr(), Bref.data_ptr(), nrhs, nrhs,
                                      trans, ws.data_ptr(), ws.numel(), s), "updes_lu_solve")
        ref = Bref.cpu().numpy()
        for call in range(2):  # two calls in a row share the library's scratch
            Bd = torch.as_tensor(B.copy(), device="cuda")
            st = lib.updes_lu_solve_noalloc(n, F.data_ptr(), ld, precision, piv.data_ptr(), Bd.data_ptr(), nrhs,
                                            nrhs, trans, s)
            assert st == _lib.OK, _lib.status_string(st)
            got = Bd.cpu().numpy()
            assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), (trans, call)
        # and both agree with the true solution as closely as the factors allow
        want = np.linalg.solve(A.T if trans else A, B)
        assert np.linalg.norm(ref - want) <= (1e-10 if precision == 0 else 1e-3) * np.linalg.norm(want)


@pytest.mark.parametrize("n,nrhs,ldb", [(700, 2, 5), (_lib.NOALLOC_MAX_N - 37, 2, 3)])
def test_noalloc_strided_columns_and_sizes_near_the_limit(n, nrhs, ldb):
    """Right-hand sides that are columns of a wider row-major block (ldb > nrhs) go through the scratch's
    column vector; the largest sizes (not a multiple of the 64-row blocks) fill its flag region.  Both
    against the workspace-based solve, twice in a row, with the block's other columns left untouched."""
    import torch
    lib = _lib.load()
    A, F, ld, piv, ws, s = _factor(n, 1, 31)
    B = np.random.default_rng(7).standard_normal((n, ldb))
    for trans in (0, 1):
        Bref = torch.as_tensor(B.copy(), device="cuda")
        _lib.check(lib.updes_lu_solve(n, F.data_ptr(), ld, 1, piv.data_ptr(), Bref.data_ptr(), nrhs, ldb, trans,
                                      ws.data_ptr(), ws.numel(), s), "updes_lu_solve")
        ref = Bref.cpu().numpy()
        for call in range(2):
            Bd = torch.as_tensor(B.copy(), device="cuda")
            st = lib.updes_lu_solve_noalloc(n, F.data_ptr(), ld, 1, piv.data_ptr(), Bd.data_ptr(), nrhs, ldb,
                                            trans, s)
            assert st == _lib.OK, _lib.status_string(st)
            got = Bd.cpu().numpy()
            assert np.linalg.norm(got[:, :nrhs] - ref[:, :nrhs]) <= 1e-12 * np.linalg.norm(ref[:, :nrhs]), (trans, call)
            np.testing.assert_array_equal(got[:, nrhs:], B[:, nrhs:])
    del A, F, ws
    torch.cuda.empty_cache()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    n = _lib.NOALLOC_MAX_N + 1
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    st = lib.updes_lu_solve_noalloc(n, dummy, n, 0, dummy, dummy, 1, 1, 0, None)
    assert st == _lib.ERR_TOO_LARGE
    assert "UPDES_NOALLOC_MAX_N" in _lib.status_string(st)
