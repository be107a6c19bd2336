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

from updes_gb300 import _lib

pytestmark = pytest.mark.gpu


def _factor(n, precision, seed):
    import torch
    lib = _lib.load()
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 0.5 * np.eye(n)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    F = torch.zeros((n, ld), dtype=torch.float32, device="cuda") if precision else Ad
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, precision, ctypes.byref(nb)), "updes_lu_workspace")
    ws = torch.empty(nb.value + 8 * n * 4 + 1024, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(-1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, precision, F.data_ptr() if precision else None,
                                   ld if precision else 0, piv.data_ptr(), ws.data_ptr(), ws.numel(),
                                   ctypes.byref(info), s), "updes_lu_factor")
    assert info.value == 0
    return A, F, ld, piv, ws, s


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


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    n = _lib.NOALLOC_MAX_N + 1
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    st = lib.updes_lu_solve_noalloc(n, dummy, n, 0, dummy, dummy, 1, 1, 0, None)
    assert st == _lib.ERR_TOO_LARGE
    assert "UPDES_NOALLOC_MAX_N" in _lib.status_string(st)
