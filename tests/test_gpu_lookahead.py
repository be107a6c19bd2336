"""GPU: the look-ahead of the mixed LU (next block factored on a second stream beside the trailing update)
gives bitwise the factors of the serial block order, and they satisfy the FP32-level backward error bound."""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Factors a seeded random system with the mixed LU through the C ABI and prints a digest of (F, piv).
_SCRIPT = r"""
import ctypes, hashlib, sys
import numpy as np, torch
sys.path.insert(0, {root!r})
from updes_gb300 import _lib
lib = _lib.load()
for n in {sizes!r}:
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 0.5 * np.eye(n)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    F = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, 1, ctypes.byref(nb)), "ws")
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(-1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, 1, F.data_ptr(), ld, piv.data_ptr(), ws.data_ptr(),
                                   ws.numel(), ctypes.byref(info), s), "factor")
    torch.cuda.synchronize()
    h = hashlib.sha256(F[:, :n].cpu().numpy().tobytes() + piv[:n].cpu().numpy().tobytes()).hexdigest()
    print(n, info.value, h)
"""

SIZES = [1024, 1300, 2113, 12600]  # 12600: the first steps fork after the whole block row, the later ones early


def _digests(lookahead, blocking=False):
    env = dict(os.environ)
    env["UPDES_LOOKAHEAD"] = "1" if lookahead else "0"
    if blocking:
        # every launch completes before the next is issued: the two streams' kernels run in issue order, so a
        # look-ahead kernel that touches data the other stream still needs shows up deterministically
        env["CUDA_LAUNCH_BLOCKING"] = "1"
    out = subprocess.run([sys.executable, "-c", _SCRIPT.format(root=ROOT, sizes=SIZES)], env=env, check=True,
                         capture_output=True, text=True, timeout=600).stdout
    return [line.split() for line in out.strip().splitlines()]


def test_lookahead_factors_bitwise_serial():
    a, b = _digests(True), _digests(False)
    assert len(a) == len(SIZES)
    for (n1, i1, h1), (n2, i2, h2) in zip(a, b):
        assert n1 == n2 and i1 == i2 == "0"
        assert h1 == h2, f"n={n1}: look-ahead factors differ from the serial block order"


def test_lookahead_factors_bitwise_serial_when_serialised():
    """The same with launches serialised in issue order (the side stream's panels are issued before the
    caller's stream applies the previous block's interchanges): the streams share no scratch they race on."""
    a, b = _digests(True, blocking=True), _digests(False)
    for (n1, i1, h1), (n2, i2, h2) in zip(a, b):
        assert n1 == n2 and i1 == i2 == "0"
        assert h1 == h2, f"n={n1}: serialised look-ahead factors differ from the serial block order"


def test_lookahead_backward_error():
    """|P A - L U| <= 2^-22 (|L| |U|) entrywise at a size where the look-ahead runs (several 256-column
    blocks, a ragged last block)."""
    import ctypes
    import torch
    from updes_gb300 import _lib
    lib = _lib.load()
    n = 1300
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 0.5 * np.eye(n)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    F = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, 1, ctypes.byref(nb)), "ws")
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(-1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, 1, F.data_ptr(), ld, piv.data_ptr(), ws.data_ptr(),
                                   ws.numel(), ctypes.byref(info), s), "factor")
    assert info.value == 0
    Fh = F[:, :n].double().cpu().numpy()
    perm = np.arange(n)
    for i, p in enumerate(piv[:n].cpu().numpy()):
        perm[[i, p]] = perm[[p, i]]
    L = np.tril(Fh, -1) + np.eye(n)
    U = np.triu(Fh)
    R = np.abs(A[perm] - L @ U)
    bound = 2.0 ** -22 * (np.abs(L) @ np.abs(U)) + 1e-300
    assert np.all(R <= bound), (R / bound).max()
