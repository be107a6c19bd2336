"""Many independent systems in one persistent launch, with a panel-width autotuner.

The reference solves each system with its own ``pde_solver`` call (updes/operators.py:559-618).
``pde_solver_batched`` prepares every system on the host exactly as ``pde_solver`` does (operator capture,
boundary rows, right-hand side) and hands them all to ``updes_solve_batched``: one CTA per SM takes systems
from a device work queue, largest first, and runs each one's assembly, LU, refinement and values by itself.

Precision per system:

* ``"fp32"`` -- the elimination in double-float arithmetic on the FP32 pipes (about 48-bit factors) with
  classical refinement sweeps on an FP64 residual;
* ``"fp64"`` -- the elimination in FP64;
* ``"auto"`` (default) -- ``"fp32"`` first.  Refinement goes on while the componentwise backward error
  still halves (converged: at most 32 FP64 unit roundoffs): beyond a condition number of about 2^48 the 48-bit factors
  no longer contract the error, and the answer keeps the backward error the elimination gave it (a few
  1e-14 on the uneven-cloud workload's flattest Gaussian systems, whose forward error no FP64 solver
  bounds either).  A system whose backward error stays above ``RELAUNCH_BACKWARD_ERROR`` (1e-12), or whose
  elimination met a zero pivot, is solved again in FP64 in a second launch of only those systems.

The autotuner (``PanelTuner``) picks the LU panel width per (GPU, kernel, precision, size bucket): it times
one launch on a single CTA for each candidate width on the largest system of the bucket in the batch, keeps
the fastest, and caches the choice in memory and, unless disabled, in a JSON file
(``$UPDES_TUNE_CACHE`` or ``~/.cache/updes_gb300/panel_widths.json``).
"""
from __future__ import annotations

import ctypes
import json
import os
import threading

from . import _lib
from .operators import (DEFAULT_OPTIONS, CollocationMatrix, SteadySol, _torch, boundary_conditions_func_to_arr,
                        compute_nb_monomials, materialize_B, prepare)
from .rbf import rbf_spec

PANEL_CANDIDATES = (16, 32, 64)
SIZE_BUCKETS = (256, 512, 1024, 2048, 4096)
MAX_N = 4096
RELAUNCH_BACKWARD_ERROR = 1e-12
LAST_BATCHED_INFO: list = []
LAST_BATCHED_TIMING: dict = {}


def size_bucket(n: int) -> int:
    for b in SIZE_BUCKETS:
        if n <= b:
            return b
    raise ValueError(f"systems of n = {n} unknowns exceed the batched solver's limit of {MAX_N}")


def _default_cache_path():
    path = os.environ.get("UPDES_TUNE_CACHE")
    if path is not None:
        return path or None  # an empty value disables the file cache
    return os.path.join(os.path.expanduser("~"), ".cache", "updes_gb300", "panel_widths.json")


class PanelTuner:
    """Panel widths of the batched LU by (GPU, kernel, precision, size bucket), measured on first use.

    ``measure(width) -> milliseconds`` is supplied by the caller for the system that represents a bucket; the tuner calls it for every candidate and keeps the fastest.  Choices persist in
    ``cache_path`` (JSON; None keeps them in memory only).
    """

    def __init__(self, cache_path="default", candidates=PANEL_CANDIDATES):
        self.cache_path = _default_cache_path() if cache_path == "default" else cache_path
        self.candidates = tuple(candidates)
        self._lock = threading.Lock()
        self.table = {}
        self.measurements = {}
        if self.cache_path and os.path.exists(self.cache_path):
            try:
                with open(self.cache_path) as fh:
                    self.table = {k: int(v) for k, v in json.load(fh).items()}
            except (OSError, ValueError):
                self.table = {}

    @staticmethod
    def key(gpu: str, kind: int, precision: str, bucket: int) -> str:
        return f"{gpu}|rbf{kind}|{precision}|n<={bucket}"

    def width(self, key: str, measure) -> int:
        with self._lock:
            if key in self.table:
                return self.table[key]
        times = {w: float(measure(w)) for w in self.candidates}
        best = min(times, key=lambda w: (times[w], w))
        with self._lock:
            self.table[key] = best
            self.measurements[key] = times
            self._save()
        return best

    def _save(self):
        if not self.cache_path:
            return
        try:
            os.makedirs(os.path.dirname(self.cache_path), exist_ok=True)
            tmp = self.cache_path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(self.table, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.cache_path)
        except OSError:
            pass  # a read-only home directory keeps the choices in memory


_TUNER = None


def default_tuner() -> PanelTuner:
    global _TUNER
    if _TUNER is None:
        _TUNER = PanelTuner()
    return _TUNER


def _align(k: int, unit: int) -> int:
    return (k + unit - 1) // unit * unit


def _pack_layout(sizes):
    """Offsets, in elements, of every system's arrays in the batch's packed buffers, each array starting on a
    256-byte boundary (32 doubles, 64 ints).  ``sizes``: (N, Ni, n) per system.  Returns (f64 offsets of nodes
    (2N), operator weights (5 Ni), boundary geometry (8 Nb) and q (N); int32 offsets of boundary kinds (Nb) and
    node pairs (2 Nb); output offsets of coefficients (n) and values (N); the three buffers' lengths)."""
    f_off, i_off, o_off = [], [], []
    fpos = ipos = opos = 0
    for N, Ni, n in sizes:
        Nb = N - Ni
        offs = []
        for sz in (2 * N, 5 * Ni, 8 * Nb, N):
            offs.append(fpos)
            fpos = _align(fpos + sz, 32)
        f_off.append(offs)
        kinds = ipos
        pairs = _align(kinds + Nb, 64)
        i_off.append((kinds, pairs))
        ipos = _align(pairs + 2 * Nb, 64)
        co = opos
        vo = _align(co + n, 32)
        o_off.append((co, vo))
        opos = _align(vo + N, 32)
    return f_off, i_off, o_off, (fpos, ipos, opos)


class _PackedProblem:
    """One system of a batch: sizes, kernel and the ``updes_problem`` struct, whose arrays live in the batch's
    packed device buffers (the object keeps them alive)."""

    def __init__(self, cloud, rbf, max_degree, device, keep):
        self.torch = _torch()
        self.device = device
        self.N, self.Ni = cloud.N, cloud.Ni
        self.M = compute_nb_monomials(max_degree)
        self.n = self.N + self.M
        self.kid, self.param = rbf_spec(rbf)
        self.keep = keep
        self.c = _lib.Problem()

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)


class _Batch:
    """Every system's arrays packed into a few device buffers (one host-to-device copy per element type), the
    C structs pointing into them, and one output buffer for all coefficients and values."""

    def __init__(self, clouds, rbfs, degrees, prepared, self_term):
        import numpy as np
        torch = _torch()
        self.torch = torch
        dev = torch.device("cuda", torch.cuda.current_device())
        c = len(prepared)
        self.count = c
        f_off, i_off, o_off, (fpos, ipos, opos) = _pack_layout(
            [(cl.N, cl.Ni, cl.N + compute_nb_monomials(deg)) for cl, deg in zip(clouds, degrees)])
        fh = np.zeros(max(fpos, 1), dtype=np.float64)
        ih = np.zeros(max(ipos, 1), dtype=np.int32)
        for cl, (W, kind, bnodes, geom, q), fo, io in zip(clouds, prepared, f_off, i_off):
            N, Ni, Nb = cl.N, cl.Ni, cl.N - cl.Ni
            fh[fo[0]:fo[0] + 2 * N] = np.asarray(cl.sorted_nodes, dtype=np.float64).ravel()
            fh[fo[1]:fo[1] + 5 * Ni] = np.asarray(W, dtype=np.float64).ravel()
            fh[fo[2]:fo[2] + 8 * Nb] = np.asarray(geom, dtype=np.float64).ravel()
            fh[fo[3]:fo[3] + N] = np.asarray(q, dtype=np.float64)
            ih[io[0]:io[0] + Nb] = np.asarray(kind, dtype=np.int32)
            ih[io[1]:io[1] + 2 * Nb] = np.asarray(bnodes, dtype=np.int32).ravel()
        self.fbuf = torch.from_numpy(fh).to(dev)
        self.ibuf = torch.from_numpy(ih).to(dev)
        self.obuf = torch.empty(max(opos, 1), dtype=torch.float64, device=dev)
        fb, ib, ob = self.fbuf.data_ptr(), self.ibuf.data_ptr(), self.obuf.data_ptr()
        keep = (self.fbuf, self.ibuf)
        self.dps = []
        qv, cv, vv = [], [], []
        for cl, rbf, deg, fo, io, oo in zip(clouds, rbfs, degrees, f_off, i_off, o_off):
            dp = _PackedProblem(cl, rbf, deg, dev, keep)
            p = dp.c
            p.N, p.Ni, p.M, p.rbf, p.rbf_param = dp.N, dp.Ni, dp.M, dp.kid, dp.param
            p.self_term = int(bool(self_term))
            p.nodes = fb + 8 * fo[0]
            p.op_weights = fb + 8 * fo[1] if dp.Ni else None
            has_bd = dp.N > dp.Ni
            p.bd_kind = ib + 4 * io[0] if has_bd else None
            p.bd_node = ib + 4 * io[1] if has_bd else None
            p.bd_geom = fb + 8 * fo[2] if has_bd else None
            self.dps.append(dp)
            qv.append(fb + 8 * fo[3])
            cv.append(ob + 8 * oo[0])
            vv.append(ob + 8 * oo[1])
        self.o_off = o_off
        self.probs = (_lib.Problem * c)(*[dp.c for dp in self.dps])
        ptrs = lambda vs: (ctypes.c_void_p * c)(*vs)
        self.qp, self.cp, self.vp = ptrs(qv), ptrs(cv), ptrs(vv)
        self.infos = (_lib.SolveInfo * c)()

    def results(self):
        """(coeffs, vals) of every system as host arrays, from one device-to-host copy."""
        host = self.obuf.cpu().numpy()
        return [(host[co:co + dp.n].copy(), host[vo:vo + dp.N].copy()) for dp, (co, vo) in zip(self.dps, self.o_off)]

    def run(self, idx, precisions, widths, max_sweeps, ctas):
        """Solve the systems ``idx`` (host indices into the batch) in one launch; returns the status."""
        torch, lib = self.torch, _lib.load()
        c = len(idx)
        sub = lambda arr, T: (T * c)(*[arr[i] for i in idx])
        probs = sub(self.probs, _lib.Problem)
        qp, cp, vp = sub(self.qp, ctypes.c_void_p), sub(self.cp, ctypes.c_void_p), sub(self.vp, ctypes.c_void_p)
        prec = (ctypes.c_int32 * c)(*[precisions[i] for i in idx])
        wid = (ctypes.c_int32 * c)(*[widths[i] for i in idx])
        infos = (_lib.SolveInfo * c)()
        nbytes = ctypes.c_size_t()
        _lib.check(lib.updes_solve_batched_workspace(probs, c, int(ctas), ctypes.byref(nbytes)),
                   "updes_solve_batched_workspace")
        ws = _workspace(nbytes.value, self.dps[0].device)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        st = lib.updes_solve_batched(probs, c, ctypes.cast(qp, ctypes.c_void_p), ctypes.cast(cp, ctypes.c_void_p),
                                     ctypes.cast(vp, ctypes.c_void_p), prec, wid, int(max_sweeps), int(ctas), infos,
                                     ws.data_ptr(), ws.numel(), stream)
        for k, i in enumerate(idx):
            self.infos[i] = infos[k]
        return st


_WS: dict = {}


def _workspace(nbytes, device):
    torch = _torch()
    buf = _WS.get(device.index)
    if buf is None or buf.numel() < nbytes:
        _WS.pop(device.index, None)
        buf = torch.empty(int(nbytes), dtype=torch.uint8, device=device)
        _WS[device.index] = buf
    return buf


def free_workspace():
    _WS.clear()


def _tune_widths(batch, precisions, tuner, max_sweeps):
    """Panel width per system from the tuner, measuring each new (kernel, precision, bucket) on the largest
    system of that bucket in the batch with one CTA."""
    torch = batch.torch
    gpu = torch.cuda.get_device_name(batch.dps[0].device)
    groups = {}
    for i, dp in enumerate(batch.dps):
        key = PanelTuner.key(gpu, dp.kid, "fp64" if precisions[i] == _lib.PREC_FP64 else "fp32", size_bucket(dp.n))
        if key not in groups or dp.n > batch.dps[groups[key]].n:
            groups[key] = i
    widths = [16] * batch.count
    chosen = {}
    for key, rep in groups.items():
        def measure(w, rep=rep):
            ws = [w] * batch.count
            batch.run([rep], precisions, ws, max_sweeps, 1)  # loads the kernel, touches the workspace
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            batch.run([rep], precisions, ws, max_sweeps, 1)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)
        chosen[key] = tuner.width(key, measure)
    for i, dp in enumerate(batch.dps):
        key = PanelTuner.key(gpu, dp.kid, "fp64" if precisions[i] == _lib.PREC_FP64 else "fp32", size_bucket(dp.n))
        widths[i] = chosen[key]
    return widths


def pde_solver_batched(systems, options=None, precision="auto", max_sweeps=4, ctas=0, tuner="default"):
    """Solve many independent systems in one persistent launch (``updes_solve_batched``).

    ``systems``: dicts with the keyword arguments of ``pde_solver`` (as for ``pde_solver_many``); callable
    boundary conditions are evaluated as in ``pde_solver_jit``.  ``precision``: ``"auto"``, ``"fp32"``,
    ``"fp64"`` or one of them per system.  ``tuner``: a ``PanelTuner``, ``"default"`` (the process-wide one)
    or None (panel width 16 everywhere).  Returns a list of ``SteadySol`` in the order of ``systems``;
    ``LAST_BATCHED_INFO`` holds each solve's report (sweeps, converged, backward_error, precision used).
    """
    import time
    torch = _torch()
    opts = options or DEFAULT_OPTIONS
    t0 = time.perf_counter()
    prepared = []
    for sysd in systems:
        cloud = sysd["cloud"]
        n = cloud.N + compute_nb_monomials(sysd["max_degree"])
        if n > MAX_N:
            raise ValueError(f"system of n = {n} unknowns exceeds the batched solver's limit of {MAX_N}")
        bcs = boundary_conditions_func_to_arr(sysd["boundary_conditions"], cloud)
        prepared.append(prepare(sysd["diff_operator"], sysd["rhs_operator"], cloud, bcs, sysd["rbf"],
                                sysd["max_degree"], sysd.get("diff_args"), sysd.get("rhs_args"), opts))
    if not prepared:
        return []
    for sysd in systems:
        if getattr(sysd["cloud"], "sorted_local_supports", None) is not None:
            raise _lib.UpdesError(_lib.ERR_UNSUPPORTED, "updes_solve_batched (local supports)")
    batch = _Batch([s["cloud"] for s in systems], [s["rbf"] for s in systems], [s["max_degree"] for s in systems],
                   prepared, opts.self_term)
    dps = batch.dps
    names = precision if isinstance(precision, (list, tuple)) else [precision] * len(dps)
    code = {"fp32": _lib.PREC_FP32, "auto": _lib.PREC_FP32, "fp64": _lib.PREC_FP64}
    precs = [code[p] for p in names]
    tuner = default_tuner() if tuner == "default" else tuner
    widths = _tune_widths(batch, precs, tuner, max_sweeps) if tuner is not None else [16] * len(dps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    st = batch.run(list(range(len(dps))), precs, widths, max_sweeps, ctas)
    e1.record()
    used = ["fp64" if p == _lib.PREC_FP64 else "fp32" for p in precs]
    redo = [i for i, nm in enumerate(names) if nm == "auto" and (batch.infos[i].lu_info != 0 or not
                                                                  batch.infos[i].backward_error <= RELAUNCH_BACKWARD_ERROR)]
    if redo:
        precs2 = list(precs)
        for i in redo:
            precs2[i] = _lib.PREC_FP64
            used[i] = "fp64 (after fp32)"
        w2 = _tune_widths(batch, precs2, tuner, max_sweeps) if tuner is not None else widths
        e1.record()
        st2 = batch.run(redo, precs2, w2, max_sweeps, ctas)
        if st == _lib.OK or st == _lib.ERR_SINGULAR:
            st = st2 if st2 != _lib.OK else st
    e2.record()
    torch.cuda.synchronize()
    LAST_BATCHED_TIMING.clear()
    LAST_BATCHED_TIMING.update(host_prepare_s=t1 - t0, launch_ms=e0.elapsed_time(e1),
                               fp64_relaunch_ms=e1.elapsed_time(e2), relaunched=len(redo))
    LAST_BATCHED_INFO[:] = [dict(batch.infos[i].as_dict(), precision=used[i], panel_width=widths[i])
                            for i in range(len(dps))]
    _lib.check(st, "updes_solve_batched")
    out = []
    for sysd, dp, (c, v) in zip(systems, dps, batch.results()):
        cloud, rbf, deg = sysd["cloud"], sysd["rbf"], sysd["max_degree"]
        out.append(SteadySol(v, c, CollocationMatrix(lambda dp=dp, cloud=cloud, rbf=rbf, deg=deg:
                                                     materialize_B(dp, cloud, rbf, deg))))
    return out
