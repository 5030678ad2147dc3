"""Batched serving of many independent FP32 simulations on one GPU (ffs_server_* in the
C ABI). Each request is one run_simulation() of the reference (src/FluidFlowSimulation.jl
23-65) for `nt` steps with its own parameters and initial fields; requests that arrive
while others run are admitted as memory and batch slots free up, and all admitted runs
advance together, one batched step per CUDA-graph replay.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .globalfile import parameters


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


STATUS = {0: "done", _lib.FFS_QUEUED: "queued", _lib.FFS_RUNNING: "running"}


class Server:
    """Python mirror of ffs_server: submit / poll / wait / results."""

    def __init__(self, device: int = 0, memory_budget: int = 120 << 30, max_active: int = 256, max_n: int = 128,
                 autotune: bool = False, class_forms: int = 0):
        self.L = _lib.load()
        cfg = _lib.FFSServerCfg()
        self.L.ffs_server_default(ctypes.byref(cfg))
        cfg.device, cfg.memory_budget, cfg.max_active, cfg.max_n = device, int(memory_budget), max_active, max_n
        cfg.autotune = int(autotune)
        cfg.class_forms = int(class_forms)
        h = ctypes.c_void_p()
        rc = self.L.ffs_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise _lib.FFSError(rc, self.L.ffs_server_last_error(None).decode())
        self.h = h
        self._shape = {}

    def _check(self, rc):
        if rc < 0:
            raise _lib.FFSError(rc, self.L.ffs_server_last_error(self.h).decode())
        return rc

    def submit(self, d_or_params, u, nt: int, keep_fields: bool = False) -> int:
        """Queue one run: `global` dict (or FFSParams), fields (u1, u2, u3) as [nz][ny][nx]."""
        p = d_or_params if isinstance(d_or_params, _lib.FFSParams) else parameters(d_or_params, precision="FP32")
        u = [np.ascontiguousarray(x, dtype=np.float64) for x in u]
        r = _lib.FFSRequest()
        r.params = p
        r.u1, r.u2, r.u3 = (_ptr(x) for x in u)
        r.nt = int(nt)
        r.keep_fields = 1 if keep_fields else 0
        rid = ctypes.c_uint64()
        self._check(self.L.ffs_submit(self.h, ctypes.byref(r), ctypes.byref(rid)))
        self._shape[rid.value] = u[0].shape
        return rid.value

    @staticmethod
    def _dict(res) -> dict:
        return {"status": res.status, "state": STATUS.get(res.status, "error"), "iteration": res.iteration,
                "time": res.time, "dt": res.dt, "stats_rows": res.stats_rows, "record_ncols": res.record_ncols,
                "submit_s": res.submit_s, "admit_s": res.admit_s, "done_s": res.done_s}

    def poll(self, rid: int) -> dict:
        res = _lib.FFSResult()
        self._check(self.L.ffs_poll(self.h, rid, ctypes.byref(res)))
        return self._dict(res)

    def wait(self, rid: int, timeout: float = 3600.0) -> dict:
        res = _lib.FFSResult()
        self._check(self.L.ffs_wait(self.h, rid, float(timeout), ctypes.byref(res)))
        out = self._dict(res)
        if res.status < 0:
            raise _lib.FFSError(res.status, self.L.ffs_server_last_error(self.h).decode())
        return out

    def pause(self, on: bool = True) -> None:
        """Hold admission (queued requests wait) or resume it."""
        self._check(self.L.ffs_server_pause(self.h, 1 if on else 0))

    def stats_rows(self, rid: int) -> np.ndarray:
        n = self._check(self.L.ffs_fetch_stats(self.h, rid, None, 0))
        res = _lib.FFSResult()
        self._check(self.L.ffs_poll(self.h, rid, ctypes.byref(res)))
        out = np.zeros((n, max(res.record_ncols, 1)))
        if n:
            self._check(self.L.ffs_fetch_stats(self.h, rid, _ptr(out), n))
        return out

    def fields(self, rid: int):
        shape = self._shape[rid]
        u = [np.zeros(shape) for _ in range(3)]
        self._check(self.L.ffs_fetch_fields(self.h, rid, *(_ptr(x) for x in u)))
        return tuple(u)

    def cancel(self, rid: int) -> None:
        """Cancel a queued or running request (it finishes with FFS_ECANCELED)."""
        self._check(self.L.ffs_cancel(self.h, rid))

    def release(self, rid: int) -> None:
        self._check(self.L.ffs_release(self.h, rid))
        self._shape.pop(rid, None)

    @property
    def tuning(self) -> str:
        """The size-class autotuner's report ('' without autotune)."""
        n = self._check(self.L.ffs_server_tuning(self.h, None, 0))
        buf = ctypes.create_string_buffer(n + 1)
        self.L.ffs_server_tuning(self.h, buf, n + 1)
        return buf.value.decode()

    def info(self) -> dict:
        i = _lib.FFSServerInfo()
        self._check(self.L.ffs_server_stats(self.h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in _lib.FFSServerInfo._fields_}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.ffs_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
