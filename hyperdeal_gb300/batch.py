"""Batched uneven advection instances over the C ABI (hd_batch_*).

The reference runs independent problems one after the other, each with its
own compile-time (dim, degree) instantiation (examples/advection/
advection.cc:26-48, :253-259).  ``AdvectionBatch`` advances many
``AdvectionOperation`` instances together: instances of one class (phase-space
dimension, degree, dtype) share ONE persistent kernel launch per RK stage
(classes with 4 or 5 dimensions and degree 2..5; other classes launch per
instance), a two-step CUDA graph can be recorded and replayed, and
``autotune`` picks each class's tile (cells per CTA, CTAs per SM) by timing.
"""
from __future__ import annotations

import ctypes
import json
import os
from typing import List, Optional, Sequence

import torch

from . import _lib
from ._lib import HdError, check
from .advection import AdvectionOperation, _stream, _swap_storage

__all__ = ["AdvectionBatch", "load_tile_table", "save_tile_table"]

_DTYPE = {_lib.HD_F64: "f64", _lib.HD_F32: "f32"}


def _ptr_array(tensors: Sequence[torch.Tensor]):
    arr = (ctypes.c_void_p * len(tensors))()
    for i, t in enumerate(tensors):
        arr[i] = t.data_ptr()
    return arr


def _dbl_array(vals: Sequence[float]):
    arr = (ctypes.c_double * len(vals))()
    for i, v in enumerate(vals):
        arr[i] = float(v)
    return arr


class AdvectionBatch:
    """Many independent advection operators advanced together with one LSRK scheme."""

    def __init__(self, ops: Sequence[AdvectionOperation], rk: str = "rk45"):
        if not ops:
            raise HdError(_lib.HD_ERR_INVALID, "AdvectionBatch needs at least one operator")
        self._L = _lib.load()
        self.ops = list(ops)  # the batch keeps pointers to the operators: keep them alive
        h = ctypes.c_void_p()
        check(self._L.hd_lsrk_create(rk.encode(), ctypes.byref(h)))
        self._rk = h
        arr = (ctypes.c_void_p * len(ops))(*[op.handle.value for op in ops])
        b = ctypes.c_void_p()
        check(self._L.hd_batch_create(arr, len(ops), self._rk, ctypes.byref(b)))
        self._h = b

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hd_batch_destroy(self._h)
            self._h = None
        if getattr(self, "_rk", None):
            self._L.hd_lsrk_destroy(self._rk)
            self._rk = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def classes(self) -> List[dict]:
        out = []
        for c in range(int(self._L.hd_batch_n_classes(self._h))):
            v = [ctypes.c_int(0) for _ in range(7)]
            check(self._L.hd_batch_class_info(self._h, c, *[ctypes.byref(x) for x in v]))
            ar = int(self._L.hd_batch_class_arithmetic(self._h, c))
            out.append({"dim": v[0].value, "degree": v[1].value, "dtype": _DTYPE[v[2].value],
                        "arithmetic": "fp32x2" if ar == _lib.HD_ARITH_FP32X2 else "native",
                        "members": v[3].value, "batched": bool(v[4].value), "cells_per_cta": v[5].value,
                        "ctas_per_sm": v[6].value})
        return out

    def set_tile(self, cls: int, cells_per_cta: int = 0, ctas_per_sm: int = 0) -> None:
        check(self._L.hd_batch_set_tile(self._h, int(cls), int(cells_per_cta), int(ctas_per_sm)))

    def apply(self, dst: Sequence[torch.Tensor], src: Sequence[torch.Tensor],
              times: Optional[Sequence[float]] = None) -> None:
        self._check(dst, "dst")
        self._check(src, "src")
        t = _dbl_array(times) if times is not None else None
        check(self._L.hd_batch_apply(self._h, _ptr_array(dst), _ptr_array(src), t, _stream()))

    def perform_time_step(self, sols: Sequence[torch.Tensor], Kis: Sequence[torch.Tensor],
                          Tis: Sequence[torch.Tensor], times: Sequence[float], dts: Sequence[float]) -> None:
        """One fused LSRK step of every instance; each solution tensor holds its new state afterwards
        (storages rotate with the instance's Ki, as in LowStorageRungeKuttaIntegrator)."""
        for vs, name in ((sols, "sol"), (Kis, "Ki"), (Tis, "Ti")):
            self._check(vs, name)
        S, K, T = _ptr_array(sols), _ptr_array(Kis), _ptr_array(Tis)
        orig = [(S[i], K[i]) for i in range(len(sols))]
        check(self._L.hd_batch_lsrk_step(self._h, S, K, T, _dbl_array(times), _dbl_array(dts), _stream()))
        for i in range(len(sols)):
            if S[i] != orig[i][0]:
                assert S[i] == orig[i][1] and K[i] == orig[i][0]
                _swap_storage(sols[i], Kis[i])

    def capture_graph(self, sols, Kis, Tis, times: Sequence[float], dts: Sequence[float]) -> None:
        """Record two steps of every instance as a CUDA graph (replay: ``replay_graph``)."""
        for vs, name in ((sols, "sol"), (Kis, "Ki"), (Tis, "Ti")):
            self._check(vs, name)
        torch.cuda.current_stream().synchronize()
        check(self._L.hd_batch_graph_capture(self._h, _ptr_array(sols), _ptr_array(Kis), _ptr_array(Tis),
                                             _dbl_array(times), _dbl_array(dts)))

    def replay_graph(self) -> None:
        """Advance every instance by two steps (the recorded graph)."""
        check(self._L.hd_batch_graph_launch(self._h, _stream()))

    def autotune(self, src: Sequence[torch.Tensor], dst: Sequence[torch.Tensor], reps: int = 3) -> List[dict]:
        """Time candidate tiles per class (apply launches: src read, dst overwritten); keeps the fastest."""
        self._check(src, "src")
        self._check(dst, "dst")
        check(self._L.hd_batch_autotune(self._h, _ptr_array(src), _ptr_array(dst), int(reps), _stream()))
        return self.classes

    def _check(self, vs, name) -> None:
        if len(vs) != len(self.ops):
            raise HdError(_lib.HD_ERR_INVALID, "%s: one vector per instance" % name)
        for op, v in zip(self.ops, vs):
            op._check_vec(v, name)


def _tile_key(c: dict) -> str:
    # "<dim>-<degree>-<dtype>", dtype "f64x" for FP64 storage in FP32x2 arithmetic
    dt = "f64x" if c.get("arithmetic") == "fp32x2" else c["dtype"]
    return "%d-%d-%s" % (c["dim"], c["degree"], dt)


def save_tile_table(batch: AdvectionBatch, path: str) -> None:
    """Write the batch's per-class tiles ({"<dim>-<degree>-<dtype>": [cells_per_cta, ctas_per_sm]})."""
    table = {}
    if os.path.exists(path):
        table = json.load(open(path))
    for c in batch.classes:
        if c["batched"]:
            table[_tile_key(c)] = [c["cells_per_cta"], c["ctas_per_sm"]]
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


def load_tile_table(batch: AdvectionBatch, path: str) -> int:
    """Apply tiles from a table written by save_tile_table; returns how many classes matched."""
    table = json.load(open(path))
    n = 0
    for i, c in enumerate(batch.classes):
        key = _tile_key(c)
        if c["batched"] and key in table:
            batch.set_tile(i, *table[key])
            n += 1
    return n
