"""Partitioned advection: v-slabs with one ghost-face exchange per Runge-Kutta stage.

The reference distributes the phase space over an x-by-v process grid and
exchanges ghost faces through its Contiguous partitioner
(include/hyper.deal/matrix_free/vector_partitioner.h:670-1381 set-up,
:1385-1607 update_ghost_values), overlapping the exchange with the cells that
do not need it (matrix_free.templates.h:1178-1234, :1494-1581).  Here the mesh
is cut into slabs of whole layers of the last v-direction (a v-only process
grid, so every part owns a contiguous range of cell ids) and only the upwind
face of the cut direction is exchanged: one layer of face traces per stage
from the upwind part into the ghost region that follows the part's cells in
each of its vectors (include/hyperdeal_gb300.h, hd_part_layout).

Per stage (and per apply) a part

1. packs the faces its downwind part reads from the stage input
   (``hd_adv_pack_faces``),
2. starts the exchange (the transport is the host's: a device copy between
   parts in one process, NCCL point-to-point between ranks),
3. runs the stage on its INTERIOR cells while the faces are in flight,
4. waits for its own ghost faces and runs the stage on its BOUNDARY layer.

``LocalPartGroup`` runs all parts of a mesh in one process (one GPU), in
lockstep, with the exchange on a second stream; ``DistributedExchange`` moves
the faces between ranks with ``torch.distributed`` (one part per rank).
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import torch

from . import _lib
from ._lib import HdError, check
from .advection import AdvectionParameters, LowStorageRungeKuttaIntegrator, _swap_storage

__all__ = ["part_layout", "PartitionedAdvectionOperation", "LocalPartGroup", "DistributedExchange"]


def part_layout(params: AdvectionParameters, n_parts: int, part: int) -> dict:
    """Layout of part `part` of `n_parts` (hd_part_layout_get: host arithmetic only, no device)."""
    L = _lib.load()
    desc = params.c()
    out = _lib.hd_part_layout()
    check(L.hd_part_layout_get(ctypes.byref(desc), int(n_parts), int(part), ctypes.byref(out)))
    return out.as_dict()


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream(s: Optional[torch.cuda.Stream] = None) -> ctypes.c_void_p:
    return ctypes.c_void_p((s or torch.cuda.current_stream()).cuda_stream)


class PartitionedAdvectionOperation:
    """The advection operator of one part (hd_adv_create_part).

    Its vectors hold the part's cells (``n_dofs`` values, numbered as the global vector
    restricted to the part's cell range) followed by ``ghost_values`` ghost values."""

    def __init__(self, params: AdvectionParameters, n_parts: int, part: int):
        self.params = params
        self.n_parts = int(n_parts)
        self.part = int(part)
        self._L = _lib.load()
        h = ctypes.c_void_p()
        desc = params.c()
        check(self._L.hd_adv_create_part(ctypes.byref(desc), self.n_parts, self.part, ctypes.byref(h)))
        self._h = h
        lay = _lib.hd_part_layout()
        check(self._L.hd_adv_part_layout(h, ctypes.byref(lay)))
        self.layout = lay.as_dict()
        self.n_dofs = int(self._L.hd_adv_n_dofs(h))
        self.ghost_values = int(self.layout["ghost_values"])
        self.dtype = torch.float64 if params.dtype == "f64" else torch.float32

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hd_adv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @property
    def kernel(self) -> str:
        return {_lib.HD_KERNEL_GENERIC: "generic", _lib.HD_KERNEL_PIPELINED: "pipelined"}[
            int(self._L.hd_adv_kernel(self._h))]

    def set_kernel(self, variant: str) -> None:
        v = {"auto": _lib.HD_KERNEL_AUTO, "generic": _lib.HD_KERNEL_GENERIC,
             "pipelined": _lib.HD_KERNEL_PIPELINED}[variant]
        check(self._L.hd_adv_set_kernel(self._h, v))

    def set_arithmetic(self, arithmetic: str) -> None:
        v = {"native": _lib.HD_ARITH_NATIVE, "fp32x2": _lib.HD_ARITH_FP32X2}[arithmetic]
        check(self._L.hd_adv_set_arithmetic(self._h, v))

    def critical_time_step(self) -> float:
        return float(self._L.hd_adv_critical_time_step(self._h))

    def device_status(self) -> int:
        st = ctypes.c_int(0)
        check(self._L.hd_adv_device_status(self._h, ctypes.byref(st)))
        return int(st.value)

    def initialize_dof_vector(self) -> torch.Tensor:
        return torch.zeros(self.n_dofs + self.ghost_values, dtype=self.dtype, device="cuda")

    def owned(self, v: torch.Tensor) -> torch.Tensor:
        return v[:self.n_dofs]

    def ghost(self, v: torch.Tensor) -> torch.Tensor:
        return v[self.n_dofs:]

    def send_values(self) -> int:
        """Values this part sends per exchange (the receiver's ghost region)."""
        return int(self.layout["layer_cells"] * self.layout["face_values"]) if self.layout["send_to"] >= 0 else 0

    def _check_vec(self, v: torch.Tensor, name: str) -> None:
        if not isinstance(v, torch.Tensor) or not v.is_cuda or v.dtype != self.dtype or not v.is_contiguous() \
                or v.numel() != self.n_dofs + self.ghost_values:
            raise HdError(_lib.HD_ERR_INVALID, "%s must be a contiguous CUDA %s vector of %d entries (cells + ghost "
                          "region)" % (name, self.dtype, self.n_dofs + self.ghost_values))

    def interpolate(self, f, dst: torch.Tensor, time: float = 0.0) -> None:
        """f at the support points of this part's cells (hd_interpolate; the ghost region is untouched)."""
        self._check_vec(dst, "dst")
        fc = f.c()
        check(self._L.hd_interpolate(self._h, ctypes.byref(fc), float(time), _ptr(dst), _stream()))

    def norm_and_error_squared(self, f, src: torch.Tensor, time: float = 0.0):
        """Squared L2 norm and error over this part's cells: the parts' values add up to the squares
        of the whole mesh's (hd_norm_and_error on the part)."""
        self._check_vec(src, "src")
        fc = f.c()
        out = (ctypes.c_double * 2)()
        check(self._L.hd_norm_and_error(self._h, ctypes.byref(fc), float(time), _ptr(src), out, _stream()))
        return float(out[0]) ** 2, float(out[1]) ** 2

    def pack(self, vec: torch.Tensor, sendbuf: torch.Tensor, stream=None) -> None:
        check(self._L.hd_adv_pack_faces(self._h, _ptr(vec), _ptr(sendbuf), _stream(stream)))

    def apply_cells(self, dst: torch.Tensor, src: torch.Tensor, time: float, cells: int) -> None:
        self._check_vec(dst, "dst")
        self._check_vec(src, "src")
        check(self._L.hd_adv_apply_cells(self._h, _ptr(dst), _ptr(src), float(time), int(cells), _stream()))

    def stage(self, integrator: LowStorageRungeKuttaIntegrator, stage: int, X: Sequence[torch.Tensor],
              time: float, dt: float, cells: int) -> None:
        arr = (ctypes.c_void_p * 3)(*[x.data_ptr() for x in X])
        check(self._L.hd_lsrk_stage(self._h, integrator._h, int(stage), arr, float(time), float(dt), int(cells),
                                    _stream()))

    @staticmethod
    def stage_input(integrator: LowStorageRungeKuttaIntegrator, stage: int) -> int:
        return int(_lib.load().hd_lsrk_stage_input(integrator._h, int(stage)))

    # one part per rank: apply and time step with an exchange object (DistributedExchange)
    def apply(self, dst: torch.Tensor, src: torch.Tensor, time: float, exchange: "DistributedExchange") -> None:
        self._check_vec(dst, "dst")
        self._check_vec(src, "src")
        pending = exchange.start(self, src)
        self.apply_cells(dst, src, time, _lib.HD_CELLS_INTERIOR)
        exchange.finish(pending)
        self.apply_cells(dst, src, time, _lib.HD_CELLS_BOUNDARY)

    def perform_time_step(self, integrator: LowStorageRungeKuttaIntegrator, solution: torch.Tensor,
                          current_time: float, time_step: float, exchange: "DistributedExchange") -> None:
        """One fused LSRK step; the stage input's faces are exchanged before each stage, the interior
        cells overlap the exchange.  On return `solution` holds the new state (storages swapped as in
        LowStorageRungeKuttaIntegrator)."""
        X = [solution, integrator.vec_Ki, integrator.vec_Ti]
        for v, n in zip(X, ("solution", "vec_Ki", "vec_Ti")):
            self._check_vec(v, n)
        for s in range(integrator.n_stages()):
            vin = X[self.stage_input(integrator, s)]
            pending = exchange.start(self, vin)
            self.stage(integrator, s, X, current_time, time_step, _lib.HD_CELLS_INTERIOR)
            exchange.finish(pending)
            self.stage(integrator, s, X, current_time, time_step, _lib.HD_CELLS_BOUNDARY)
        _swap_storage(solution, integrator.vec_Ki)  # the new solution was accumulated in X1 = vec_Ki


class DistributedExchange:
    """Ghost-face transport between ranks (one part per rank) with torch.distributed point-to-point:
    the part packs its sent layer into a buffer, sends it to its downwind part and receives its own
    ghost region from its upwind part, in one batch (no ordering deadlock on a periodic ring).
    With the NCCL backend the transfer runs on NCCL's stream after the pack, the interior cells run
    meanwhile on the current stream, and finish() makes the current stream wait for the receive.
    A backend without device tensors (gloo) stages the faces through pinned host buffers: the send
    waits for the pack on the host, and finish() copies the received faces into the ghost region."""

    def __init__(self, op: PartitionedAdvectionOperation, group=None, rank_of_part=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank_of_part = rank_of_part or (lambda p: p)
        n = op.send_values()
        self.sendbuf = torch.empty(max(n, 1), dtype=op.dtype, device="cuda")
        self.host = dist.get_backend(group) == "gloo"
        if self.host:
            self.h_send = torch.empty(max(n, 1), dtype=op.dtype, pin_memory=True)
            self.h_recv = torch.empty(max(op.ghost_values, 1), dtype=op.dtype, pin_memory=True)

    def start(self, op: PartitionedAdvectionOperation, vec: torch.Tensor):
        lay = op.layout
        ops = []
        if lay["send_to"] >= 0:
            op.pack(vec, self.sendbuf)
            buf = self.sendbuf[:op.send_values()]
            if self.host:
                self.h_send[:op.send_values()].copy_(buf)  # synchronous: the pack is complete
                buf = self.h_send[:op.send_values()]
            ops.append(self.dist.P2POp(self.dist.isend, buf, self.rank_of_part(lay["send_to"]), self.group))
        if lay["recv_from"] >= 0:
            dst = self.h_recv[:op.ghost_values] if self.host else op.ghost(vec)
            ops.append(self.dist.P2POp(self.dist.irecv, dst, self.rank_of_part(lay["recv_from"]), self.group))
        reqs = self.dist.batch_isend_irecv(ops) if ops else []
        return (reqs, op, vec)

    def finish(self, pending) -> None:
        reqs, op, vec = pending
        for req in reqs:
            req.wait()
        if self.host and op.layout["recv_from"] >= 0:
            op.ghost(vec).copy_(self.h_recv[:op.ghost_values], non_blocking=True)


class LocalPartGroup:
    """All parts of a partitioned mesh in one process on one GPU.  Each stage runs, for every part,
    the launches one rank per part would run (pack, exchange, interior cells, boundary cells); the
    exchange is a device copy from the sender's buffer into the receiver's ghost region on a second
    stream, so it overlaps the interior cells."""

    def __init__(self, params: AdvectionParameters, n_parts: int):
        self.params = params
        self.ops: List[PartitionedAdvectionOperation] = [PartitionedAdvectionOperation(params, n_parts, p)
                                                         for p in range(n_parts)]
        self.sendbufs = [torch.empty(max(op.send_values(), 1), dtype=op.dtype, device="cuda") for op in self.ops]
        self.comm = torch.cuda.Stream()

    def initialize_dof_vectors(self) -> List[torch.Tensor]:
        return [op.initialize_dof_vector() for op in self.ops]

    def scatter(self, global_vec: torch.Tensor, vecs: List[torch.Tensor]) -> None:
        """Copy each part's cells out of a vector of the whole mesh (ghost regions untouched)."""
        NC = (self.params.degree + 1) ** (self.params.dim_x + self.params.dim_v)
        for op, v in zip(self.ops, vecs):
            a = op.layout["first_cell"] * NC
            op.owned(v).copy_(global_vec[a:a + op.n_dofs])

    def gather(self, vecs: List[torch.Tensor]) -> torch.Tensor:
        return torch.cat([op.owned(v) for op, v in zip(self.ops, vecs)])

    def _exchange_start(self, vecs: List[torch.Tensor]) -> torch.cuda.Event:
        """Pack every part's faces and copy them into their receivers' ghost regions on the comm stream
        (after the work already queued on the current stream)."""
        self.comm.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.comm):
            for op, v, buf in zip(self.ops, vecs, self.sendbufs):
                if op.layout["send_to"] >= 0:
                    op.pack(v, buf, self.comm)
            for op, v in zip(self.ops, vecs):
                src = op.layout["recv_from"]
                if src >= 0:
                    op.ghost(v).copy_(self.sendbufs[src][:self.ops[src].send_values()], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.comm)
        return done

    def exchange(self, vecs: List[torch.Tensor]) -> None:
        torch.cuda.current_stream().wait_event(self._exchange_start(vecs))

    def apply(self, dsts: List[torch.Tensor], srcs: List[torch.Tensor], time: float = 0.0) -> None:
        done = self._exchange_start(srcs)
        for op, d, s in zip(self.ops, dsts, srcs):
            op.apply_cells(d, s, time, _lib.HD_CELLS_INTERIOR)
        torch.cuda.current_stream().wait_event(done)
        for op, d, s in zip(self.ops, dsts, srcs):
            op.apply_cells(d, s, time, _lib.HD_CELLS_BOUNDARY)

    def perform_time_step(self, integrators: List[LowStorageRungeKuttaIntegrator], sols: List[torch.Tensor],
                          current_time: float, time_step: float) -> None:
        Xs = [[s, it.vec_Ki, it.vec_Ti] for s, it in zip(sols, integrators)]
        ns = integrators[0].n_stages()
        for st in range(ns):
            k = PartitionedAdvectionOperation.stage_input(integrators[0], st)
            done = self._exchange_start([X[k] for X in Xs])
            for op, it, X in zip(self.ops, integrators, Xs):
                op.stage(it, st, X, current_time, time_step, _lib.HD_CELLS_INTERIOR)
            torch.cuda.current_stream().wait_event(done)
            for op, it, X in zip(self.ops, integrators, Xs):
                op.stage(it, st, X, current_time, time_step, _lib.HD_CELLS_BOUNDARY)
        for s, it in zip(sols, integrators):
            _swap_storage(s, it.vec_Ki)
