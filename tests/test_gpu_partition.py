"""Partitioned operator on the GPU, through the C ABI.

* All parts of a mesh in one process (LocalPartGroup: pack, exchange on a
  second stream, interior cells, boundary cells) give the single operator's
  apply and fused rk45 steps bit for bit, on the generic kernel (FP64, FP32,
  FP32x2 arithmetic, even and odd dimension, both velocity signs, periodic and
  inhomogeneous Dirichlet in v) and on the TMA-pipelined 3x+3v kernel (whose
  v2 face comes from the ghost region by a bulk copy at the part boundary).
* The face pack writes exactly the sent layer's slabs.
* Two ranks on the one GPU exchange through gloo with host staging
  (DistributedExchange): the parts' kernels never wait on each other -- the
  host moves the faces between launches -- and the result equals the single
  operator's bit for bit.  (NCCL between GPUs is the same code path with
  device buffers; it is not exercised on a one-GPU machine.)
"""
import math
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from hyperdeal_gb300 import _lib  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402
    from hyperdeal_gb300 import partition as Pt  # noqa: E402

CASES = {
    # name: (dim_x, dim_v, cells, velocity, periodic_v, dtype, arithmetic, kernel, boundary function)
    "1x1v_f64": (1, 1, [3, 6], [1.0, 0.5], True, "f64", "native", "generic", False),
    "2x2v_f64_negative": (2, 2, [3, 2, 2, 5], [0.7, -0.4, 0.3, -0.6], True, "f64", "native", "generic", False),
    "2x1v_f64_dirichlet": (2, 1, [2, 3, 6], [0.5, 0.3, 0.8], False, "f64", "native", "generic", True),
    "2x2v_fp32x2": (2, 2, [2, 3, 2, 4], [0.6, 0.5, -0.4, 0.7], True, "f64", "fp32x2", "generic", False),
    "3x2v_f32": (3, 2, [2, 2, 3, 2, 4], [0.6, 0.5, 0.4, 0.3, 0.2], True, "f32", "native", "generic", False),
    "3x3v_f32_generic": (3, 3, [2, 2, 2, 2, 2, 4], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2], True, "f32", "native",
                         "generic", False),
    "3x3v_f32_pipelined": (3, 3, [2, 2, 2, 2, 2, 4], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2], True, "f32", "native",
                           "pipelined", False),
    "3x3v_f32_pipelined_negative": (3, 3, [4, 2, 2, 2, 2, 4], [-1.0, 0.8, -0.6, 0.4, 0.3, -0.2], True, "f32",
                                    "native", "pipelined", False),
}


def case_params(name):
    dx, dv, cells, vel, per_v, dtype, _, _, bfun = CASES[name]
    D = dx + dv
    hi = [1.0 + 0.25 * d for d in range(D)]
    bc = A.Function(2, 0.7, omega=[2 * math.pi / hi[d] for d in range(D)], speed=vel, phase=[0.3] * D,
                    cosine=[d % 2 for d in range(D)]) if bfun else None
    return A.AdvectionParameters(dx, dv, 3, cells[:dx], cells[dx:], [0.0] * dx, hi[:dx], [0.0] * dv, hi[dx:], vel,
                                 periodic_v=per_v, dtype=dtype, boundary=bc)


def _configure(op, name):
    arith, kernel = CASES[name][6], CASES[name][7]
    if arith != "native":
        op.set_arithmetic(arith)
    op.set_kernel(kernel)
    assert op.kernel == kernel


def _single(name):
    op = A.AdvectionOperation(case_params(name))
    _configure(op, name)
    return op


def _group(name, n_parts):
    g = Pt.LocalPartGroup(case_params(name), n_parts)
    for op in g.ops:
        _configure(op, name)
    return g


PARTS = [("1x1v_f64", 2), ("1x1v_f64", 3), ("2x2v_f64_negative", 2), ("2x2v_f64_negative", 5),
         ("2x1v_f64_dirichlet", 3), ("2x2v_fp32x2", 2), ("3x2v_f32", 4), ("3x3v_f32_generic", 2),
         ("3x3v_f32_pipelined", 2), ("3x3v_f32_pipelined", 4), ("3x3v_f32_pipelined_negative", 3)]


@pytest.mark.parametrize("name,n_parts", PARTS)
def test_parts_apply_and_steps_equal_the_single_operator(name, n_parts):
    op = _single(name)
    u = torch.tensor(np.random.default_rng(3).standard_normal(op.n_dofs), dtype=op.dtype, device="cuda")
    ref = op.initialize_dof_vector()
    op.apply(ref, u, 0.3)
    g = _group(name, n_parts)
    assert any(o.ghost_values > 0 for o in g.ops)
    srcs, dsts = g.initialize_dof_vectors(), g.initialize_dof_vectors()
    g.scatter(u, srcs)
    g.apply(dsts, srcs, 0.3)
    assert torch.equal(g.gather(dsts), ref)
    # two fused rk45 steps, the stage inputs' faces exchanged before every stage
    dt = 0.2 * op.critical_time_step() / 3 ** 1.5
    sol = u.clone()
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    it = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    sols = g.initialize_dof_vectors()
    g.scatter(u, sols)
    its = [A.LowStorageRungeKuttaIntegrator(p.initialize_dof_vector(), p.initialize_dof_vector(), "rk45")
           for p in g.ops]
    for s in range(2):
        it.perform_time_step(sol, s * dt, dt, op)
        g.perform_time_step(its, sols, s * dt, dt)
    assert torch.equal(g.gather(sols), sol)
    if CASES[name][7] == "pipelined":
        assert all(p.device_status() == 0 for p in g.ops)


def test_pack_writes_the_sent_layer_slabs():
    g = _group("2x2v_f64_negative", 2)
    op = g.ops[0]
    lay = op.layout
    v = op.initialize_dof_vector()
    op.owned(v).copy_(torch.arange(op.n_dofs, dtype=v.dtype, device="cuda"))
    buf = torch.full((op.send_values(),), -1.0, dtype=v.dtype, device="cuda")
    op.pack(v, buf)
    NC, NF = 256, 64
    cells = op.owned(v).view(-1, NC)[lay["send_first_cell"]:lay["send_first_cell"] + lay["layer_cells"]]
    expect = cells[:, lay["send_slab"] * NF:(lay["send_slab"] + 1) * NF].reshape(-1)
    assert torch.equal(buf, expect)


def test_whole_step_entry_points_refuse_parts_with_ghosts():
    g = _group("1x1v_f64", 2)
    op = g.ops[0]
    L = _lib.load()
    a, b, c = (op.initialize_dof_vector() for _ in range(3))
    X = [A.ctypes.c_void_p(t.data_ptr()) for t in (a, b, c)]
    it = A.LowStorageRungeKuttaIntegrator(b, c, "rk45")
    rc = L.hd_lsrk_step(op.handle, it._h, A.ctypes.byref(X[0]), A.ctypes.byref(X[1]), A.ctypes.byref(X[2]), 0.0,
                        0.01, None)
    assert rc == _lib.HD_ERR_UNSUPPORTED
    with pytest.raises(_lib.HdError):
        from hyperdeal_gb300 import batch as Bt
        Bt.AdvectionBatch([op])


# ---- two ranks on one GPU, exchange through gloo with host staging --------------------------------

def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, name, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from hyperdeal_gb300 import advection as A2
        from hyperdeal_gb300 import partition as P2
        p = case_params(name)
        single = A2.AdvectionOperation(p)
        u = torch.tensor(np.random.default_rng(5).standard_normal(single.n_dofs), dtype=single.dtype, device="cuda")
        dt = 0.2 * single.critical_time_step() / 3 ** 1.5
        ref = single.initialize_dof_vector()
        single.apply(ref, u, 0.1)
        sol_ref = u.clone()
        it_ref = A2.LowStorageRungeKuttaIntegrator(single.initialize_dof_vector(), single.initialize_dof_vector())
        for s in range(2):
            it_ref.perform_time_step(sol_ref, s * dt, dt, single)
        op = P2.PartitionedAdvectionOperation(p, world, rank)
        ex = P2.DistributedExchange(op)
        NC = 4 ** (p.dim_x + p.dim_v)
        a = op.layout["first_cell"] * NC
        src, dst = op.initialize_dof_vector(), op.initialize_dof_vector()
        op.owned(src).copy_(u[a:a + op.n_dofs])
        op.apply(dst, src, 0.1, ex)
        ok_apply = bool(torch.equal(op.owned(dst), ref[a:a + op.n_dofs]))
        sol = op.initialize_dof_vector()
        op.owned(sol).copy_(u[a:a + op.n_dofs])
        it = A2.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector())
        for s in range(2):
            op.perform_time_step(it, sol, s * dt, dt, ex)
        ok_step = bool(torch.equal(op.owned(sol), sol_ref[a:a + op.n_dofs]))
        torch.cuda.synchronize()
        q.put((rank, ok_apply, ok_step))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["2x2v_f64_negative", "3x3v_f32_pipelined"])
def test_two_ranks_exchange_through_gloo_on_one_gpu(name):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, name, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=600) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out == [(0, True, True), (1, True, True)]


def test_part_interpolate_and_norms_add_up_to_the_whole_mesh():
    name = "2x2v_f64_negative"
    op = _single(name)
    f = A.Function(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4, phase=[0.1, 0.2, 0.3, 0.4])
    u = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, u, 0.0)
    n_ref, e_ref = A.VectorTools.norm_and_error(op, f, u, 0.05)
    g = _group(name, 3)
    vecs = g.initialize_dof_vectors()
    n2 = e2 = 0.0
    for p, v in zip(g.ops, vecs):
        p.interpolate(f, v, 0.0)
        a, b = p.norm_and_error_squared(f, v, 0.05)
        n2 += a
        e2 += b
    assert torch.equal(g.gather(vecs), u)
    assert abs(math.sqrt(n2) - n_ref) <= 1e-13 * n_ref
    assert abs(math.sqrt(e2) - e_ref) <= 1e-12 * max(e_ref, 1e-300) + 1e-15 * n_ref
