"""Partitioned operator (v-slabs, one ghost-face exchange per stage) on the CPU.

* The part layout of the C ABI (hd_part_layout_get: host arithmetic only, no
  device) covers the mesh with contiguous cell ranges of whole layers of the
  last direction, pairs every receiver with one sender, and puts the boundary
  layer at the upwind end of each part.
* Two and three gloo ranks run the oracle partitioned with those tables: each
  rank packs the faces its downwind part reads (the slab `send_slab` of the
  layer at `send_first_cell`), exchanges them point-to-point, places its ghost
  faces into the upwind neighbour cells of an otherwise empty global vector and
  applies the oracle; its cells' results equal the unpartitioned oracle's, for
  apply and for rk45 steps with an exchange before every stage.  (The oracle
  restates the reference's flux, which also reads the downwind neighbour and
  multiplies it by zero; the partitioned run leaves that neighbour empty, so
  the results agree to round-off rather than bit for bit.)
"""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from hyperdeal_gb300 import _lib  # noqa: E402
from hyperdeal_gb300.advection import AdvectionParameters  # noqa: E402
from hyperdeal_gb300.partition import part_layout  # noqa: E402

CASES = {
    # name: (dim_x, dim_v, cells, velocity, periodic_v)
    "1x1v": (1, 1, [3, 6], [1.0, 0.5], True),
    "2x2v_negative": (2, 2, [3, 2, 2, 5], [0.7, -0.4, 0.3, -0.6], True),
    "2x1v_dirichlet": (2, 1, [2, 3, 6], [0.5, 0.3, 0.8], False),
    "3x3v": (3, 3, [2, 2, 2, 2, 2, 4], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2], True),
}


def case_params(name, dtype="f64"):
    dx, dv, cells, vel, per_v = CASES[name]
    D = dx + dv
    hi = [1.0 + 0.25 * d for d in range(D)]
    return AdvectionParameters(dx, dv, 3, cells[:dx], cells[dx:], [0.0] * dx, hi[:dx], [0.0] * dv, hi[dx:], vel,
                               periodic_v=per_v, dtype=dtype)


@pytest.mark.parametrize("name", sorted(CASES))
def test_layout_tables_cover_the_mesh(name):
    p = case_params(name)
    D = p.dim_x + p.dim_v
    cells = list(p.cells_x) + list(p.cells_v)
    L = cells[-1]
    n_cells = int(np.prod(cells))
    layer = n_cells // L
    step_up = -1 if p.velocity[-1] > 0 else +1  # the upwind neighbour's layer offset
    for n_parts in range(1, L + 1):
        lays = [part_layout(p, n_parts, k) for k in range(n_parts)]
        first = 0
        for k, lay in enumerate(lays):
            assert lay["first_cell"] == first and lay["n_cells"] % layer == 0 and lay["n_cells"] > 0
            first += lay["n_cells"]
            assert lay["layer_cells"] == layer and lay["face_values"] == 4 ** (D - 1)
            if n_parts == 1:
                assert lay["ghost_values"] == 0 and lay["send_to"] == -1 and lay["recv_from"] == -1
                continue
            up = k + step_up
            if not 0 <= up < n_parts:
                up = up % n_parts if p.periodic_v else -1
            assert lay["recv_from"] == up
            assert lay["ghost_values"] == (layer * lay["face_values"] if up >= 0 else 0)
            assert lay["boundary_cells"] == (layer if up >= 0 else 0)
            if up >= 0:  # the boundary layer sits at the upwind end of the part
                assert lay["boundary_first"] == (0 if step_up < 0 else lay["n_cells"] - layer)
                sender = lays[up]
                assert sender["send_to"] == k
                # the sender's layer is the one adjacent to this part's boundary layer
                sent_first_global = sender["first_cell"] + sender["send_first_cell"]
                bnd_first_global = lay["first_cell"] + lay["boundary_first"]
                assert (sent_first_global - bnd_first_global) % n_cells == (step_up * layer) % n_cells
                assert sender["send_slab"] == (3 if step_up < 0 else 0)
        assert first == n_cells
        assert sum(1 for lay in lays if lay["send_to"] >= 0) == sum(1 for lay in lays if lay["recv_from"] >= 0)


def test_layout_rejects_bad_partitions():
    p = case_params("1x1v")
    for n_parts, part in ((7, 0), (0, 0), (2, 2), (2, -1)):
        with pytest.raises(_lib.HdError) as e:
            part_layout(p, n_parts, part)
        assert e.value.code == _lib.HD_ERR_INVALID
    g = case_params("1x1v")
    g.quadrature = "gauss"
    with pytest.raises(_lib.HdError) as e:
        part_layout(g, 2, 0)
    assert e.value.code == _lib.HD_ERR_UNSUPPORTED


# ---- gloo ranks, oracle --------------------------------------------------------------------------

def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _oracle_problem(p):
    from oracle import oracle as O
    D = p.dim_x + p.dim_v
    return O.Problem(p.dim_x, p.dim_v, p.degree, list(p.cells_x) + list(p.cells_v), list(p.lo_x) + list(p.lo_v),
                     list(p.hi_x) + list(p.hi_v), list(p.velocity)[:D], periodic_x=p.periodic_x,
                     periodic_v=p.periodic_v)


def _rank_main(rank, world, port, name, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    from oracle import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = case_params(name)
        prob = _oracle_problem(p)
        D = p.dim_x + p.dim_v
        NC, NF = 4 ** D, 4 ** (D - 1)
        n_glob = prob.n_dofs // NC
        lay = part_layout(p, world, rank)
        first, n = lay["first_cell"], lay["n_cells"]
        layer = lay["layer_cells"]
        step_up = -1 if p.velocity[D - 1] > 0 else +1
        rng = np.random.default_rng(7)
        u = rng.standard_normal(prob.n_dofs)

        def part_apply(src, dst, t):
            ops = []
            if lay["send_to"] >= 0:
                cells = src.reshape(n, NC)[lay["send_first_cell"]:lay["send_first_cell"] + layer]
                send = torch.from_numpy(np.ascontiguousarray(cells[:, lay["send_slab"] * NF:(lay["send_slab"] + 1) * NF]
                                                             ).reshape(-1))
                ops.append(dist.P2POp(dist.isend, send, lay["send_to"]))
            ghost = torch.zeros(max(lay["ghost_values"], 1), dtype=torch.float64)
            if lay["recv_from"] >= 0:
                ops.append(dist.P2POp(dist.irecv, ghost[:lay["ghost_values"]], lay["recv_from"]))
            for req in (dist.batch_isend_irecv(ops) if ops else []):
                req.wait()
            g = np.zeros(prob.n_dofs)
            g[first * NC:(first + n) * NC] = src
            if lay["recv_from"] >= 0:
                gh = ghost.numpy()
                slab = 3 if step_up < 0 else 0  # the neighbour's face read by the boundary layer
                for i in range(layer):
                    gb = first + lay["boundary_first"] + i
                    nb = (gb + step_up * layer) % n_glob
                    g[nb * NC + slab * NF:nb * NC + (slab + 1) * NF] = gh[i * NF:(i + 1) * NF]
            dst[:] = O.apply(prob, g, t)[first * NC:(first + n) * NC]

        loc = u[first * NC:(first + n) * NC].copy()
        out = np.empty_like(loc)
        part_apply(loc, out, 0.25)
        ref = O.apply(prob, u, 0.25)[first * NC:(first + n) * NC]
        err_apply = float(np.abs(out - ref).max() / np.abs(ref).max())
        sol = loc.copy()
        dt = 0.2 * O.critical_time_step(prob) / 3 ** 1.5
        for s in range(2):
            O.lsrk_step_op("rk45", sol, s * dt, dt, part_apply)
        ref_sol = u.copy()
        for s in range(2):
            O.lsrk_step(prob, "rk45", ref_sol, s * dt, dt)
        ref_sol = ref_sol[first * NC:(first + n) * NC]
        err_step = float(np.abs(sol - ref_sol).max() / np.abs(ref_sol).max())
        q.put((rank, err_apply, err_step, lay["ghost_values"]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("1x1v", 2), ("1x1v", 3), ("2x2v_negative", 2), ("2x1v_dirichlet", 3),
                                        ("3x3v", 2)])
def test_gloo_ranks_partitioned_oracle_equals_unpartitioned(name, world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, name, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == list(range(world))
    assert any(o[3] > 0 for o in out)  # ghost faces were exchanged
    for rank, err_apply, err_step, _ in out:
        assert err_apply < 1e-13, (rank, err_apply)
        assert err_step < 1e-13, (rank, err_step)
