"""Pins the DoF layout and the face pairing to reference fixtures (no GPU).

* tests/vector_tools/vector_tools_02 (1+1D, k=3, 2..5 refinements of [0,1]) and
  vector_tools_03 (2+2D, k=3, 3 refinements of [-1,1]) print the v-integrated
  x-vector and the x-integrated v-vector in the reference's DoF order.  These
  dumps depend on the node order inside a cell and on the cell order, so
  reproducing them entry by entry pins the layout the oracle (and the GPU
  path, tests/test_gpu_layout.py) uses, not only integrated quantities.
  deal.II numbers the cells of a globally refined cube hierarchically: in 1D
  that is left to right, in 2D the Morton (Z) order of the cell coordinates
  with the first coordinate as the low bit.  This library's meshes are built
  with 0 refinements (lexicographic cells), so the 2D comparison maps the
  lexicographic cells through that permutation.
* tests/matrix_free/fefaceevalutation_02 checks that for f = x_dir the trace
  on every face equals the face-point coordinate, for every (dim_x, dim_v) in
  {1,2,3}^2.  Restated as a property of the operator: with the velocity along
  one direction e only and u = x_dir interpolated, the upwind flux sees no jump
  on a face unless the pairing of the neighbour's face nodes is wrong, so the
  result is 0 for e != dir, and -1 (= -a . grad x_dir) for e == dir except at
  the inflow nodes of the cells whose upwind face is the periodic wrap.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def printed_equal(ours, ref):
    """The reference prints with %.3e and compares with numdiff -a 1e-5 -r 1e-8: equal when our value
    prints the same, or lies within numdiff's absolute tolerance (round-off noise printed as 1e-17)."""
    return ("%.3e" % ours) == ("%.3e" % ref) or abs(ours - ref) <= 1e-5


def morton_order(cells_per_dim: int, dim: int) -> np.ndarray:
    """perm[h] = lexicographic cell index of the h-th cell in deal.II's hierarchical order of a
    globally refined cube (child c has offset bit d = (c >> d) & 1)."""
    bits = int(round(math.log2(cells_per_dim)))
    n = cells_per_dim ** dim
    perm = np.empty(n, dtype=np.int64)
    for h in range(n):
        coord = [0] * dim
        for b in range(bits):
            for d in range(dim):
                coord[d] |= ((h >> (b * dim + d)) & 1) << b
        lex = 0
        for d in reversed(range(dim)):
            lex = lex * cells_per_dim + coord[d]
        perm[h] = lex
    return perm


def hierarchical(vec: np.ndarray, cells_per_dim: int, dim: int, nodes_per_cell: int) -> np.ndarray:
    """Reorder a vector of lexicographic cells into deal.II's hierarchical cell order."""
    cells = vec.reshape(-1, nodes_per_cell)
    return cells[morton_order(cells_per_dim, dim)].reshape(-1)


VT02 = GOLD["vector_tools_02"]


@pytest.mark.parametrize("entry", VT02, ids=["refs%d-%s" % (e["refinements"], e["function"]) for e in VT02])
def test_vector_tools_02_ordered_dumps(entry):
    """vector_tools_02.cc:99-146: interpolate (GL points) then integrate over v / over x."""
    c = 2 ** entry["refinements"]
    prob = O.Problem(1, 1, 3, [c, c], [0.0, 0.0], [1.0, 1.0], [1.0, 1.0])
    if entry["function"] == "zero":
        f = O.make_func(0)
    elif entry["function"] == "one":
        f = O.make_func(1, 1.0)
    else:  # tests_functions.h:22-38: sin(pi x) cos(pi v)
        f = O.make_func(2, 1.0, omega=[math.pi, math.pi], speed=[0.0, 0.0], cosine=[0, 1])
    u = O.interpolate(prob, f)
    vec_x = O.velocity_moment(prob, u)
    vec_v = O.coordinate_moment(prob, u)
    assert len(vec_x) == len(entry["vec_x"]) and len(vec_v) == len(entry["vec_v"])
    for ours, ref in zip(vec_x, entry["vec_x"]):
        assert printed_equal(ours, ref), (ours, ref)
    for ours, ref in zip(vec_v, entry["vec_v"]):
        assert printed_equal(ours, ref), (ours, ref)


def vt03_problem():
    g = GOLD["vector_tools_03"]
    c = 2 ** g["refinements"]
    return O.Problem(2, 2, 3, [c] * 4, [g["lo"]] * 4, [g["hi"]] * 4, [1.0] * 4), c


def vt03_values(prob):
    """tests_functions.h:41-55: max(0, 0.5 - |p|) at the support points."""
    x = O.node_coordinates(prob)
    return np.maximum(0.0, 0.5 - np.sqrt((x * x).sum(axis=1)))


def test_vector_tools_03_ordered_dumps():
    """vector_tools_03.cc:80-134 (2+2D): the cell order is hierarchical, the nodes lexicographic."""
    g = GOLD["vector_tools_03"]
    prob, c = vt03_problem()
    u = vt03_values(prob)
    vec_x = hierarchical(O.velocity_moment(prob, u), c, 2, 16)
    vec_v = hierarchical(O.coordinate_moment(prob, u), c, 2, 16)
    nonzero = 0
    for ours, ref in zip(vec_x, g["vec_x"]):
        assert printed_equal(ours, ref), (ours, ref)
        nonzero += ref != 0.0
    for ours, ref in zip(vec_v, g["vec_v"]):
        assert printed_equal(ours, ref), (ours, ref)
    assert nonzero > 100  # the dump is not trivially zero
    # a wrong node order inside the cell is detected: transpose the 4x4 nodes of every cell
    wrong = O.velocity_moment(prob, u).reshape(-1, 4, 4).transpose(0, 2, 1).reshape(-1)
    wrong = hierarchical(wrong, c, 2, 16)
    assert not all(printed_equal(a, b) for a, b in zip(wrong, g["vec_x"]))


# ---- the face-trace property of tests/matrix_free/fefaceevalutation_02 ----------------------------

SPLITS = [(dx, dv) for dx in (1, 2, 3) for dv in (1, 2, 3)]


def face_property_cells(dim_x, dim_v):
    D = dim_x + dim_v
    return [3 if D <= 4 else 2] * D


def linear_coordinate(prob, direction):
    return np.ascontiguousarray(O.node_coordinates(prob)[:, direction])


def face_property_expected(prob, direction, e, result, collocation=True):
    """Checks the operator result for u = x_dir and velocity e_e; returns the worst deviation."""
    D = prob.dim
    n = prob.degree + 1
    cells = [int(c) for c in prob.cells]
    r = result.reshape(-1, n ** D)
    if e != direction:
        return float(np.abs(r).max())
    # cell coordinate c_e and node digit i_e of every entry
    gid = np.arange(r.shape[0])
    ce = (gid // int(np.prod(cells[:e]))) % cells[e]
    node = np.arange(n ** D)
    ie = (node // n ** e) % n
    wrap_cell = ce == 0  # velocity +1: the upwind face of the first cell is the periodic wrap
    mask = np.ones_like(r, dtype=bool)
    if collocation:
        mask[np.ix_(wrap_cell, ie == 0)] = False
    else:
        mask[wrap_cell, :] = False
    return float(np.abs(r[mask] + 1.0).max())


def test_face_trace_golden_covers_every_split():
    rows = GOLD["fefaceevalutation_02"]["rows"]
    assert all(r[5] for r in rows)
    assert sorted({(r[0], r[1]) for r in rows}) == SPLITS


@pytest.mark.parametrize("dim_x,dim_v", SPLITS)
@pytest.mark.parametrize("collocation", [True, False], ids=["collocation", "gauss"])
def test_face_trace_property_oracle(dim_x, dim_v, collocation):
    D = dim_x + dim_v
    cells = face_property_cells(dim_x, dim_v)
    worst = 0.0
    for direction in range(D):
        for e in range(D):
            vel = [0.0] * D
            vel[e] = 1.0
            prob = O.Problem(dim_x, dim_v, 3, cells, [0.0] * D, [1.0 + 0.5 * d for d in range(D)], vel,
                             collocation=collocation)
            u = linear_coordinate(prob, direction)
            worst = max(worst, face_property_expected(prob, direction, e, O.apply(prob, u), collocation))
    assert worst < 1e-11, worst


def test_face_trace_property_is_sensitive_to_the_pairing():
    """For a tangential direction the trace of x_dir varies across the face, so a neighbour trace read
    with its tangential nodes permuted (e.g. deal.II's zx swap applied where it does not belong) would
    differ from the own trace: the zero-jump property above then fails."""
    prob = O.Problem(2, 1, 3, [3, 3, 3], [0.0] * 3, [1.0, 1.5, 2.0], [0.0, 0.0, 1.0])
    u = linear_coordinate(prob, 0).reshape(-1, 4, 4, 4)  # [cell][i2][i1][i0]
    face = u[:, 3, :, :]  # the x2 face slab i2 = N-1 of every cell
    assert np.abs(face - face.transpose(0, 2, 1)).max() > 0.1
