"""Extracts the reference's golden outputs for the advection path into
``reference_goldens.json`` (run once in a checkout that has the reference tree).

Usage:  python tests/golden/make_goldens.py /path/to/hyperdeal

Sources (paths relative to the reference root):
  examples/vlasov_poisson/tests/*.configuration, *.json, *.out
      -- Vlasov-Poisson diagnostics (field energy, mass, L2, kinetic energy, momentum)
  examples/advection/tests/*.configuration, *.json, *.out
      -- application time series "Time, norm, error" (compared by numdiff
         -a 1e-5 -r 1e-8, cmake/macros/macro_hyper_deal_pickup_tests.cmake:57)
  tests/time_discretization/time_integrators_01.output  -- stage counts
  tests/time_discretization/time_integrators_02.mpirun=1.output -- rk45 KAT
  tests/vector_tools/vector_tools_01.mpirun=1.output   -- interpolate + L2
  tests/vector_tools/vector_tools_02.mpirun=1.output   -- ordered dumps of the
      v-integrated x-vector and the x-integrated v-vector, 1+1D k=3, 2..5
      refinements of [0,1], functions 0, 1, sin(pi x) cos(pi v)
  tests/vector_tools/vector_tools_03.mpirun=1.output   -- the same for 2+2D k=3,
      3 refinements of [-1,1], max(0, 0.5 - |p|)
  tests/matrix_free/fefaceevalutation_02.mpirun=1.output -- the face-trace
      property (trace of f = x_dir equals the face-point coordinate) and the
      (dim_x, dim_v, dir, loop, face) combinations it passed for
The fixture holds numbers and run parameters only.
"""
import glob
import json
import os
import re
import sys

NUM = r"[-+]?\d+\.?\d*(?:e[-+]?\d+)?"


def parse_configuration(path):
    out = {}
    for tok in open(path).read().split():
        k, v = tok.split("=")
        out[k] = int(v)
    return out


def main(root):
    here = os.path.dirname(os.path.abspath(__file__))
    adv_dir = os.path.join(root, "examples", "advection", "tests")
    advection = []
    for jpath in sorted(glob.glob(os.path.join(adv_dir, "*.json"))):
        name = os.path.basename(jpath)[:-5]
        prefix = name.split(".")[0]
        conf = parse_configuration(os.path.join(adv_dir, prefix + ".configuration"))
        prm = json.load(open(jpath))
        rows = []
        for line in open(os.path.join(adv_dir, name + ".out")):
            vals = re.findall(r"[-+]?\d\.\d+e[-+]\d+", line)
            if vals:
                rows.append([float(v) for v in vals])
        case = prm["Case"]
        sub_x = [int(v) for v in case["NSubdivisionsX"].values()]
        sub_v = [int(v) for v in case["NSubdivisionsV"].values()]
        td = prm["TemporalDiscretization"]
        advection.append({
            "name": name,
            "dim_x": conf["DIM_X"], "dim_v": conf["DIM_V"],
            "degree": conf["DEGREE"], "n_points": conf["N_POINTS"],
            "subdivisions": sub_x[:conf["DIM_X"]] + sub_v[:conf["DIM_V"]],
            "periodic_x": case["PeriodicX"] == "true",
            "periodic_v": case["PeriodicV"] == "true",
            "collocation": prm["SpatialDiscretization"]["DoCollocation"] == "true",
            "use_ecl": prm["Matrixfree"]["UseECL"] == "true",
            "skew": float(prm["AdvectionOperation"]["SkewFactor"]),
            "rk": td["RKType"],
            "time_step": float(td["TimeStep"]),
            "start_time": float(td["StartTime"]),
            "final_time": float(td["FinalTime"]),
            "cfl": float(td["CFLNumber"]),
            "tick": float(td["DiagnosticsTick"]),
            "rows": rows,
        })
    ti01 = [int(v) for v in re.findall(r"DEAL::(\d+)", open(
        os.path.join(root, "tests", "time_discretization", "time_integrators_01.output")).read())]
    ti02 = [float(v) for v in re.findall(r"= (" + NUM + ")", open(
        os.path.join(root, "tests", "time_discretization", "time_integrators_02.mpirun=1.output")).read())]
    vt01 = []
    for line in open(os.path.join(root, "tests", "vector_tools", "vector_tools_01.mpirun=1.output")):
        vals = re.findall(NUM, line.split("::", 1)[1]) if "::" in line else []
        if len(vals) == 2:
            vt01.append([float(v) for v in vals])
    # ordered vector dumps ("Vector data:" followed by one line of values)
    def vector_dumps(path):
        lines = open(path).read().splitlines()
        out = []
        for i, line in enumerate(lines):
            if line.strip() == "Vector data:":
                out.append([float(v) for v in lines[i + 1].split()])
        return out

    vt02_all = vector_dumps(os.path.join(root, "tests", "vector_tools", "vector_tools_02.mpirun=1.output"))
    # vector_tools_02.cc:99-129, :139-146: for refs 2..5, for f in (0, 1, sin(pi x) cos(pi v)): vec_x, vec_v
    vt02 = []
    k = 0
    for refs in range(2, 6):
        for fname in ("zero", "one", "sin_cos"):
            vt02.append({"refinements": refs, "function": fname, "vec_x": vt02_all[k], "vec_v": vt02_all[k + 1]})
            k += 2
    assert k == len(vt02_all)
    vt03_all = vector_dumps(os.path.join(root, "tests", "vector_tools", "vector_tools_03.mpirun=1.output"))
    assert len(vt03_all) == 2
    vt03 = {"dim_x": 2, "dim_v": 2, "degree": 3, "refinements": 3, "lo": -1.0, "hi": 1.0,
            "function": "max(0, 0.5 - |p|)", "vec_x": vt03_all[0], "vec_v": vt03_all[1]}
    ff02 = []
    for line in open(os.path.join(root, "tests", "matrix_free", "fefaceevalutation_02.mpirun=1.output")):
        m = re.match(r"DEAL:0:dim_x=(\d):(\d):dir=(\d):(FCL|ECL):dir=(\d+)::(.*)$", line.strip())
        if m:
            ff02.append([int(m.group(1)), int(m.group(2)), int(m.group(3)), m.group(4), int(m.group(5)),
                         "succeeded" in m.group(6)])

    vp = []
    vp_dir = os.path.join(root, "examples", "vlasov_poisson", "tests")
    for jpath in sorted(glob.glob(os.path.join(vp_dir, "*.json"))):
        name = os.path.basename(jpath)[:-5]
        conf = parse_configuration(os.path.join(vp_dir, name.split(".")[0] + ".configuration"))
        prm = json.load(open(jpath))
        rows = [[float(v) for v in line.split()] for line in open(os.path.join(vp_dir, name + ".out"))
                if line.strip() and not line.startswith("#")]
        td = prm["TemporalDiscretization"]
        case = prm["Case"]
        vp.append({
            "name": name, "dim_x": conf["DIM_X"], "dim_v": conf["DIM_V"], "degree": conf["DEGREE"],
            "n_points": conf["N_POINTS"],
            "cells_x": 2 ** int(case["NRefinementsX"]) * int(case["NSubdivisionsX"]["X"]),
            "cells_v": 2 ** int(case["NRefinementsV"]) * int(case["NSubdivisionsV"]["X"]),
            "collocation": prm["SpatialDiscretization"]["DoCollocation"] == "true",
            "final_time": float(td["FinalTime"]), "time_step": float(td["TimeStep"]), "cfl": float(td["CFLNumber"]),
            "columns": "time, field energy per x-direction, mass, L2 norm, kinetic energy, momentum (3)",
            "rows": rows,
        })
    out = {
        "numdiff": {"abs": 1e-5, "rel": 1e-8},
        "vlasov_poisson": vp,
        "advection": advection,
        "time_integrators_01_stages": ti01,
        "time_integrators_02_rk45_values": ti02,
        "vector_tools_01_rows": vt01,
        "vector_tools_02": vt02,
        "vector_tools_03": vt03,
        "fefaceevalutation_02": {"columns": "dim_x, dim_v, dir (of f = x_dir), loop, face, succeeded",
                                 "rows": ff02},
    }
    with open(os.path.join(here, "reference_goldens.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(advection), "advection cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_goldens.py <root of the hyper.deal tree>")
    main(sys.argv[1])
