"""The C++ host side: include/hyperdeal_gb300.hpp and the advection application
built on it (hyperdeal_gb300/cpp/advection_hyperrectangle.cc)."""
import json
import os
import re
import subprocess

import pytest

from hyperdeal_gb300 import build as B

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def _rows(text):
    return [tuple(float(v) for v in re.findall(r"[-+]?\d\.\d+e[-+]\d+", line)) for line in text.splitlines()
            if "Time:" in line]


def test_cpp_application_builds_and_reports_usage():
    exe = B.build_cpp_app()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name,args", [
    ("adv_2D_2D_k3.hyperrectangle_05", ["2", "2", "3", "4", "0", "1.0", "rk45"]),
])
def test_cpp_application_reproduces_reference_golden(name, args):
    """The reference's golden time series (ECL + Dirichlet + Gauss-Lobatto collocation) from the C++ host."""
    exe = B.build_cpp_app()
    r = subprocess.run([exe] + args + ["f64"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _rows(r.stdout)
    ref = [c for c in GOLD["advection"] if c["name"] == name][0]["rows"]
    assert len(rows) == len(ref)
    for (t, n, e), (rt, rn, re_) in zip(rows, ref):
        assert abs(t - rt) <= 0.5e-3 * max(abs(rt), 1e-3) + 1e-12
        assert abs(n - rn) <= max(1e-5, 1e-8 * abs(rn)) and abs(n - rn) / rn < 1e-9
        assert abs(e - re_) <= max(1e-5, 1e-8 * abs(re_))
    # FP64 storage with FP32x2 contractions meets the same golden bar and prints the FP64 run's norms
    # (to the printed 11 digits, one unit of the last one)
    rx = subprocess.run([exe] + args + ["f64x"], capture_output=True, text=True, timeout=600)
    assert rx.returncode == 0, rx.stderr
    rows_x = _rows(rx.stdout)
    assert len(rows_x) == len(ref)
    for (t, n, e), (tx, nx, ex), (rt, rn, re_) in zip(rows, rows_x, ref):
        assert abs(nx - rn) <= max(1e-5, 1e-8 * abs(rn)) and abs(ex - re_) <= max(1e-5, 1e-8 * abs(re_))
        assert abs(nx - n) <= 2e-10 * abs(n)
    # the FP32-storage form of the same run stays within 1e-5 of the FP64 norms
    r32 = subprocess.run([exe] + args + ["f32"], capture_output=True, text=True, timeout=600)
    assert r32.returncode == 0, r32.stderr
    for (t, n, e), (t2, n2, e2) in zip(rows, _rows(r32.stdout)):
        assert abs(n2 - n) / n < 1e-5


@pytest.mark.gpu
def test_cpp_application_gauss_golden():
    """A Gauss-quadrature golden (adv_2D_2D_k3.hyperrectangle_01, periodic) from the C++ host."""
    exe = B.build_cpp_app()
    r = subprocess.run([exe, "2", "2", "3", "4", "1", "1.0", "rk45", "f64", "0.1", "0.3", "0.1", "gauss"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _rows(r.stdout)
    ref = [c for c in GOLD["advection"] if c["name"] == "adv_2D_2D_k3.hyperrectangle_01"][0]["rows"]
    assert len(rows) == len(ref)
    for (t, n, e), (rt, rn, re_) in zip(rows, ref):
        assert abs(n - rn) <= max(1e-5, 1e-8 * abs(rn))
        assert abs(e - re_) <= max(1e-5, 1e-8 * abs(re_))


def test_cpp_vp_application_builds_and_reports_usage():
    exe = B.build_cpp_app("vlasov_poisson_hyperrectangle")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_cpp_vp_application_matches_oracle():
    """The Vlasov-Poisson application through the C++ interface against the oracle's run of the same
    case (collocation, 1x1v k=3, 8x8 cells)."""
    from oracle import oracle as O
    exe = B.build_cpp_app("vlasov_poisson_hyperrectangle")
    r = subprocess.run([exe, "1", "3", "8", "8", "0.05", "f64", "0.05", "0.01"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _rows(r.stdout)
    rows_o, _ = O.run_vp_hyperrectangle(1, 1, 3, 8, 8, collocation=True, final_time=0.05, tick=0.01)
    assert len(rows) == len(rows_o) and len(rows) >= 5
    for a, b in zip(rows, rows_o):
        assert abs(a[0] - b[0]) <= 1e-12
        for x, y in zip(a[1:], b[1:]):
            assert abs(x - y) <= 1e-8 * abs(y) + 1e-12


@pytest.mark.gpu
def test_cpp_vp_application_gauss_golden():
    """The reference's Vlasov-Poisson golden vp_2D_2D_k3.hyperrectangle_01 (Gauss quadrature, 2x2v, k = 3,
    4 cells per direction, rk45 to t = 0.5) from the C++ host: every row within numdiff's tolerances."""
    from test_oracle_golden import numdiff_equal
    case = GOLD["vlasov_poisson"][0]
    exe = B.build_cpp_app("vlasov_poisson_hyperrectangle")
    r = subprocess.run([exe, "2", "3", "4", "4", str(case["final_time"]), "f64", str(case["cfl"]), "0.1", "gauss"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _rows(r.stdout)
    assert len(rows) == len(case["rows"])
    for a, g in zip(rows, case["rows"]):
        assert abs(a[0] - g[0]) <= 1e-3
        for x, y in zip(a[1:], g[1:]):
            assert numdiff_equal(x, y), (a[0], x, y)


def test_cpp_partitioned_application_builds_and_reports_usage():
    exe = B.build_cpp_app("partitioned_advection")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("args", [["2", "2", "3", "3", "3", "2", "f64"], ["1", "2", "4", "4", "4", "2", "f64"],
                                  ["3", "3", "3", "2", "2", "1", "f32"], ["2", "1", "2", "5", "5", "2", "f32"]])
def test_cpp_partitioned_parts_equal_the_single_operator(args):
    """PartitionedAdvectionOperation + GhostExchange of include/hyperdeal_gb300.hpp: the parts of one mesh in
    one process (device-copy exchange, stages in lockstep) give the single operator's apply and rk45 steps
    bit for bit (the 3x+3v FP32 case runs the pipelined kernel)."""
    exe = B.build_cpp_app("partitioned_advection")
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("max_diff")][0]
    assert [float(v) for v in line.split()[1:]] == [0.0, 0.0], line
