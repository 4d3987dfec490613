"""The bounds-checked build (-DHD_CHECK) compiles (no GPU): the pipelined kernel
and one generated generic-kernel unit, compiled for sm_103a with the checks on.
tests/test_gpu_check_build.py runs the checked library on the GPU."""
import os
import subprocess
import tempfile

import pytest

from hyperdeal_gb300 import build as B


@pytest.mark.parametrize("unit", ["hd_ecl6.cu", "gen:ecl_4_4"])
def test_checked_units_compile(unit):
    nvcc = B.nvcc()
    if not os.path.exists(nvcc) and subprocess.run(["which", nvcc], capture_output=True).returncode != 0:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as tmp:
        if unit.startswith("gen:"):
            src = os.path.join(tmp, "u.cu")
            with open(src, "w") as f:
                f.write('#include "hd_ecl.cuh"\nnamespace hd {\nEclLaunchers ecl_launchers_4_4() '
                        '{ return make_launchers<4, 4>(); }\n}\n')
        else:
            src = os.path.join(B.CSRC, unit)
        cmd = [nvcc] + B.ARCH + B.NVCC_FLAGS + ["-I", B.CSRC, "-DHD_CHECK", "-c", src, "-o", os.path.join(tmp, "u.o")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
