"""GPU tests of the reference-style drivers over the model files: the Python
command line (``python -m vulkanfem_gb300``, src/main.cpp:28-127) and the C++
driver tests/inout_example.cpp over include/vfem_inout.hpp.  Both must write the
same solution as the library's API, and that solution must agree with the oracle
to the solve tolerance."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from tests.conftest import ROOT
from tests.test_inout import compile_example
from vulkanfem_gb300 import api, domains, inout
from vulkanfem_gb300 import build as vbuild

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    d = domains.cantilever(16, 8, 8)
    ke = domains.hex8_stiffness()
    tmp = tmp_path_factory.mktemp("model")
    inout.save_domain(d, str(tmp / "cant"), ke=ke)
    A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3, 0)
    f = d.load_vector()
    u_api, st = A.solve(f, precision="fp64")
    A.close()
    o = oracle.Oracle(d.voxels, ke, d.fixed, 3, 0)
    u_or, _, _ = o.pcg(f, 1e-6)
    return {"dir": tmp, "d": d, "f": f, "u_api": u_api, "u_oracle": u_or, "iters": st["iterations"]}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_python_driver_writes_the_api_solution(model):
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "vulkanfem_gb300", "cant.dat", "-n", "3", "--precision", "fp64"],
                       cwd=str(model["dir"]), env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Degrees of freedom: %d" % model["f"].size in r.stdout
    u = inout.loadVector(str(model["dir"] / "cant"))
    assert np.array_equal(u, model["u_api"])  # 17 digits: loss-free
    assert _rel(u, model["u_oracle"]) < 1e-5
    comp = float(r.stdout.split("Compliance:")[1].split()[0])
    assert comp == pytest.approx(float(model["f"] @ model["u_oracle"]), rel=1e-6)


def test_cpp_driver_writes_the_api_solution(model, tmp_path):
    api.load_library()
    exe = compile_example(tmp_path, vbuild.LIB)
    r = subprocess.run([exe, "cant.dat", "-n", "3"], cwd=str(model["dir"]), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Iterations: %d" % model["iters"] in r.stdout
    u = inout.loadVector(str(model["dir"] / "cant"))
    assert np.array_equal(u, model["u_api"])
    assert _rel(u, model["u_oracle"]) < 1e-5
