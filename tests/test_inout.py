"""CPU tests of the reference-format model files (vulkanfem_gb300/inout.py and
the C++ shim include/vfem_inout.hpp), following src/inout.cpp:6-128,206-225."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT
from vulkanfem_gb300 import domains, inout


def _write_armadillo(armadillo, d):
    name = os.path.join(str(d), "armadillo_128")
    inout.writeVoxel(name, armadillo["voxels"])
    inout.writeBoundaryConditions(name, armadillo["fixed"], (armadillo["load_nodes"], armadillo["load_values"]))
    inout.writeKe(name, armadillo["ke0"])
    return name


def test_armadillo_round_trip_and_layout(armadillo, tmp_path):
    name = _write_armadillo(armadillo, tmp_path)
    with open(name + ".dat") as fh:
        assert fh.readline() == "112 128 128\n"  # sx sy sz (inout.cpp:15-21)
        first = fh.readline()
    assert first.count(",") == 112 * 128 - 1
    model, dims = inout.loadVoxel(name)
    assert dims == (112, 128, 128) and model.shape == (128, 128, 112)
    assert np.array_equal(inout.occupancy(model), armadillo["voxels"])
    fixed, loads = inout.getBoundaryConditions(name)
    # the reference's file lists 2,535 ids of which 1,750 are distinct (a std::set keeps those)
    assert armadillo["fixed"].size == 2535
    assert fixed.size == 1750 and np.array_equal(fixed, np.unique(armadillo["fixed"]))
    nodes, vals = inout.loads_as_arrays(loads)
    order = np.argsort(armadillo["load_nodes"])
    assert nodes.size == 1331
    assert np.array_equal(nodes, armadillo["load_nodes"][order])
    assert np.array_equal(vals, armadillo["load_values"][order])
    assert np.array_equal(inout.getKe(name), armadillo["ke0"])
    d = inout.load_domain(name)
    assert d.num_dofs == 562455  # the reference's armadillo DOF count
    assert np.array_equal(d.meta["Ke"], armadillo["ke0"])


def test_set_and_map_semantics(tmp_path):
    """Fixed ids are a set (duplicates collapse, ascending); a later load line for
    the same node replaces the earlier one (inout.cpp:95,113-123)."""
    name = str(tmp_path / "m")
    with open(name + "_fixed.dat", "w") as fh:
        fh.write("5\n7\n3\n7\n1\n3\n")
    with open(name + "_loading.dat", "w") as fh:
        fh.write("3\n9\t1\t2\t3\n4\t0\t0\t-1.5e-3\n9\t4\t5\t6\n")
    fixed, loads = inout.getBoundaryConditions(name)
    assert fixed.tolist() == [0, 2, 6]
    assert list(loads.keys()) == [3, 8]
    assert loads[8] == (4.0, 5.0, 6.0) and loads[3] == (0.0, 0.0, -1.5e-3)


def test_voxel_values_other_than_one_are_empty(tmp_path):
    name = str(tmp_path / "v")
    with open(name + ".dat", "w") as fh:
        fh.write("2 1 2\n1,2\n0,1,\n")  # a trailing comma is tolerated
    model, dims = inout.loadVoxel(name)
    assert dims == (2, 1, 2)
    assert model.reshape(-1).tolist() == [1, 2, 0, 1]
    assert inout.occupancy(model).reshape(-1).tolist() == [1, 0, 0, 1]


def test_ke_falls_back_to_data_ke0(tmp_path, gauss_ke):
    os.makedirs(tmp_path / "data")
    inout.writeKe(str(tmp_path / "data" / "Ke0"), gauss_ke)
    os.rename(tmp_path / "data" / "Ke0_Ke0.dat", tmp_path / "data" / "Ke0.dat")
    assert np.array_equal(inout.getKe("model", directory=str(tmp_path)), gauss_ke)


def test_errors_name_the_file_and_line(tmp_path):
    name = str(tmp_path / "bad")
    with pytest.raises(FileNotFoundError):
        inout.loadVoxel(name)
    with open(name + ".dat", "w") as fh:
        fh.write("2 2 1\n1,1,x,1\n")
    with pytest.raises(ValueError, match=r"bad\.dat:2"):
        inout.loadVoxel(name)
    with open(name + ".dat", "w") as fh:
        fh.write("2 2 2\n1,1,1,1\n1,1,1\n")
    with pytest.raises(ValueError, match="expected 4 values"):
        inout.loadVoxel(name)
    with open(name + "_fixed.dat", "w") as fh:
        fh.write("2\n0\n")
    with open(name + "_loading.dat", "w") as fh:
        fh.write("0\n")
    with pytest.raises(ValueError):
        inout.getBoundaryConditions(name)


def test_save_vector_full_precision_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    u = np.concatenate([rng.standard_normal(1000) * 10.0 ** rng.integers(-12, 3, 1000),
                        [0.0, -0.0, 5e-324, 1.7976931348623157e308, 1e-7]])
    inout.saveVector(u, str(tmp_path / "u"))
    back = inout.loadVector(str(tmp_path / "u"))
    assert np.array_equal(back.view(np.int64), u.view(np.int64))


def test_save_vector_reference_form(tmp_path):
    """digits=-1 is std::to_string(double): fixed notation, 6 decimals."""
    inout.saveVector([1e-7, -0.5, 2.0, -3.25e-4, 1234.5678915], str(tmp_path / "r"), digits=-1)
    with open(str(tmp_path / "r") + "_out.csv") as fh:
        assert fh.read() == "0.000000,-0.500000,2.000000,-0.000325,1234.567892\n"


def test_model_name_like_the_reference():
    assert inout.model_name_of("data/armadillo_128.dat") == "data/armadillo_128"
    assert inout.model_name_of("./m.dat") == "./m"
    assert inout.model_name_of("m") == "m"


def test_save_domain_round_trip(tmp_path):
    d = domains.cantilever(8, 4, 4)
    name = str(tmp_path / "cant")
    inout.save_domain(d, name, ke=domains.hex8_stiffness())
    e = inout.load_domain(name)
    assert np.array_equal(e.voxels, d.voxels)
    assert np.array_equal(e.fixed, np.sort(d.fixed))
    assert np.array_equal(e.load_vector(), d.load_vector())
    with pytest.raises(ValueError):
        inout.save_domain(domains.spheres(16, count=2, levels=2), name)


def compile_example(tmp_path, lib):
    """Build tests/inout_example.cpp against libvfem.so."""
    exe = tmp_path / "inout_example"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "inout_example.cpp"), lib, "-Wl,-rpath," + os.path.dirname(lib),
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def test_cpp_readers_agree_with_python(armadillo, tmp_path):
    """include/vfem_inout.hpp reads the same values as inout.py (parse-only run,
    no GPU call) and writes the same CSV."""
    from vulkanfem_gb300 import api
    from vulkanfem_gb300 import build as vbuild
    api.load_library()
    exe = compile_example(tmp_path, vbuild.LIB)
    name = _write_armadillo(armadillo, tmp_path)
    with open(name + "_loading.dat", "a") as fh:  # a repeated node: the later line wins
        n0 = int(armadillo["load_nodes"][0]) + 1
        fh.write("%d\t0.25\t-0.5\t1e-9\n" % n0)
    with open(name + "_loading.dat") as fh:
        lines = fh.read().split("\n")
    lines[0] = str(int(lines[0]) + 1)
    with open(name + "_loading.dat", "w") as fh:
        fh.write("\n".join(lines))
    r = subprocess.run([exe, name + ".dat", "--parse-only"], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    got = dict(line.split(" ", 1) for line in r.stdout.strip().split("\n"))
    model, dims = inout.loadVoxel(name)
    ke = inout.getKe(name)
    fixed, loads = inout.getBoundaryConditions(name)
    flat = model.reshape(-1).astype(np.int64)
    i = np.arange(flat.size, dtype=np.int64)
    assert got["dims"] == "%d %d %d" % dims
    assert int(got["filled"]) == int((flat == 1).sum())
    assert int(got["weighted"]) == int(((i % 9973) * flat).sum())
    w = 1 + np.arange(24)[:, None] + 24 * np.arange(24)[None, :]
    assert float(got["ke"]) == pytest.approx(float((ke * w).sum()), rel=1e-14)
    assert got["fixed"] == "%d %d" % (fixed.size, int(fixed.sum()))
    nodes, vals = inout.loads_as_arrays(loads)
    cnt, idsum, vsum = got["loads"].split()
    assert int(cnt) == nodes.size and int(idsum) == int(nodes.sum())
    assert float(vsum) == pytest.approx(float((vals * [1, 2, 3]).sum()), rel=1e-12)
    assert loads[n0 - 1] == (0.25, -0.5, 1e-9)
    # saveVector: same text from C++ and Python
    with open(name + "_loadz_out.csv") as fh:
        cpp_text = fh.read()
    inout.saveVector(vals[:, 2], name + "_py")
    with open(name + "_py_out.csv") as fh:
        assert fh.read() == cpp_text
