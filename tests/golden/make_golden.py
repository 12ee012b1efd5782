"""Generate the committed golden fixtures from the reference's own data files.

Run once in a checkout that has the reference project mounted (pass its root as
the first argument).  Outputs, next to this script:

* ``armadillo_128.npz`` -- the reference's only model fixture
  (``data/armadillo_128{,_fixed,_loading}.dat`` and ``data/Ke0.dat``), read with
  the reference's own file conventions (``src/inout.cpp:6-128``: dims line, one
  comma-separated z-slice per line with x fastest; 1-based node ids converted to
  0-based as at ``inout.cpp:95,113``).  Occupancy is bit-packed.
* ``restriction_tables.npz`` -- the transfer tables of
  ``include/RestrictionOperator.hpp`` (restrictionOnElementValues,
  restrictionOnElement4Values, restrictionOperatorValues,
  restrictionOperator4Values, restrictionOperatorDoFValues,
  restrictionOperatorDoF4Values), parsed as numbers.

These are inputs and tables only; the reference publishes no outputs.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_voxels(path):
    with open(path) as fh:
        sx, sy, sz = (int(v) for v in fh.readline().split())
        vals = []
        for _ in range(sz):
            line = fh.readline().strip().rstrip(",")
            row = [int(v) for v in line.split(",")]
            assert len(row) == sx * sy, (len(row), sx * sy)
            vals.extend(row)
    vox = np.asarray(vals, dtype=np.uint8)
    assert set(np.unique(vox)) <= {0, 1}
    return (sx, sy, sz), vox


def read_fixed(path):
    with open(path) as fh:
        n = int(fh.readline())
        ids = [int(fh.readline()) - 1 for _ in range(n)]
    return np.asarray(ids, dtype=np.int64)


def read_loads(path):
    with open(path) as fh:
        n = int(fh.readline())
        nodes, loads = [], []
        for _ in range(n):
            parts = fh.readline().split("\t")
            nodes.append(int(parts[0]) - 1)
            loads.append([float(p) for p in parts[1:4]])
    return np.asarray(nodes, dtype=np.int64), np.asarray(loads, dtype=np.float64)


def read_ke(path):
    rows = []
    with open(path) as fh:
        for _ in range(24):
            rows.append([float(v) for v in fh.readline().strip().split(",")])
    ke = np.asarray(rows, dtype=np.float64)
    assert ke.shape == (24, 24)
    return ke


def parse_tables(path):
    text = open(path).read()
    out = {}
    for m in re.finditer(r"std::array<(int|double),\s*(\d+)>\s+(\w+)\s*=\s*\{([^}]*)\}", text):
        typ, n, name, body = m.group(1), int(m.group(2)), m.group(3), m.group(4)
        nums = [float(v) for v in re.split(r"[,\s]+", body.strip()) if v]
        assert len(nums) == n, (name, len(nums), n)
        out[name] = np.asarray(nums, dtype=np.int32 if typ == "int" else np.float64)
    return out


def main(ref_root):
    data = os.path.join(ref_root, "data")
    dims, vox = read_voxels(os.path.join(data, "armadillo_128.dat"))
    fixed = read_fixed(os.path.join(data, "armadillo_128_fixed.dat"))
    lnodes, lvals = read_loads(os.path.join(data, "armadillo_128_loading.dat"))
    ke0 = read_ke(os.path.join(data, "Ke0.dat"))
    np.savez_compressed(
        os.path.join(HERE, "armadillo_128.npz"),
        dims=np.asarray(dims, dtype=np.int32),
        voxels_packed=np.packbits(vox),
        nvox=np.int64(vox.size),
        fixed=fixed,
        load_nodes=lnodes,
        load_values=lvals,
        ke0=ke0,
    )
    tables = parse_tables(os.path.join(ref_root, "include", "RestrictionOperator.hpp"))
    np.savez_compressed(os.path.join(HERE, "restriction_tables.npz"), **tables)
    print("dims", dims, "filled", int(vox.sum()), "fixed", fixed.size, "loads", lnodes.size)
    print("tables", {k: v.size for k, v in tables.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <reference project root>")
    main(sys.argv[1])
