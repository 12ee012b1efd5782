"""Readers and writers for the reference's model files (src/inout.cpp), with the
reference's names, plus writers so synthetic domains can be exported in the same
format and a loss-free result output.

File formats (the reference's; paths relative to the working directory unless a
directory is given):

* ``<name>.dat``: ``"sx sy sz"``, then ``sz`` lines, each the ``sx*sy`` values of
  one z-slice (x fastest), comma-separated; a value of 1 is a filled voxel
  (src/FEM.cpp:75 tests ``== 1``), anything else is empty (inout.cpp:6-41).
* ``<name>_Ke0.dat``: 24 lines of 24 comma-separated numbers; ``data/Ke0.dat`` is
  read when it is absent (inout.cpp:43-72).
* ``<name>_fixed.dat``: a count, then one 1-based node id per line; kept as a set
  (inout.cpp:82-97).
* ``<name>_loading.dat``: a count, then ``id<TAB>fx<TAB>fy<TAB>fz`` per line with
  1-based ids; kept in a map, so a later line for a node replaces an earlier one
  (inout.cpp:99-125).
* ``<name>_out.csv``: the solution on one comma-separated line.  The reference
  writes ``std::to_string`` (fixed, 6 decimals, inout.cpp:206-225), which loses
  everything below 5e-7; :func:`saveVector` writes 17 significant digits by
  default (exact round trip) and the reference's form with ``digits=-1``.

Errors: a missing file raises ``FileNotFoundError``; a malformed one raises
``ValueError`` naming the file and line (the reference throws from ``std::stoi``
or reads from a stream that failed to open).
"""
import os

import numpy as np

from . import domains


def model_name_of(file_name):
    """The model name the reference derives from its argument: everything before
    the first '.' after position 0 (src/main.cpp:38)."""
    k = file_name.find(".", 1)
    return file_name if k < 0 else file_name[:k]


def _path(name, suffix, directory=None):
    p = name + suffix
    return os.path.join(directory, p) if directory else p


def _fields(line, sep):
    parts = line.rstrip("\r\n").split(sep)
    while parts and not parts[-1].strip():
        parts.pop()
    return parts


def _bad(path, line_no, what):
    return ValueError("%s:%d: %s" % (path, line_no, what))


def _int(tok, path, ln):
    try:
        return int(tok.strip())
    except ValueError:
        raise _bad(path, ln, "bad integer %r" % tok) from None


def _real(tok, path, ln):
    try:
        v = float(tok.strip())
    except ValueError:
        raise _bad(path, ln, "bad number %r" % tok) from None
    if not np.isfinite(v):
        raise _bad(path, ln, "non-finite number %r" % tok)
    return v


def _lines(path):
    with open(path) as fh:
        return fh.read().split("\n")


def loadVoxel(model_name, directory=None):
    """Voxel values of ``<model_name>.dat`` as int32 [z, y, x] and the sizes
    (sizeX, sizeY, sizeZ) (inout.cpp:6-41)."""
    path = _path(model_name, ".dat", directory)
    lines = _lines(path)
    try:
        sx, sy, sz = (int(v) for v in lines[0].split())
    except (ValueError, IndexError):
        raise _bad(path, 1, "bad dimensions line %r" % (lines[0] if lines else "")) from None
    if min(sx, sy, sz) <= 0:
        raise _bad(path, 1, "dimensions must be positive")
    if len(lines) < sz + 1:
        raise _bad(path, len(lines), "expected %d slice lines" % sz)
    model = np.empty((sz, sy * sx), np.int32)
    for z in range(sz):
        f = _fields(lines[z + 1], ",")
        if len(f) != sx * sy:
            raise _bad(path, z + 2, "expected %d values, found %d" % (sx * sy, len(f)))
        try:
            model[z] = np.asarray(f, dtype=np.int64)
        except ValueError:
            for t in f:
                _int(t, path, z + 2)
            raise
    return model.reshape(sz, sy, sx), (sx, sy, sz)


def occupancy(model):
    """1 where the voxel value is 1 (src/FEM.cpp:75), else 0, as uint8."""
    return (np.asarray(model) == 1).astype(np.uint8)


def getKe(model_name, directory=None):
    """The 24x24 element stiffness of ``<model_name>_Ke0.dat``, else
    ``data/Ke0.dat`` (inout.cpp:43-72).  Node order is the reference's
    (its index -> local corner permutation is ``domains.KE0_NODE_PERM``)."""
    path = _path(model_name, "_Ke0.dat", directory)
    if not os.path.exists(path):
        path = os.path.join(directory, "data", "Ke0.dat") if directory else os.path.join("data", "Ke0.dat")
    lines = _lines(path)
    ke = np.empty((24, 24), np.float64)
    for i in range(24):
        if i >= len(lines):
            raise _bad(path, i + 1, "unexpected end of file")
        f = _fields(lines[i], ",")
        if len(f) != 24:
            raise _bad(path, i + 1, "expected 24 values, found %d" % len(f))
        ke[i] = [_real(t, path, i + 1) for t in f]
    return ke


def getBoundaryConditions(model_name, directory=None):
    """(fixedNodes, loadedNodes): the fixed node ids as a sorted, duplicate-free
    int64 array (the reference's std::set) and the loads as a dict node ->
    (fx, fy, fz) in ascending node order (its std::map); ids 0-based
    (inout.cpp:77-128)."""
    path = _path(model_name, "_fixed.dat", directory)
    lines = _lines(path)
    n = _int(lines[0], path, 1) if lines else 0
    if n < 0 or len(lines) < n + 1:
        raise _bad(path, 1, "count %d does not match the file" % n)
    fixed = set()
    for i in range(n):
        v = _int(lines[i + 1], path, i + 2)
        if v < 1:
            raise _bad(path, i + 2, "node ids are 1-based")
        fixed.add(v - 1)
    path = _path(model_name, "_loading.dat", directory)
    lines = _lines(path)
    n = _int(lines[0], path, 1) if lines else 0
    if n < 0 or len(lines) < n + 1:
        raise _bad(path, 1, "count %d does not match the file" % n)
    loads = {}
    for i in range(n):
        f = _fields(lines[i + 1], "\t")
        if len(f) != 4:
            raise _bad(path, i + 2, "expected id<TAB>fx<TAB>fy<TAB>fz")
        v = _int(f[0], path, i + 2)
        if v < 1:
            raise _bad(path, i + 2, "node ids are 1-based")
        loads[v - 1] = tuple(_real(t, path, i + 2) for t in f[1:])
    return np.asarray(sorted(fixed), np.int64), dict(sorted(loads.items()))


def loads_as_arrays(loadedNodes):
    nodes = np.asarray(list(loadedNodes.keys()), np.int64)
    vals = np.asarray(list(loadedNodes.values()), np.float64).reshape(-1, 3)
    return nodes, vals


def format_value(v, digits=17):
    """One number as :func:`saveVector` writes it."""
    return ("%f" % v) if digits < 0 else ("%.*g" % (digits, v))


def saveVector(data, name, digits=17, directory=None):
    """Write ``<name>_out.csv``: the values on one comma-separated line
    (inout.cpp:206-225).  digits=17 round-trips every double; digits=-1 is the
    reference's std::to_string form."""
    path = _path(name, "_out.csv", directory)
    a = np.asarray(data, np.float64).reshape(-1)
    with open(path, "w") as fh:
        fh.write(",".join(format_value(float(v), digits) for v in a))
        fh.write("\n")
    return path


def loadVector(name, directory=None):
    """Read a ``<name>_out.csv`` written by :func:`saveVector` or the reference."""
    path = _path(name, "_out.csv", directory)
    lines = _lines(path)
    return np.asarray([_real(t, path, 1) for t in _fields(lines[0], ",")], np.float64)


# ---------------------------------------------------------------- writers

def writeVoxel(model_name, model, directory=None):
    """Write values [z, y, x] as ``<model_name>.dat`` in the reference's layout."""
    m = np.asarray(model)
    sz, sy, sx = m.shape
    path = _path(model_name, ".dat", directory)
    with open(path, "w") as fh:
        fh.write("%d %d %d\n" % (sx, sy, sz))
        for z in range(sz):
            fh.write(",".join(str(int(v)) for v in m[z].reshape(-1)))
            fh.write("\n")
    return path


def writeKe(model_name, ke, directory=None):
    """Write a 24x24 element matrix as ``<model_name>_Ke0.dat`` (17 digits)."""
    k = np.asarray(ke, np.float64).reshape(24, 24)
    path = _path(model_name, "_Ke0.dat", directory)
    with open(path, "w") as fh:
        for row in k:
            fh.write(",".join("%.17g" % v for v in row) + "\n")
    return path


def writeBoundaryConditions(model_name, fixedNodes, loadedNodes, directory=None):
    """Write ``<model_name>_fixed.dat`` and ``_loading.dat`` (1-based ids).
    ``loadedNodes`` is a dict node -> (fx, fy, fz) or a (nodes, values) pair."""
    fixed = np.asarray(fixedNodes, np.int64).reshape(-1)
    if isinstance(loadedNodes, dict):
        nodes, vals = loads_as_arrays(loadedNodes)
    else:
        nodes, vals = np.asarray(loadedNodes[0], np.int64), np.asarray(loadedNodes[1], np.float64).reshape(-1, 3)
    p1 = _path(model_name, "_fixed.dat", directory)
    with open(p1, "w") as fh:
        fh.write("%d\n" % fixed.size)
        fh.write("".join("%d\n" % (v + 1) for v in fixed))
    p2 = _path(model_name, "_loading.dat", directory)
    with open(p2, "w") as fh:
        fh.write("%d\n" % nodes.size)
        for nd, v in zip(nodes, vals):
            fh.write("%d\t%.17g\t%.17g\t%.17g\n" % (nd + 1, v[0], v[1], v[2]))
    return p1, p2


# ---------------------------------------------------------------- domains

def load_domain(model_name, num_levels=3, directory=None):
    """A :class:`domains.Domain` from the reference's model files, plus its Ke
    (``domain.meta["Ke"]``, reference node order)."""
    model, dims = loadVoxel(model_name, directory)
    fixed, loads = getBoundaryConditions(model_name, directory)
    nodes, vals = loads_as_arrays(loads)
    d = domains.Domain(name=os.path.basename(model_name), voxels=occupancy(model), fixed=fixed,
                       load_nodes=nodes, load_values=vals, num_levels=num_levels)
    d.meta["Ke"] = getKe(model_name, directory)
    d.meta["dims"] = dims
    return d


def save_domain(d, model_name, ke=None, directory=None):
    """Export a domain in the reference's format (uniform modulus only: the
    reference's files carry no per-voxel modulus)."""
    if d.E is not None:
        raise ValueError("the reference's model files cannot carry a per-voxel modulus")
    writeVoxel(model_name, d.voxels, directory)
    writeBoundaryConditions(model_name, d.fixed, (d.load_nodes, d.load_values), directory)
    if ke is not None:
        writeKe(model_name, ke, directory)
