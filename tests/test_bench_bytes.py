"""The algorithmic bytes behind bench.py's roofline fractions, for the 256^3
grid (257^3 nodes, 256^3 voxels, a 129^3-node first coarse level, 13,872
coarse free DOFs): each formula against its count written out by hand."""
import bench

N, NE, NC, NCF = 257 ** 3, 256 ** 3, 129 ** 3, 13872
G0 = {"nodes": N, "voxels": NE}
G1 = {"nodes": NC, "coarse_free": NCF}


def test_fp32_kernel_bytes():
    s = 4
    ab = lambda k: bench.algorithmic_bytes(k, G0, G1, s)
    # product: x in, Kx out (3 values per node each), modulus, occupancy and fixed bits
    assert ab("matvec") == 2 * 3 * s * N + 4 * NE + NE / 8 + N / 8
    # fused product: p_old, z, x in; p, x, Kp out
    assert ab("matvec_px") == 6 * 3 * s * N + 4 * NE + NE / 8 + N / 8
    # residual update + first restriction: r, Ap in, r out; coarse r out
    assert ab("update_restrict") == 3 * 3 * s * N + 3 * s * NC
    # up-leg: coarse z in; r in (FP32), D^-1 in (FP16), z out; fixed bits
    assert ab("prolong") == 3 * s * NC + (12 + 6 + 12) * N + N / 8
    # coarsest solve: the FP16 lower block triangle, about n^2 bytes
    assert ab("coarse") == NCF * NCF
    assert round(ab("matvec_px") / 1e6) == 1293


def test_fp64_kernel_bytes():
    s = 8
    ab = lambda k: bench.algorithmic_bytes(k, G0, G1, s)
    assert ab("matvec") == 2 * 3 * s * N + 4 * NE + NE / 8 + N / 8
    assert ab("prolong") == 3 * s * NC + 3 * 3 * s * N + N / 8
    assert ab("update_xr") == 6 * 3 * s * N
    assert ab("update_p") == 3 * 3 * s * N
    assert ab("coarse") == 8 * NCF * NCF
