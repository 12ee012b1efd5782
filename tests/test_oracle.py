"""CPU tests of the oracle: pinned to the reference's fixture data and to
derived known-answer facts, and cross-checked against the structured dense-grid
formulation that the CUDA kernels implement."""
import os

import numpy as np
import pytest

import oracle
from vulkanfem_gb300 import domains
from tests.conftest import GOLDEN
from tests import structured_ref as sr


def test_ke0_is_permuted_gauss_hex(armadillo, gauss_ke):
    """data/Ke0.dat == 2x2x2-Gauss trilinear hex (E=1, nu=0.3) under the GMGS-3D
    node permutation (scripts/outputToC.m:13-14)."""
    P = domains.KE0_NODE_PERM
    idx = np.array([3 * P[i] + c for i in range(8) for c in range(3)])
    assert np.abs(armadillo["ke0"] - gauss_ke[np.ix_(idx, idx)]).max() < 1e-14
    k = 1872.0 * gauss_ke
    assert np.abs(k - np.round(k)).max() < 1e-9
    assert np.abs(np.round(k)).max() == 440


def test_gauss_ke_rigid_modes(gauss_ke):
    X = np.array([[a & 1, (a >> 1) & 1, a >> 2] for a in range(8)], float) - 0.5
    for ax in range(3):
        w = np.zeros(3)
        w[ax] = 1
        assert np.abs(gauss_ke @ np.cross(w, X).reshape(-1)).max() < 1e-14
        t = np.zeros((8, 3))
        t[:, ax] = 1
        assert np.abs(gauss_ke @ t.reshape(-1)).max() < 1e-14
    ev = np.linalg.eigvalsh(gauss_ke)
    assert (ev[:6] < 1e-12).all() and (ev[6:] > 1e-3).all()


def test_restriction_tables_are_trilinear():
    """The reference's transfer tables (include/RestrictionOperator.hpp) equal the
    trilinear tensor-product weights used by the kernels."""
    t = np.load(os.path.join(GOLDEN, "restriction_tables.npz"))
    for div, name, nb in ((2, "restrictionOperatorValues", 27), (4, "restrictionOperator4Values", 125)):
        R = t[name].reshape(nb, 8)
        n = div + 1
        for s in range(nb):
            sx, sy, sz = s % n, (s // n) % n, s // (n * n)
            for b in range(8):
                bx, by, bz = b & 1, (b >> 1) & 1, b >> 2
                w = 1.0
                for a, bb in ((sx, bx), (sy, by), (sz, bz)):
                    w *= (div - a) / div if bb == 0 else a / div
                assert R[s, b] == pytest.approx(w, abs=1e-6)
    for div, name, nb in ((2, "restrictionOperatorDoFValues", 27), (4, "restrictionOperatorDoF4Values", 125)):
        RD = t[name].reshape(3 * nb, 24)
        R = t["restrictionOperatorValues" if div == 2 else "restrictionOperator4Values"].reshape(nb, 8)
        assert np.abs(RD - np.kron(R, np.eye(3))).max() < 1e-6
    for div, name in ((2, "restrictionOnElementValues"), (4, "restrictionOnElement4Values")):
        M = t[name].reshape(div ** 3, 8)
        n = div + 1
        for ch in range(div ** 3):
            cx, cy, cz = ch % div, (ch // div) % div, ch // (div * div)
            for a in range(8):
                assert M[ch, a] == (cx + (a & 1)) + n * ((cy + ((a >> 1) & 1)) + n * (cz + (a >> 2)))


def test_armadillo_counts(armadillo):
    """Facts of the reference's only fixture: 112x128x128 voxels, 166,090 filled,
    187,485 used nodes = 562,455 DOFs, 2,535 fixed, 1,331 loaded (+z, total 2.0),
    fixed and loaded disjoint, ids in the compressed numbering."""
    vox = armadillo["voxels"]
    assert vox.shape == (128, 128, 112)
    assert int(vox.sum()) == 166090
    assert int(domains.used_nodes_mask(vox).sum()) == 187485
    assert armadillo["fixed"].size == 2535 and armadillo["load_nodes"].size == 1331
    assert np.abs(armadillo["load_values"][:, :2]).max() == 0
    assert armadillo["load_values"][:, 2].sum() == pytest.approx(2.0)
    assert not set(armadillo["fixed"]) & set(armadillo["load_nodes"])
    assert armadillo["load_nodes"].max() == 187484


def _oracle(d, ke=None, levels=None, skip=0):
    ke = domains.hex8_stiffness() if ke is None else ke
    return oracle.Oracle(d.voxels, ke, d.fixed, levels or d.num_levels, skip)


def test_cantilever_converges():
    d = domains.cantilever()
    o = _oracle(d)
    assert o.num_levels == 3
    assert [o.num_dofs(l) for l in range(3)] == [28611, 3 * 9 * 9 * 17, 3 * 5 * 5 * 9]
    f = d.load_vector()
    x, it, err = o.pcg(f)
    assert err < 1e-6
    r = f - o.matvec(x)
    assert np.linalg.norm(r) / np.linalg.norm(f) < 1e-6
    assert 10 < it < 60
    # the solution sags in -z, compliance f.u > 0
    assert f @ x > 0
    assert x.reshape(-1, 3)[d.load_nodes, 2].mean() < 0


def _random_domain(shape, fill, seed):
    rng = np.random.default_rng(seed)
    vox = (rng.random(shape) < fill).astype(np.uint8)
    vox[0] = 1  # grounded
    vox = domains.keep_grounded(vox)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0])
    return vox, fixed


@pytest.mark.parametrize("shape,levels,skip", [((8, 6, 10), 3, 0), ((12, 8, 8), 3, 0), ((16, 16, 16), 2, 1)])
def test_structured_formulation_matches_oracle(shape, levels, skip):
    """The dense-grid formulation of the kernels (full weighting with no W tables,
    masked trilinear prolongation, fixed dilation, Galerkin-diagonal rule) agrees
    with the oracle's element-list restatement of FEM.cpp / MultigridPreconditioner.hpp."""
    vox, fixed = _random_domain(shape, 0.7, 3)
    ke = domains.hex8_stiffness()
    o = oracle.Oracle(vox, ke, fixed, levels, skip)
    rng = np.random.default_rng(1)
    elem = vox.astype(bool)
    masks = [sr.used_mask(elem)]
    fixed_d = np.zeros(masks[0].shape, bool)
    fixed_d.reshape(-1)[np.flatnonzero(masks[0].reshape(-1))[fixed]] = True
    fixeds = [fixed_d]
    for lv in range(o.num_levels - 1):
        div = 4 if (lv == 0 and skip) else 2
        elem = sr.coarsen(elem, div)
        masks.append(sr.used_mask(elem))
        fixeds.append(sr.fixed_dilate(fixeds[-1], masks[-1].shape, div))
        assert o.num_dofs(lv + 1) == 3 * int(masks[-1].sum())
        # numbering: used nodes in linear order.  The reference halves the level
        # dims even for the skipped 4x level (FEM.cpp:256-260), so compare coordinates.
        lin = np.flatnonzero(masks[-1].reshape(-1))
        ex, ey, _ = o.level_dims(lv + 1)
        on = o.nodes(lv + 1)
        oz, oy, ox = on // ((ex + 1) * (ey + 1)), (on // (ex + 1)) % (ey + 1), on % (ex + 1)
        mz, my, mx = np.unravel_index(lin, masks[-1].shape)
        assert np.array_equal(oz, mz) and np.array_equal(oy, my) and np.array_equal(ox, mx)
        # fixed sets
        assert np.array_equal(o.fixed(lv + 1), np.flatnonzero(fixeds[-1].reshape(-1)[lin]))
        # restriction and interpolation
        v = rng.standard_normal(o.num_dofs(lv))
        rc = sr.to_compressed(sr.restrict(sr.to_dense(v, masks[lv]), masks[-1].shape, div), masks[-1])
        assert np.abs(o.restrict(lv, v) - rc).max() < 1e-12 * max(1, np.abs(rc).max())
        c = rng.standard_normal(o.num_dofs(lv + 1))
        pf = sr.to_compressed(sr.prolong(sr.to_dense(c, masks[-1]), masks[lv], div), masks[lv])
        assert np.abs(o.interpolate(lv, c) - pf).max() < 1e-12 * max(1, np.abs(pf).max())


def test_operator_and_preconditioner_symmetric():
    vox, fixed = _random_domain((10, 9, 11), 0.65, 7)
    o = oracle.Oracle(vox, domains.hex8_stiffness(), fixed, 3, 0)
    rng = np.random.default_rng(0)
    n = o.num_dofs()
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    for v in (a, b):
        v.reshape(-1, 3)[fixed] = 0
    assert abs(a @ o.matvec(b) - b @ o.matvec(a)) < 1e-10 * abs(a @ o.matvec(b))
    assert abs(a @ o.precond(b) - b @ o.precond(a)) < 1e-10 * abs(a @ o.precond(b))
    assert a @ o.matvec(a) > 0 and a @ o.precond(a) > 0


def test_matvec_matches_dense_ebe():
    vox, fixed = _random_domain((7, 5, 6), 0.6, 11)
    ke = domains.hex8_stiffness()
    o = oracle.Oracle(vox, ke, fixed, 1, 0)
    mask = sr.used_mask(vox.astype(bool))
    fm = np.zeros(mask.shape, bool)
    fm.reshape(-1)[np.flatnonzero(mask.reshape(-1))[fixed]] = True
    x = np.random.default_rng(2).standard_normal(o.num_dofs())
    y = sr.to_compressed(sr.matvec(vox.astype(float), ke, sr.to_dense(x, mask), fm), mask)
    assert np.abs(o.matvec(x) - y).max() < 1e-13 * np.abs(y).max()


def test_float_coefficient_variant_close():
    """FEMGPU.cpp:226-242 stores W and D^-1 as float; the iteration count stays put."""
    d = domains.cantilever()
    o = _oracle(d)
    f = d.load_vector()
    _, it64, _ = o.pcg(f)
    o.set_float_coeffs(True)
    _, it32, err = o.pcg(f)
    assert abs(it32 - it64) <= 1 and err < 1e-6


def test_armadillo_hierarchy(armadillo):
    o = oracle.Oracle(armadillo["voxels"], armadillo["ke0"], armadillo["fixed"], 3, 0)
    assert o.num_dofs(0) == 562455
    assert o.num_levels == 3
    assert o.level_dims(1) == (56, 64, 64) and o.level_dims(2) == (28, 32, 32)


def test_patch_test_known_answers():
    """Analytic known answers (tests/patch_test.py): the oracle's product of a
    linear field on a solid box is zero inside and the consistent traction
    loads on the faces (to 1e-12 of the largest load), and its MG-PCG solve
    with those loads returns the linear field (to 1e-9 at rtol 1e-12)."""
    from tests import patch_test as pt
    vox, fixed, coords = pt.box()
    o = oracle.Oracle(vox, domains.hex8_stiffness(pt.E, pt.NU), fixed, 2, 0)
    for name, u, f in pt.fields(vox, coords):
        g = pt.expected_product(f, fixed)
        y = o.matvec(u)
        assert np.max(np.abs(y - g)) < 1e-12 * np.max(np.abs(g)), name
        x, it, _ = o.pcg(g, tol=1e-12)
        assert np.linalg.norm(x - u) < 1e-9 * np.linalg.norm(u), (name, it)
