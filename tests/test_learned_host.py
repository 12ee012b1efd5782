"""Host-side layout of the learned part (vulkanfem_gb300/learned.py, no GPU):
node features, training targets and the loss mask on the padded grid must put
every used node's values at its grid position, in the library's compressed
node order (x fastest), so that the network's output maps back to the solver's
numbering."""
import numpy as np

from vulkanfem_gb300 import domains, learned


def _field():
    for seed in range(20):
        try:
            return domains.training_field(16, seed=seed, levels=2)
        except ValueError:
            continue
    raise AssertionError("no training field with a grounded component")


def test_feature_target_and_mask_layout():
    d = _field()
    n_pad = learned.padded(17)
    rng = np.random.default_rng(0)
    u = rng.standard_normal(d.num_dofs)
    u.reshape(-1, 3)[d.fixed] = 0.0
    feats, mask, scale = learned.node_features(d.voxels, d.E, d.fixed, d.load_nodes, d.load_values, n_pad, z0=u)
    nz, ny, nx = mask.shape
    assert feats.shape == (n_pad, n_pad, n_pad, learned.NCH) and scale > 0
    used = feats[:nz, :ny, :nx]
    assert np.array_equal(used[..., 0] > 0, mask)
    # everything outside the node grid is zero padding
    assert not feats[nz:].any() and not feats[:, ny:].any() and not feats[:, :, nx:].any()
    # fixed flags at exactly the fixed nodes (compressed order)
    at = used[mask]
    assert np.array_equal(np.flatnonzero(at[:, 2]), np.unique(d.fixed))
    # loads normalised by the largest component, at the loaded nodes
    lv = np.asarray(d.load_values).reshape(-1, 3)
    assert np.allclose(at[np.asarray(d.load_nodes), 3:6], lv / np.abs(lv).max())
    # the V-cycle response channels carry z0 / rms(z0) in compressed order
    rms = np.sqrt(np.mean(u * u))
    assert np.allclose(at[:, 6:9], (u.reshape(-1, 3) / rms).astype(np.float32), rtol=1e-6, atol=1e-7)
    # targets: u / rms(u) at the used nodes; the loss mask excludes fixed nodes
    t = learned.target_grid(u, mask, scale, n_pad)
    assert np.allclose(t[:nz, :ny, :nx][mask], (u.reshape(-1, 3) / rms).astype(np.float32), rtol=1e-6, atol=1e-7)
    m = learned.loss_mask(mask, d.fixed, n_pad)[:nz, :ny, :nx][mask]
    assert m[np.asarray(d.fixed)].sum() == 0
    assert m.sum() == mask.sum() - np.unique(d.fixed).size
