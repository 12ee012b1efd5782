"""GPU test of vfem_apply_operator_device_noalloc, the operator product for
callers that cannot allocate GPU memory at the call site (hosts whose own
memory pool owns the device memory, loops that must not hit cudaMalloc's
device synchronisation).

Its result must equal the regular entry point vfem_apply_operator (same
tolerance as the other operator parity tests, 1e-11 relative), on two calls
in a row, since the calls share the library's fixed scratch array.  The second
call puts NaN into x at the unused nodes, which the entry point documents as
ignored, and checks that free device memory is the same before and after it.
The device buffers below are the caller's (allocated by torch here, as a host
pool would).
"""
import ctypes

import numpy as np
import pytest

from vulkanfem_gb300 import api, domains

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _domain():
    rng = np.random.default_rng(21)
    vox = (rng.random((9, 11, 13)) < 0.75).astype(np.uint8)
    vox[0] = 1
    vox = domains.keep_grounded(vox)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0])
    return vox, fixed


def test_noalloc_product_matches_apply_operator_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    vox, fixed = _domain()
    ke = domains.hex8_stiffness()
    E = np.random.default_rng(3).lognormal(0.0, 0.5, vox.shape).astype(np.float32)
    A = api.assembleSystemMatrix(vox, ke, fixed, 3, E=E)
    lib = api.load_library()
    mask = domains.used_nodes_mask(vox)
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream()
    for call in range(2):
        x = rng.standard_normal(A.rows())
        y_ref = A @ x                                   # the existing entry point
        xd = np.zeros(mask.shape + (3,))
        if call == 1:
            xd[~mask] = np.nan                          # ignored: no element touches these nodes
        xd[mask] = x.reshape(-1, 3)
        tx = torch.from_numpy(xd.reshape(-1)).cuda()
        ty = torch.full_like(tx, float("nan"))
        tdot = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        s = lib.vfem_apply_operator_device_noalloc(A._h, ctypes.c_void_p(tx.data_ptr()),
                                                   ctypes.c_void_p(ty.data_ptr()),
                                                   ctypes.c_void_p(tdot.data_ptr()),
                                                   ctypes.c_void_p(stream.cuda_stream))
        assert s == 0, api.STATUS_NAMES.get(s, s)
        torch.cuda.synchronize()
        if call == 1:                                   # after the first call's one-time set-up
            assert torch.cuda.mem_get_info()[0] == free_before
        yd = ty.cpu().numpy().reshape(mask.shape + (3,))
        y = yd[mask].reshape(-1)
        assert np.isfinite(yd).all()
        assert np.abs(yd[~mask]).max(initial=0.0) == 0.0
        assert np.linalg.norm(y - y_ref) <= TOL * np.linalg.norm(y_ref), call
        ref_dot = float(x @ y_ref)
        assert abs(float(tdot.item()) - ref_dot) <= TOL * abs(ref_dot), call
