"""pdg_gradients_static_scratch (library-owned scratch, no allocation at call time) against pdg_gradients.

Both run the same gradient kernels on the same densities, so they agree to round-off; the tolerance below
is 1e-12 Hartree/Bohr.  Two calls in a row check that nothing of one call leaks into the next.  This file
is collected last so that it also runs after every other GPU test has used the device.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1.0e-12   # Hartree/Bohr


def _engine_and_densities(n_waters, n_frames, seed):
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, workloads
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X = workloads.water_cluster(n_waters, seed=seed)
    frames = workloads.perturbed_frames(X, n_frames, sigma=0.03, seed=seed + 1)
    eng = QCEngine("am1", Z, 0)
    qc = torch.as_tensor(frames, dtype=torch.float64, device="cuda")
    out = eng.run(qc, DIISSCFConverger(), gradients=False, warm_start=False)
    assert (out["status"].cpu().numpy() == 0).all()
    return eng, qc, eng.density.clone()


def test_static_scratch_gradients_match_workspace_path_twice():
    import torch
    eng, qc, P = _engine_and_densities(16, 6, seed=11)
    ref = eng.gradients(qc, P).cpu().numpy()
    for _ in range(2):
        g = eng.gradients_static_scratch(qc, P)
        torch.cuda.synchronize()
        np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=0, atol=TOL)


def test_static_scratch_call_leaves_free_device_memory_unchanged():
    """The property the entry point exists for: once a first call on the device has loaded the kernels and looked
    up the scratch's address, a further call allocates no device memory.  Every buffer of the call exists before
    it, so torch's caching allocator stays idle, and the driver's free-memory count (cudaMemGetInfo) must be the
    same before and after."""
    import torch
    from pdynamo_mirror_gb300 import _native
    from pdynamo_mirror_gb300.engine import ANGSTROMS_TO_BOHRS
    eng, qc, P = _engine_and_densities(16, 6, seed=12)
    xyz = (qc * ANGSTROMS_TO_BOHRS).contiguous()
    g = torch.empty((qc.shape[0], eng.n_atoms, 3), dtype=torch.float64, device="cuda")
    stream = _native.stream_handle(torch.cuda.current_stream())

    def call():
        _native.check(eng.L.pdg_gradients_static_scratch(eng.handle, qc.shape[0], _native.ptr(xyz), _native.ptr(P),
                                                         _native.ptr(g), stream), "pdg_gradients_static_scratch")
        torch.cuda.synchronize()

    call()                                     # first call: kernels loaded, scratch address looked up
    ref = g.clone()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    call()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, "the call changed free device memory by %d bytes" % (free0 - free1)
    np.testing.assert_allclose(g.cpu().numpy(), ref.cpu().numpy(), rtol=0, atol=TOL)


def test_static_scratch_rejects_requests_beyond_its_size():
    import torch
    from pdynamo_mirror_gb300 import _native, workloads
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X = workloads.water_cluster(22, seed=5)            # 66 atoms, 2145 pairs: 6464 doubles per frame
    eng = QCEngine("am1", Z, 0)
    n = 82                                                # 82 * 6464 = 530048 > 524288
    qc = torch.as_tensor(np.repeat(X[None], n, axis=0), dtype=torch.float64, device="cuda")
    P = torch.zeros((n, eng.n_basis, eng.n_basis), dtype=torch.float64, device="cuda")
    with pytest.raises(_native.NativeError, match="static scratch|more than the 524288"):
        eng.gradients_static_scratch(qc, P)
    g = eng.gradients_static_scratch(qc[:81], P[:81])     # 81 frames fit
    assert g.shape == (81, len(Z), 3)
