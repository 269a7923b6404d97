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
