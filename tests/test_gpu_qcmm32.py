"""QC/MM gradients with FP32 pair terms (pdg_qcmm_gradients with PDG_QCMM_FP32_PAIRS, the mixed method's
choice) against the FP64 kernels on the same inputs: the QC/MM water box (ABFS spline, 65 QC atoms, 12000 MM
atoms) and NBModelFull (1/r), QC and MM sides.  Tolerance 1e-6 Hartree/Bohr, ten times inside the gate against
the oracle (1e-5); measured up to ~6e-7, set by the FP32 rounding of absolute coordinates (~2e-6 A at 25 A) on
the closest contacts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model", [0, 1])
def test_fp32_pair_gradients_match_fp64(model):
    import torch
    from pdynamo_mirror_gb300 import NBModelABFS, _native, workloads
    L = _native.load()
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    frames = workloads.perturbed_frames(X, 4, sigma=0.02, seed=8)
    nq = len(sel)
    qc = torch.as_tensor(frames[:, :nq], device="cuda").contiguous()
    mm = torch.as_tensor(frames[:, nq:], device="cuda").contiguous()
    q = torch.as_tensor(Q[nq:], device="cuda")
    rng = np.random.default_rng(3)
    qcq = torch.as_tensor(rng.uniform(-0.9, 0.5, size=(4, nq)), device="cuda")
    knots = torch.as_tensor(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0).knots(), dtype=torch.float64, device="cuda") if model == 1 else None
    nk = 0 if knots is None else knots.numel() // 3
    sh = _native.stream_handle(torch.cuda.current_stream())
    wb = int(L.pdg_qcmm_workspace_bytes(4, mm.shape[1]))
    ws = torch.empty(wb, dtype=torch.uint8, device="cuda")
    out = {}
    for flag in (0, _native.QCMM_FP32_PAIRS):
        gq = torch.empty((4, nq, 3), dtype=torch.float64, device="cuda")
        gm = torch.empty((4, mm.shape[1], 3), dtype=torch.float64, device="cuda")
        _native.check(L.pdg_qcmm_gradients(model | flag, 4, nq, mm.shape[1], _native.ptr(qc), _native.ptr(mm), _native.ptr(q), _native.ptr(qcq),
                                           nk, _native.ptr(knots), 12.0, _native.ptr(gq), _native.ptr(gm), _native.ptr(ws), wb, sh),
                      "pdg_qcmm_gradients")
        out[flag] = (gq.cpu().numpy(), gm.cpu().numpy())
    (gq64, gm64), (gq32, gm32) = out[0], out[_native.QCMM_FP32_PAIRS]
    assert np.abs(gq64).max() > 1e-3 and np.abs(gm64).max() > 1e-4
    np.testing.assert_allclose(gq32, gq64, rtol=0, atol=1e-6)
    np.testing.assert_allclose(gm32, gm64, rtol=0, atol=1e-6)
