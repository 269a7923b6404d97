"""QC/MM electrostatics through the per-frame near lists (pdg_qcmm_potentials / pdg_qcmm_gradients) against the
oracle's scan over every MM atom (PairwiseInteractionABFS_QCMMPotentials / _QCMMGradients, PairwiseInteraction.c:612,
:542, which the reference runs over its cell-grid pair list): the benchmark's water box (4000 TIP3P waters, 12 A
outer cutoff) on several perturbed frames at once, a frame whose QC region sits far from every MM atom (empty near
list: zero potentials and gradients), and a frame that wraps its QC region in MM atoms exactly at the cutoff margin.
Tolerance 1e-11 (potentials in a.u., gradients in Hartree/Bohr): the same FP64 pair terms as the oracle, summed in MM
index order; MM atoms outside the cutoff of every QC atom must get exactly zero gradient."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run(L, model, qcx, mmx, q, qcq, knots, flag=0):
    import torch
    from pdynamo_mirror_gb300 import _native
    F, nq, nm = qcx.shape[0], qcx.shape[1], mmx.shape[1]
    dq = torch.as_tensor(qcx, dtype=torch.float64, device="cuda").contiguous()
    dm = torch.as_tensor(mmx, dtype=torch.float64, device="cuda").contiguous()
    dc = torch.as_tensor(q, dtype=torch.float64, device="cuda").contiguous()
    dqq = torch.as_tensor(qcq, dtype=torch.float64, device="cuda").contiguous()
    kn = None if knots is None else torch.as_tensor(knots, dtype=torch.float64, device="cuda")
    nk = 0 if kn is None else kn.numel() // 3
    wb = int(L.pdg_qcmm_workspace_bytes(F, nm))
    ws = torch.full((wb,), 0xAB, dtype=torch.uint8, device="cuda")     # stale contents must not matter
    s = _native.stream_handle(torch.cuda.current_stream())
    phi = torch.empty((F, nq), dtype=torch.float64, device="cuda")
    gq = torch.empty((F, nq, 3), dtype=torch.float64, device="cuda")
    gm = torch.full((F, nm, 3), float("nan"), dtype=torch.float64, device="cuda")
    _native.check(L.pdg_qcmm_potentials(model, F, nq, nm, _native.ptr(dq), _native.ptr(dm), _native.ptr(dc), nk, _native.ptr(kn), 12.0,
                                        _native.ptr(phi), _native.ptr(ws), wb, s), "pdg_qcmm_potentials")
    _native.check(L.pdg_qcmm_gradients(model | flag, F, nq, nm, _native.ptr(dq), _native.ptr(dm), _native.ptr(dc), _native.ptr(dqq), nk,
                                       _native.ptr(kn), 12.0, _native.ptr(gq), _native.ptr(gm), _native.ptr(ws), wb, s), "pdg_qcmm_gradients")
    torch.cuda.synchronize()
    return phi.cpu().numpy(), gq.cpu().numpy(), gm.cpu().numpy()


def test_near_lists_match_full_scan_oracle():
    from pdynamo_mirror_gb300 import NBModelABFS, _native, workloads
    L = _native.load()
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    nq = len(sel)
    frames = workloads.perturbed_frames(X, 5, sigma=0.02, seed=41)
    frames[3, :nq] += np.array([200.0, 0.0, 0.0])           # QC region far from every MM atom: empty near list
    # frame 4: an MM atom placed just inside and one just outside the cutoff of the first QC atom
    frames[4, nq] = frames[4, 0] + np.array([11.999, 0.0, 0.0])
    frames[4, nq + 1] = frames[4, 0] + np.array([0.0, 0.0, 12.0005])
    rng = np.random.default_rng(5)
    qcq = rng.uniform(-0.9, 0.5, size=(5, nq))
    knots_o = O.abfs_knots(8.0, 12.0)
    knots = NBModelABFS(innerCutoff=8.0, outerCutoff=12.0).knots()
    phi, gq, gm = _run(L, 1, frames[:, :nq], frames[:, nq:], Q[nq:], qcq, knots)
    for f in range(5):
        po, gqo, gmo = O.qcmm("abfs", frames[f, :nq], frames[f, nq:], Q[nq:], qcq=qcq[f], knots=knots_o)
        np.testing.assert_allclose(phi[f], po, rtol=0, atol=1e-11, err_msg=str(f))
        np.testing.assert_allclose(gq[f], gqo, rtol=0, atol=1e-11, err_msg=str(f))
        np.testing.assert_allclose(gm[f], gmo, rtol=0, atol=1e-11, err_msg=str(f))
        far = np.all(gmo == 0.0, axis=1)
        assert np.all(gm[f][far] == 0.0)
    assert np.all(phi[3] == 0.0) and np.all(gq[3] == 0.0) and np.all(gm[3] == 0.0)
    # the FP32-pair form over the same near lists
    _, gq32, gm32 = _run(L, 1, frames[:, :nq], frames[:, nq:], Q[nq:], qcq, knots, _native.QCMM_FP32_PAIRS)
    np.testing.assert_allclose(gq32, gq, rtol=0, atol=1e-6)
    np.testing.assert_allclose(gm32, gm, rtol=0, atol=1e-6)


def test_full_model_near_list_holds_every_mm_atom():
    """NBModelFull has no cutoff: every MM atom is near, and the sums equal the oracle's full 1/r sums."""
    from pdynamo_mirror_gb300 import _native, workloads
    L = _native.load()
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=2, n_mm_waters=300, box=25.0)
    nq = len(sel)
    frames = workloads.perturbed_frames(X, 2, sigma=0.02, seed=42)
    qcq = np.random.default_rng(6).uniform(-0.9, 0.5, size=(2, nq))
    phi, gq, gm = _run(L, 0, frames[:, :nq], frames[:, nq:], Q[nq:], qcq, None)
    for f in range(2):
        po, gqo, gmo = O.qcmm("full", frames[f, :nq], frames[f, nq:], Q[nq:], qcq=qcq[f])
        np.testing.assert_allclose(phi[f], po, rtol=0, atol=1e-11)
        np.testing.assert_allclose(gq[f], gqo, rtol=0, atol=1e-11)
        np.testing.assert_allclose(gm[f], gmo, rtol=0, atol=1e-11)
