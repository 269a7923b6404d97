"""Perturbative density steps of the mixed method (csrc/scf.cu density_step_pert): after the first FP64 step of
a frame keeps its base, the later density steps solve the block-diagonalisation equation in the base's
eigenvector basis with FP32 products of small quantities.  Converged energies, gradients and densities against
the plain FP64 method on the same frames (QC/MM water box with the tensor-core purification before: one FP64
step per frame, the rest perturbative, no fallbacks; a water cluster beyond the one-tile purification, whose
early cycles are FP64 steps, some after a perturbative attempt the base could not carry).  Tolerances: energies 1e-8 Hartree (SCF runs
stopped at a 1e-8 density change along different DIIS paths differ by ~1e-9 on the 40-water cluster); gradients
5e-6 Hartree/Bohr (the mixed method takes the sp-sp pair gradient terms in FP32; the gate against the oracle is
1e-5); densities: RMS 2e-8 and any element 5e-7 (two SCF paths that each stop at an RMS density change of 1e-8
differ by about that much)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(Z, frames, method, phi_inputs=None):
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger
    from pdynamo_mirror_gb300.engine import QCEngine
    conv = DIISSCFConverger(**({"densityStep": "purification", "purificationProducts": 6, "purificationSwitch": 1e-5}
                                if method == "mixed" else {}))
    eng = QCEngine("am1", Z[0], Z[1])
    qc = torch.as_tensor(frames, device="cuda").contiguous()
    mm = q = nb = None
    if phi_inputs is not None:
        mm, q, nb = phi_inputs
    r = eng.run(qc, conv, mm, q, nb, gradients=True, warm_start=False)
    T = eng.timings(qc.shape[0])
    assert (r["status"].cpu().numpy() == 0).all()
    return (r["energies"][:, 0].cpu().numpy(), r["qc_gradients"].cpu().numpy(), eng.density.cpu().numpy(),
            r["ncycles"].cpu().numpy(), T)


def _check(Z, frames, phi_inputs=None, tensor_step=True):
    Ef, Gf, Pf, Cf, _ = _run(Z, frames, "fp64", phi_inputs)
    Em, Gm, Pm, Cm, T = _run(Z, frames, "mixed", phi_inputs)
    np.testing.assert_allclose(Em, Ef, rtol=0, atol=1e-8)
    np.testing.assert_allclose(Gm, Gf, rtol=0, atol=5e-6)   # FP32 pair gradient terms in the mixed method
    np.testing.assert_allclose(Pm, Pf, rtol=0, atol=5e-7)
    assert np.sqrt(((Pm - Pf) ** 2).mean(axis=(1, 2))).max() < 2e-8
    assert np.all(T["QC Densities Perturbative Steps"] >= 1)
    if tensor_step:   # purification carries the early cycles: one FP64 step (the base), then no fallback
        assert np.all(T["QC Densities Steps"] == 1) and np.all(T["QC Densities Purification Steps"] >= 1)
        assert np.all(T["QC Densities Perturbative Fallbacks"] == 0)
    else:             # FP64 steps carry the early cycles; each failed perturbative attempt is followed by one
        assert np.all(T["QC Densities Steps"] >= 1 + T["QC Densities Perturbative Fallbacks"] - 1)
    assert np.abs(Cm - Cf).max() <= 2


def test_perturbative_steps_match_fp64_on_the_qcmm_water_box():
    import torch
    from pdynamo_mirror_gb300 import NBModelABFS, workloads
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    frames = workloads.perturbed_frames(X, 8, sigma=0.02, seed=5)
    nq = len(sel)
    mm = torch.as_tensor(frames[:, nq:], device="cuda").contiguous()
    q = torch.as_tensor(Q[nq:], device="cuda")
    _check(([Z[i] for i in sel], charge), frames[:, :nq], (mm, q, NBModelABFS(innerCutoff=8.0, outerCutoff=12.0)))


def test_perturbative_steps_match_fp64_beyond_the_tensor_tile():
    from pdynamo_mirror_gb300 import workloads
    Z, X = workloads.water_cluster(40, seed=9)   # N = 160: FP64 steps until the base, then perturbative steps
    frames = workloads.perturbed_frames(X, 3, sigma=0.02, seed=6)
    _check((list(Z), 0), frames, tensor_step=False)
