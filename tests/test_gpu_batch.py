"""Heterogeneous batches (pdg_batch_*, MoleculeBatch): water clusters of different sizes computed by one
launch per kernel (integrals, the persistent SCF, gradients), against the single-molecule path of the same
library, against the oracle, replayed from a CUDA graph, and under every schedule the autotuner tries.
Tolerances: the accuracy gate |dE| < 1e-6 Hartree, max |dG| < 1e-5 Hartree/Bohr against the oracle; the
batch and single-molecule paths run the same FP64 arithmetic and are compared at 1e-10; with the mixed method
the perturbative density steps' FP32 products follow the CTA shape of the schedule, so the two paths agree to
that method's precision (energies 1e-9 relative, gradients and densities 1e-7 (two SCF paths converged to a 1e-8
density tolerance), SCF cycles within one)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

A2B = 1.0e-10 / 5.291772083e-11
E_TOL, G_TOL = 1.0e-6, 1.0e-5
# repeated sizes share one system; 26 waters (N = 156) is beyond the one-tile purification step and, with two
# CTAs per SM, beyond the shared-memory matrix (FP64 step on the workspace copy)
SIZES = [3, 7, 2, 7, 12, 5, 26, 4]


def _clusters(sizes, seed):
    from pdynamo_mirror_gb300 import workloads
    return [workloads.water_cluster(w, seed=seed + k) for k, w in enumerate(sizes)]


def _converger(step):
    from pdynamo_mirror_gb300 import DIISSCFConverger
    if step == "purification":
        return DIISSCFConverger(densityStep="purification", purificationProducts=6, purificationSwitch=1e-5)
    return DIISSCFConverger()


@pytest.mark.parametrize("step", ["fp64", "purification"])
def test_batch_matches_the_single_molecule_path(step):
    import torch
    from pdynamo_mirror_gb300 import MoleculeBatch
    from pdynamo_mirror_gb300.engine import QCEngine
    mols = _clusters(SIZES, 40)
    conv = _converger(step)
    b = MoleculeBatch("pm3", mols)
    assert len(b._engines) == len(set(SIZES))
    r = b.run(b.coordinates(mols), conv)
    assert (r["status"].cpu().numpy() == 0).all()
    E, G, C = r["energies"].cpu().numpy(), r["gradients"].cpu().numpy(), r["ncycles"].cpu().numpy()
    for k, (Z, X) in enumerate(mols):
        eng = QCEngine("pm3", Z, 0)
        s = eng.run(torch.as_tensor(X[None], device="cuda"), conv, gradients=True, warm_start=False)
        exact = step == "fp64"
        np.testing.assert_allclose(E[k, :7], s["energies"][0, :7].cpu().numpy(), atol=1e-10 if exact else 0.0, rtol=0 if exact else 1e-9)
        # the mixed method's FP32 products round differently in the batch kernel's and the single path's CTA shapes;
        # both stop at the 1e-8 RMS density tolerance, so densities and gradients agree to ~1e-7
        np.testing.assert_allclose(G[b.atom_offsets[k]:b.atom_offsets[k + 1]], s["qc_gradients"][0].cpu().numpy(), atol=1e-10 if exact else 1e-6, rtol=0)
        assert abs(C[k] - int(s["ncycles"][0])) <= (0 if exact else 1)
        np.testing.assert_allclose(b.density(r, k).cpu().numpy(), eng.density[0].cpu().numpy(), atol=1e-10 if exact else 1e-6, rtol=0)


def test_batch_matches_oracle():
    from pdynamo_mirror_gb300 import MoleculeBatch
    mols = _clusters([2, 4, 3, 5], 70)
    b = MoleculeBatch("pm3", mols)
    r = b.run(b.coordinates(mols), _converger("purification"))
    E, G = r["energies"].cpu().numpy(), r["gradients"].cpu().numpy()
    for k, (Z, X) in enumerate(mols):
        ref = O.System(O.Hamiltonian("pm3", list(Z)), list(Z)).energy(X)
        e = E[k, 1] + E[k, 2] + E[k, 3]
        assert abs(e - (ref["eelectronic"] + ref["enuclear"] + ref["baseline"])) < E_TOL
        assert np.abs(G[b.atom_offsets[k]:b.atom_offsets[k + 1]] - ref["gradients"]).max() < G_TOL


def test_graph_replay_matches_direct_calls():
    import torch
    from pdynamo_mirror_gb300 import MoleculeBatch, workloads
    mols = _clusters([6, 3, 9, 4, 6], 90)
    conv = _converger("purification")
    b = MoleculeBatch("pm3", mols)
    xyz = b.coordinates(mols)
    direct = b.run(xyz, conv)
    E0, G0 = direct["energies"].clone(), direct["gradients"].clone()
    g = b.capture(xyz, conv)
    out = g.launch()
    torch.cuda.synchronize()
    assert torch.equal(out["energies"], E0) and torch.equal(out["gradients"], G0)
    # new coordinates written into the captured input buffer: the replay recomputes them
    moved = torch.as_tensor(workloads.perturbed_frames(xyz.cpu().numpy(), 1, sigma=0.02, seed=5)[0], device="cuda")
    out["xyz_bohr"].copy_(moved * A2B)
    g.launch()
    ref = b.run(moved, conv)
    torch.cuda.synchronize()
    assert torch.equal(out["energies"], ref["energies"]) and torch.equal(out["gradients"], ref["gradients"])
    assert not torch.equal(out["energies"], E0)


def test_every_schedule_gives_the_same_results():
    from pdynamo_mirror_gb300 import MoleculeBatch
    from pdynamo_mirror_gb300.batch import SCHEDULES
    mols = _clusters([26, 4, 30, 11, 2, 17], 120)
    conv = _converger("purification")
    b = MoleculeBatch("pm3", mols)
    xyz = b.coordinates(mols)
    ref = None
    for sch in SCHEDULES:
        b.schedule(*sch)
        r = b.run(xyz, conv)
        assert (r["status"].cpu().numpy() == 0).all()
        E, G = r["energies"][:, 0].cpu().numpy(), r["gradients"].cpu().numpy()
        if ref is None:
            ref = (E, G)
        else:
            # the same method, but the FP32 products of the perturbative steps round differently in the 256- and
            # 512-thread CTAs' tile shapes: energies agree to that rounding (~1e-8 Hartree), far inside the 1e-6 gate
            assert np.abs(E - ref[0]).max() < 1e-7
            assert np.abs(G - ref[1]).max() < 1e-6
    times = b.autotune(xyz, conv, repeats=1)
    assert set(times) == set(SCHEDULES) and (b.tuning["best"]["threads"], b.tuning["best"]["ctas_per_sm"]) in ((256, 1), (256, 2), (512, 1))
