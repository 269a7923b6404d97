"""One density step (pdg_density) against numpy's eigendecomposition: the FP64 eigensolve to round-off, the
split-BF16 purification to the accuracy of its partial products (3: ~1e-4, 6: ~3e-6 in max |P - P_exact|,
limited by the FP32 accumulation)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _fock_cases():
    from pdynamo_mirror_gb300 import workloads
    out = []
    for nw, seed in ((16, 0), (22, 3)):   # N = 96 and N = 132 (> 128: the second tensor-core tile)
        Z, X = workloads.water_cluster(nw, seed=seed)
        osys = O.System(O.Hamiltonian("am1", list(Z)), list(Z), charge=0)
        r = osys.energy(X, gradients=False)
        Fp, _ = osys.fock(X, r["density"])
        out.append((Z, Fp))
    return out


@pytest.mark.parametrize("case", [0, 1])
@pytest.mark.parametrize("step,tol", [(0, 1e-9), (3, 2e-4), (6, 1e-5)])
def test_density_step_matches_exact_projector(case, step, tol):
    import torch
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, Fp = _fock_cases()[case]
    eng = QCEngine("am1", Z, 0)
    N, nocc = eng.n_basis, eng.n_occupied
    F = np.zeros((N, N)); k = 0
    for i in range(N):
        for j in range(i + 1):
            F[i, j] = F[j, i] = Fp[k]; k += 1
    w, V = np.linalg.eigh(F)
    Pex = 2.0 * V[:, :nocc] @ V[:, :nocc].T
    P, en, st = eng.density_step(torch.as_tensor(F[None], device="cuda"), step)
    assert int(st[0].item()) == 0
    err = np.abs(P[0].cpu().numpy() - Pex).max()
    assert err < tol, (case, step, err)
