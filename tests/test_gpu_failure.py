"""Failure detection without a GPU fault: the per-frame error statuses of the SCF kernel, driven by data made on
the host, and the bounded tensor-core completion wait, driven by a barrier that nothing arrives on.

* A NaN in one frame's QC/MM potentials (made on the host; the potentials enter only the Fock diagonal and the
  q.phi energy, no index is derived from them) stops that frame's SCF at its first Fock build with PDG_NAN; the other
  frames of the same launch converge to the oracle's energies (|dE| < 1e-6 Hartree) and the device stays usable.
* pdg_tc_selftest with kprod = 0 waits a few polls on an mbarrier that no tensor-core operation will ever signal
  (none is issued) and reports status 1 instead of hanging; a real product runs correctly afterwards.
* The Python surface raises SCFNotConverged (the reference's ValueError, pMolecule.QCModel.pyx:177) naming each
  failing frame's status.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KJ = 2625.5


def test_nan_potential_stops_only_its_frame():
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, _native, workloads
    from pdynamo_mirror_gb300.engine import ANGSTROMS_TO_BOHRS, QCEngine
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1, n_mm_waters=800, box=30.0)
    nq = len(sel)
    frames = workloads.perturbed_frames(X, 4, sigma=0.02, seed=31)
    knots = O.abfs_knots(8.0, 12.0)
    phi = np.stack([O.qcmm("abfs", fr[:nq], fr[nq:], Q[nq:], knots=knots)[0] for fr in frames])
    bad = 2
    phi[bad, 5] = np.nan
    eng = QCEngine("am1", Z[:nq], charge)
    F, N = len(frames), eng.n_basis
    dev = "cuda"
    xyz = torch.as_tensor(frames[:, :nq] * ANGSTROMS_TO_BOHRS, dtype=torch.float64, device=dev).contiguous()
    d_phi = torch.as_tensor(phi, dtype=torch.float64, device=dev).contiguous()
    P = torch.empty((F, N, N), dtype=torch.float64, device=dev)
    E = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=dev)
    G = torch.empty((F, nq, 3), dtype=torch.float64, device=dev)
    C = torch.empty((F, nq), dtype=torch.float64, device=dev)
    st = torch.full((F,), -1, dtype=torch.int32, device=dev)
    nc = torch.empty(F, dtype=torch.int32, device=dev)
    ws = eng.workspace(F)
    opts = DIISSCFConverger().options()
    import ctypes
    _native.check(eng.L.pdg_energy_gradients(eng.handle, F, _native.ptr(xyz), _native.ptr(d_phi), ctypes.byref(opts), _native.ptr(P), 0,
                                             _native.ptr(E), _native.ptr(G), _native.ptr(C), _native.ptr(st), _native.ptr(nc),
                                             _native.ptr(ws), ws.numel(), _native.stream_handle(torch.cuda.current_stream())),
                  "pdg_energy_gradients")
    torch.cuda.synchronize()
    status = st.cpu().numpy()
    assert status[bad] == _native.PDG_NAN
    assert (np.delete(status, bad) == _native.PDG_OK).all()
    En = E.cpu().numpy()
    ham = O.Hamiltonian("am1", list(Z[:nq]))
    for f in range(F):
        if f == bad:
            continue
        r = O.System(ham, list(Z[:nq]), charge=charge).energy(frames[f][:nq], phi=phi[f], gradients=False)
        assert abs(En[f, 0] - (r["eelectronic"] + r["eqcmm"])) < 1e-6, f
    # the device is still usable: the same frames without the NaN all converge
    out = eng.run(torch.as_tensor(frames[:, :nq], dtype=torch.float64, device=dev).contiguous(), DIISSCFConverger(),
                  gradients=False, warm_start=False)
    assert (out["status"].cpu().numpy() == _native.PDG_OK).all()


@pytest.mark.parametrize("limit", [1, 4, 64])
def test_bounded_tensor_wait_reports_timeout(limit):
    import torch
    from pdynamo_mirror_gb300 import _native
    L = _native.load()
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _native.check(L.pdg_tc_selftest(0, 0, limit, None, None, _native.ptr(st), _native.stream_handle(torch.cuda.current_stream())),
                  "pdg_tc_selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == 1
    # a real product on the same context afterwards
    n = 40
    rng = np.random.default_rng(1)
    X = rng.uniform(0.0, 0.1, (n, n)).astype(np.float32)
    X = 0.5 * (X + X.T)
    x = torch.as_tensor(X, device="cuda")
    c = torch.empty_like(x)
    _native.check(L.pdg_tc_selftest(n, 6, 0, _native.ptr(x), _native.ptr(c), _native.ptr(st),
                                    _native.stream_handle(torch.cuda.current_stream())), "pdg_tc_selftest")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = X.astype(np.float64) @ X.astype(np.float64)
    assert np.abs(c.cpu().numpy() - ref).max() < 1e-5 * np.abs(ref).max()
