"""Learned start density (csrc/guess.cu): the MLP's backward kernels against torch autograd on the same
weights, and a small training run whose guess is several times closer to the converged density than the
diagonal guess on held-out frames, while the SCF started from it converges to the same energies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _water_box_engine(n_frames, seed, sigma=0.05):
    import torch
    from pdynamo_mirror_gb300 import NBModelABFS, workloads
    from pdynamo_mirror_gb300.engine import QCEngine
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    frames = workloads.perturbed_frames(X, n_frames, sigma=sigma, seed=seed)
    nq = len(sel)
    eng = QCEngine("am1", [Z[i] for i in sel], charge)
    qc = torch.as_tensor(frames[:, :nq], device="cuda").contiguous()
    mm = torch.as_tensor(frames[:, nq:], device="cuda").contiguous()
    q = torch.as_tensor(Q[nq:], device="cuda")
    return eng, qc, mm, q, NBModelABFS()


def test_mlp_backward_matches_autograd():
    import torch
    from pdynamo_mirror_gb300 import LearnedDensityGuess
    eng, qc, mm, q, nb = _water_box_engine(4, seed=3)
    g = LearnedDensityGuess(eng, seed=1)
    b, rows_ptr, xyz = g._forward(qc, None, True)
    rows = int(b["offsets"][-1].item())
    x = b["x"][:rows].clone()
    Ws = [p["w"].float().clone().requires_grad_(True) for p in g.params]
    bs = [p["bm"].clone().requires_grad_(True) for p in g.params]
    h = x
    for li, p in enumerate(g.params):
        z = h @ Ws[li].T + bs[li]
        h = torch.nn.functional.silu(z) if p["act"] else z
    np.testing.assert_allclose(h.detach().cpu().numpy(), b["h2"][:rows].cpu().numpy(), rtol=1e-4, atol=1e-5)
    dy = torch.randn_like(h)
    (h * dy).sum().backward()
    # kernel backward with the same dy, learning rate 0 (gradients only): use the segment partials
    from pdynamo_mirror_gb300 import _native
    dz = torch.zeros((b["rows"], 16), dtype=torch.float32, device="cuda")
    dz[:rows] = dy
    for li in (2, 1, 0):
        p = g.params[li]
        hin = b["x"] if li == 0 else b["h%d" % (li - 1)]
        part = torch.empty(4 * p["n"] * (p["k"] + 1), dtype=torch.float32, device="cuda")
        dzin = torch.empty((b["rows"], p["k"]), dtype=torch.float32, device="cuda") if li > 0 else None
        _native.check(g.L.pdg_mlp_backward(b["rows"], rows_ptr, p["n"], p["k"], _native.ptr(dz), _native.ptr(p["w"]),
                                           _native.ptr(b["z%d" % (li - 1)]) if li > 0 else None, _native.ptr(hin), _native.ptr(dzin),
                                           4, _native.ptr(part), g._sh()), "backward")
        gw = part.view(4, p["n"], p["k"] + 1).sum(0)
        np.testing.assert_allclose(gw[:, :p["k"]].cpu().numpy(), Ws[li].grad.cpu().numpy(), rtol=2e-3, atol=2e-3)
        np.testing.assert_allclose(gw[:, p["k"]].cpu().numpy(), bs[li].grad.cpu().numpy(), rtol=2e-3, atol=2e-3)
        dz = dzin


def test_learned_guess_is_closer_than_the_diagonal_guess_and_keeps_the_energies():
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, LearnedDensityGuess
    eng, qc, mm, q, nb = _water_box_engine(160, seed=11)
    conv = DIISSCFConverger()
    ref = eng.run(qc, conv, mm, q, nb, gradients=False, warm_start=False)
    assert (ref["status"].cpu().numpy() == 0).all()
    P, phi = eng.density.clone(), ref["phi"].clone()
    tr, te = slice(0, 128), slice(128, 160)
    g = LearnedDensityGuess(eng, seed=0)
    hist = g.fit(qc[tr].contiguous(), phi[tr].contiguous(), P[tr].contiguous(), epochs=40, batch=16, lr=1e-3)
    assert hist[-1] < 0.2 * hist[0]
    N = eng.n_basis
    Pg = g.predict(qc[te].contiguous(), phi[te].contiguous())
    diag = torch.zeros_like(Pg)
    diag.diagonal(dim1=1, dim2=2).fill_(2.0 * eng.n_occupied / N)
    err = lambda A: ((A - P[te]) ** 2).sum(dim=(1, 2)).sqrt().mean().item() / N
    assert err(Pg) < 0.25 * err(diag), (err(Pg), err(diag))
    qt, mt = qc[te].contiguous(), mm[te].contiguous()
    base = eng.run(qt, conv, mt, q, nb, gradients=False, warm_start=False)
    learned = eng.run(qt, conv, mt, q, nb, gradients=False, warm_start=False, guess=g)
    assert (learned["status"].cpu().numpy() == 0).all()
    e0, e1 = base["energies"][:, 0].cpu().numpy(), learned["energies"][:, 0].cpu().numpy()
    assert np.abs(e1 - e0).max() < 1e-8
    # held-out validation: the guess stays on only where it saves cycles; when off, the diagonal guess runs
    v = g.validate(qt, conv, mt, q, nb)
    assert v["enabled"] == (v["mean_scf_cycles_learned_guess"] < v["mean_scf_cycles_diagonal_guess"])
    assert v["max_abs_dE_hartree"] < 1e-8
    g.enabled = False
    off = eng.run(qt, conv, mt, q, nb, gradients=False, warm_start=False, guess=g)
    assert (off["ncycles"] == base["ncycles"]).all()
    assert np.abs(off["energies"][:, 0].cpu().numpy() - e0).max() < 1e-12
