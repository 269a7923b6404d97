"""Learned SCF start density: a per-atom-pair MLP trained on densities the SCF itself converged.

The kernels are in csrc/guess.cu (features, MLP forward / backward / Adam, assembly, loss); this class owns
the parameters (FP32 masters, BF16 copies, Adam moments) and the buffers, and drives training and
prediction on one CUDA stream.  The model is tied to a QC region's elements (the features carry element
one-hots and environment functions of the first two element types) but not to its size.  No counterpart
in the reference: pDynamo starts the SCF from the diagonal guess (QCOnePDM.c:280) or from the previous
density (pMolecule.QCModel.pyx:153).
"""

import ctypes

import numpy as np
import torch

from . import _native

IN, H, OUT = 64, 256, 16
LAYERS = ((IN, H, 1), (H, H, 1), (H, OUT, 0))   # (inputs, outputs, SiLU)


class LearnedDensityGuess:
    def __init__(self, engine, seed=0):
        self.eng = engine
        self.L = engine.L
        dev = engine.device
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.params = []
        for k, n, act in LAYERS:
            bound = (6.0 / (k + n)) ** 0.5 * (0.1 if act == 0 else 1.0)
            wm = ((torch.rand((n, k), generator=g, dtype=torch.float32) * 2 - 1) * bound).to(dev)
            self.params.append({"k": k, "n": n, "act": act, "wm": wm, "bm": torch.zeros(n, dtype=torch.float32, device=dev),
                                "w": wm.to(torch.bfloat16).contiguous(),
                                "m1": torch.zeros(n * (k + 1), dtype=torch.float32, device=dev),
                                "m2": torch.zeros(n * (k + 1), dtype=torch.float32, device=dev)})
        self.step = 0
        self._buf = {}
        self.enabled = True       # False after validate() found no cycles saved: the SCF falls back to the diagonal guess
        self.validation = None

    # -- buffers
    def _buffers(self, F):
        if F not in self._buf:
            dev, na, npairs = self.eng.device, self.eng.n_atoms, self.eng.n_pairs
            rows = max(F * npairs, 1)
            b = {"env": torch.empty(F * na * 8, dtype=torch.float32, device=dev),
                 "count": torch.empty(F, dtype=torch.int32, device=dev),
                 "offsets": torch.empty(F + 1, dtype=torch.int32, device=dev),
                 "x": torch.empty((rows, IN), dtype=torch.float32, device=dev),
                 "row_frame": torch.empty(rows, dtype=torch.int32, device=dev),
                 "row_pair": torch.empty(rows, dtype=torch.int32, device=dev),
                 "rows": rows}
            for li, (k, n, act) in enumerate(LAYERS):
                b["z%d" % li] = torch.empty((rows, n), dtype=torch.float32, device=dev)
                b["h%d" % li] = torch.empty((rows, n), dtype=torch.float32, device=dev)
            self._buf[F] = b
        return self._buf[F]

    def _sh(self):
        return _native.stream_handle(torch.cuda.current_stream(self.eng.device))

    def _forward(self, qc_xyz, phi, train):
        F = qc_xyz.shape[0]
        b = self._buffers(F)
        xyz = qc_xyz.contiguous()
        P_ = _native.ptr
        _native.check(self.L.pdg_guess_features(self.eng.handle, F, P_(xyz), P_(phi), P_(b["env"]), P_(b["count"]), P_(b["offsets"]),
                                                P_(b["x"]), P_(b["row_frame"]), P_(b["row_pair"]), self._sh()), "pdg_guess_features")
        rows_ptr = ctypes.c_void_p(b["offsets"].data_ptr() + 4 * F)
        x = b["x"]
        for li, p in enumerate(self.params):
            _native.check(self.L.pdg_mlp_forward(b["rows"], rows_ptr, p["k"], p["n"], P_(x), P_(p["w"]), P_(p["bm"]),
                                                 P_(b["z%d" % li]) if train else None, P_(b["h%d" % li]), p["act"], self._sh()),
                          "pdg_mlp_forward")
            x = b["h%d" % li]
        return b, rows_ptr, xyz

    def predict(self, qc_xyz, phi=None):
        """Start densities [F, N, N] (device float64) for QC coordinates [F, n, 3] in Angstrom."""
        F, N = qc_xyz.shape[0], self.eng.n_basis
        b, rows_ptr, xyz = self._forward(qc_xyz, phi, False)
        P = torch.empty((F, N, N), dtype=torch.float64, device=self.eng.device)
        _native.check(self.L.pdg_guess_assemble(self.eng.handle, F, _native.ptr(xyz), _native.ptr(b["offsets"]), _native.ptr(b["row_pair"]),
                                                _native.ptr(b["h2"]), _native.ptr(P), self._sh()), "pdg_guess_assemble")
        return P

    def train_step(self, qc_xyz, phi, target, lr=1e-3, segments=16):
        """One Adam step on the squared error of the assembled start densities against target [F, N, N].
        Returns the loss per frame (device)."""
        F, N = qc_xyz.shape[0], self.eng.n_basis
        b, rows_ptr, xyz = self._forward(qc_xyz, phi, True)
        P_ = _native.ptr
        P = torch.empty((F, N, N), dtype=torch.float64, device=self.eng.device)
        _native.check(self.L.pdg_guess_assemble(self.eng.handle, F, P_(xyz), P_(b["offsets"]), P_(b["row_pair"]), P_(b["h2"]), P_(P),
                                                self._sh()), "pdg_guess_assemble")
        dy = torch.empty((b["rows"], OUT), dtype=torch.float32, device=self.eng.device)
        loss = torch.empty(F, dtype=torch.float64, device=self.eng.device)
        _native.check(self.L.pdg_guess_loss(self.eng.handle, F, P_(xyz), P_(b["offsets"]), P_(b["row_pair"]), P_(P), P_(target.contiguous()),
                                            P_(dy), P_(loss), self._sh()), "pdg_guess_loss")
        self.step += 1
        scale = 1.0 / F
        dz = dy
        for li in (2, 1, 0):
            p = self.params[li]
            hin = b["x"] if li == 0 else b["h%d" % (li - 1)]
            part = torch.empty(segments * p["n"] * (p["k"] + 1), dtype=torch.float32, device=self.eng.device)
            dzin = torch.empty((b["rows"], p["k"]), dtype=torch.float32, device=self.eng.device) if li > 0 else None
            _native.check(self.L.pdg_mlp_backward(b["rows"], rows_ptr, p["n"], p["k"], P_(dz), P_(p["w"]),
                                                  P_(b["z%d" % (li - 1)]) if li > 0 else None, P_(hin), P_(dzin), segments, P_(part),
                                                  self._sh()), "pdg_mlp_backward")
            _native.check(self.L.pdg_mlp_adam(p["n"], p["k"], segments, P_(part), ctypes.c_float(scale), P_(p["wm"]), P_(p["bm"]),
                                              P_(p["m1"]), P_(p["m2"]), P_(p["w"]), ctypes.c_float(lr), ctypes.c_float(0.9),
                                              ctypes.c_float(0.999), self.step, self._sh()), "pdg_mlp_adam")
            dz = dzin
        return loss

    def fit(self, qc_frames, phis, densities, epochs=100, batch=32, lr=1e-3, seed=0):
        """Train on frames [F, n, 3] (device, Angstrom), potentials [F, n] or None, converged densities
        [F, N, N].  Returns the mean loss per frame of each epoch."""
        rng = np.random.default_rng(seed)
        F = qc_frames.shape[0]
        hist = []
        for ep in range(epochs):
            order = rng.permutation(F)
            tot = 0.0
            for s0 in range(0, F - batch + 1, batch):
                idx = torch.as_tensor(order[s0:s0 + batch], device=self.eng.device)
                ph = None if phis is None else phis[idx].contiguous()
                loss = self.train_step(qc_frames[idx].contiguous(), ph, densities[idx], lr=lr)
                tot += float(loss.sum())
            hist.append(tot / F)
        return hist

    def validate(self, qc_xyz, converger, mm_xyz=None, mm_charges=None, nbmodel=None):
        """Held-out check, the converged SCF deciding: run the frames [F, n, 3] cold from the standard start (the
        diagonal guess, or the shared base's density with a sharedBase converger whose base exists; the
        "diagonal_guess" figures then describe that start) and from this guess, compare the mean SCF cycles and the
        energies, and keep the guess enabled only if it saved cycles (else the standard start is the fallback).
        Returns the figures as a dict."""
        eng = self.eng
        self.enabled = True
        std = eng.run(qc_xyz, converger, mm_xyz, mm_charges, nbmodel, gradients=False, warm_start=False)
        e_std, c_std = std["energies"].sum(1).clone(), float(std["ncycles"].double().mean())
        P_std, phi = eng.density.clone(), std["phi"]
        N = eng.n_basis
        P_g = self.predict(qc_xyz, phi)
        diag = torch.zeros_like(P_g)
        diag.diagonal(dim1=1, dim2=2).fill_(2.0 * eng.n_occupied / N)
        err = lambda A: float(((A - P_std) ** 2).sum(dim=(1, 2)).sqrt().mean()) / N
        lrn = eng.run(qc_xyz, converger, mm_xyz, mm_charges, nbmodel, gradients=False, warm_start=False, guess=self)
        c_lrn = float(lrn["ncycles"].double().mean())
        ok = bool((std["status"] == 0).all()) and bool((lrn["status"] == 0).all())
        self.enabled = ok and c_lrn < c_std
        shared = bool(getattr(converger, "sharedBase", False)) and getattr(eng, "_base", None) is not None
        self.validation = {"frames": int(qc_xyz.shape[0]), "standard_start": "shared base density" if shared else "diagonal guess",
                           "rms_error_learned": err(P_g), "rms_error_diagonal": err(diag),
                           "mean_scf_cycles_diagonal_guess": c_std, "mean_scf_cycles_learned_guess": c_lrn,
                           "iterations_saved": c_std - c_lrn,
                           "max_abs_dE_hartree": float((lrn["energies"].sum(1) - e_std).abs().max()),
                           "enabled": self.enabled}
        return self.validation

    def state_dict(self):
        return {"w%d" % i: p["wm"].cpu().numpy() for i, p in enumerate(self.params)} | \
               {"b%d" % i: p["bm"].cpu().numpy() for i, p in enumerate(self.params)}

    def load_state_dict(self, d):
        for i, p in enumerate(self.params):
            p["wm"].copy_(torch.as_tensor(d["w%d" % i]))
            p["bm"].copy_(torch.as_tensor(d["b%d" % i]))
            p["w"].copy_(p["wm"].to(torch.bfloat16))


class LinearResponseGuess:
    """Start density from a linear model of the converged density in the geometry and the environment (not in the
    reference): P(x, phi) ~ P_mean + (f - f_mean) J over the packed lower triangle of P, with features f = the QC
    atoms' Cartesian coordinates (A) and the QC/MM potentials at them (a.u.), J by ridge regression on standardised
    features over densities the SCF itself converged.  It learns the density's linear response to the displacements
    and to the MM field around the frames it was trained on (MD or sampled frames of one QC region in a fixed
    frame of reference).  The sums of the normal equations stay on the device in FP64, so that training can go on
    batch by batch; prediction is one FP32 GEMM (features x J) and the unpacking.  The prediction enters the SCF as
    a start density (use_density 1), DIIS history included.  validate() keeps it on only where it saves SCF cycles."""

    start_mode = 1

    def __init__(self, engine, ridge=1.0):
        self.eng = engine
        self.ridge = float(ridge)
        dev = engine.device
        N = engine.n_basis
        self.N = N
        il = torch.tril_indices(N, N, device=dev)
        self._lower, self._upper = il[0] * N + il[1], il[1] * N + il[0]
        nf = 4 * engine.n_atoms
        self.nf, self.npk = nf, il.shape[1]
        self.n = 0
        self._sf = torch.zeros(nf, dtype=torch.float64, device=dev)
        self._sp = torch.zeros(self.npk, dtype=torch.float64, device=dev)
        self._sff = torch.zeros((nf, nf), dtype=torch.float64, device=dev)
        self._sfp = torch.zeros((nf, self.npk), dtype=torch.float64, device=dev)
        self.J = self.f_mean = self.p_mean = None
        self.enabled = False
        self.validation = None

    def _features(self, qc_xyz, phi):
        F = qc_xyz.shape[0]
        x = qc_xyz.reshape(F, -1).to(torch.float64)
        p = phi.to(torch.float64) if phi is not None else torch.zeros((F, self.eng.n_atoms), dtype=torch.float64, device=x.device)
        return torch.cat([x, p], 1)

    def fit(self, qc_xyz, phi, P):
        """Add frames (qc_xyz [F, n, 3] A, phi [F, n] or None, converged densities P [F, N, N]) to the normal
        equations and solve them; the model is then enabled until validate() says otherwise."""
        f = self._features(qc_xyz, phi)
        p = P.reshape(P.shape[0], -1)[:, self._lower].to(torch.float64)
        self.n += f.shape[0]
        self._sf += f.sum(0)
        self._sp += p.sum(0)
        self._sff += f.T @ f
        self._sfp += f.T @ p
        n = float(self.n)
        fm, pm = self._sf / n, self._sp / n
        C = self._sff / n - torch.outer(fm, fm)
        S = self._sfp / n - torch.outer(fm, pm)
        sd = torch.sqrt(torch.clamp(torch.diagonal(C), min=1e-30))
        Cs = C / torch.outer(sd, sd) + (self.ridge / n) * torch.eye(self.nf, dtype=torch.float64, device=C.device)
        # the (4 N_A)^2 system is solved on the host (training only; no device solver library needed)
        Js = np.linalg.solve(Cs.cpu().numpy(), (S / sd[:, None]).cpu().numpy())
        self.J = (torch.from_numpy(Js).to(C.device) / sd[:, None]).to(torch.float32).contiguous()
        self.f_mean, self.p_mean = fm, pm
        self.enabled = True
        return self

    def predict(self, qc_xyz, phi=None):
        """Start densities [F, N, N] (FP64) for frames qc_xyz [F, n, 3] (A) with potentials phi [F, n]."""
        F = qc_xyz.shape[0]
        d = (self._features(qc_xyz, phi) - self.f_mean).to(torch.float32)
        pk = torch.mm(d, self.J).to(torch.float64) + self.p_mean
        P = torch.empty((F, self.N * self.N), dtype=torch.float64, device=pk.device)
        P[:, self._lower] = pk
        P[:, self._upper] = pk
        return P.view(F, self.N, self.N)

    def validate(self, qc_xyz, converger, mm_xyz=None, mm_charges=None, nbmodel=None):
        """Held-out check, the converged SCF deciding: the frames from the standard start (the diagonal guess, or
        the shared base's density with a sharedBase converger whose base exists) and from this guess; the guess
        stays enabled only if it saves SCF cycles.  Returns the figures as a dict."""
        eng = self.eng
        self.enabled = True
        std = eng.run(qc_xyz, converger, mm_xyz, mm_charges, nbmodel, gradients=False, warm_start=False)
        e_std, c_std = std["energies"].sum(1).clone(), float(std["ncycles"].double().mean())
        P_std, phi = eng.density.clone(), std["phi"]
        N = eng.n_basis
        P_g = self.predict(qc_xyz, phi)
        err = lambda A: float(((A - P_std) ** 2).sum(dim=(1, 2)).sqrt().mean()) / N
        lrn = eng.run(qc_xyz, converger, mm_xyz, mm_charges, nbmodel, gradients=False, warm_start=False, guess=self)
        c_lrn = float(lrn["ncycles"].double().mean())
        ok = bool((std["status"] == 0).all()) and bool((lrn["status"] == 0).all())
        self.enabled = ok and c_lrn < c_std
        shared = bool(getattr(converger, "sharedBase", False)) and getattr(eng, "_base", None) is not None
        self.validation = {"model": "linear response (ridge regression on QC coordinates and QC/MM potentials)",
                           "training_frames": self.n, "frames": int(qc_xyz.shape[0]),
                           "standard_start": "shared base density" if shared else "diagonal guess",
                           "rms_error_learned": err(P_g), "mean_scf_cycles_standard_start": c_std,
                           "mean_scf_cycles_learned_guess": c_lrn, "iterations_saved": c_std - c_lrn,
                           "max_abs_dE_hartree": float((lrn["energies"].sum(1) - e_std).abs().max()),
                           "enabled": self.enabled}
        return self.validation
