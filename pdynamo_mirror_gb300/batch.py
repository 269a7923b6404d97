"""MoleculeBatch: independent molecules of different sizes computed together on one GPU.

One launch per kernel covers the whole batch: pair integrals and H, a persistent SCF kernel whose CTAs take
molecules from a queue largest first (so the longest SCFs start first and the smallest fill the tail), and
the gradients.  ``capture`` records that sequence once as a CUDA graph on fixed buffers; ``autotune`` times
the SCF schedules (the 256- or 512-thread SCF variant, CTAs per SM and so the shared memory each CTA may plan
for, and the queue order) on the batch itself and keeps the fastest.  The reference evaluates one molecule per ``QCModel.Energy`` call
(pMolecule.QCModel.pyx:146-185); the per-molecule results here are the same quantities.
"""

import ctypes

import numpy as np
import torch

from . import _native
from .engine import GRADIENT_TO_KJ_PER_A, HARTREES_TO_KJ, QCEngine, require_cuda
from .parameters import ANGSTROMS_TO_BOHRS

# (threads per SCF CTA, SCF CTAs per SM, queue order: 0 largest first, 1 item order)
SCHEDULES = ((256, 2, 0), (256, 1, 0), (512, 1, 0), (256, 2, 1))


class BatchGraph:
    """A captured batch evaluation: launch() replays it; the result tensors are overwritten each time."""

    def __init__(self, batch, handle, buffers):
        self.batch, self.handle, self.buffers = batch, handle, buffers

    def launch(self, stream=None):
        st = stream or torch.cuda.current_stream(self.batch.device)
        _native.check(self.batch.L.pdg_graph_launch(self.handle, _native.stream_handle(st)), "pdg_graph_launch")
        return self.buffers

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.batch.L.pdg_graph_destroy(self.handle)
        except Exception:
            pass


class MoleculeBatch:
    """molecules: a list of atomic-number sequences (or (atomic numbers, coordinates) pairs, whose
    coordinates are ignored here); charges: one total charge per molecule (default 0)."""

    def __init__(self, hamiltonian, molecules, charges=None, device=None):
        require_cuda()
        self.L = _native.load()
        self.device = torch.device(device or "cuda")
        mols = [m[0] if isinstance(m, tuple) else m for m in molecules]
        charges = [0] * len(mols) if charges is None else [int(c) for c in charges]
        if len(charges) != len(mols):
            raise ValueError("one charge per molecule")
        self._engines = {}
        items = []
        for Z, q in zip(mols, charges):
            key = (tuple(int(z) for z in Z), q)
            if key not in self._engines:
                self._engines[key] = QCEngine(hamiltonian, key[0], q, self.device)
            items.append(self._engines[key])
        self.items = items
        self.n = len(items)
        arr = (ctypes.c_void_p * self.n)(*[e.handle.value for e in items])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self.L.pdg_batch_create(arr, self.n, ctypes.byref(h)), "pdg_batch_create")
        self.handle = h
        self.n_atoms = [e.n_atoms for e in items]
        self.n_basis = [e.n_basis for e in items]
        self.atom_offsets = np.concatenate([[0], np.cumsum(self.n_atoms)]).astype(np.int64)
        self.density_offsets = np.concatenate([[0], np.cumsum([N * N for N in self.n_basis])]).astype(np.int64)
        self.ws = torch.empty(int(self.L.pdg_batch_workspace_bytes(h)), dtype=torch.uint8, device=self.device)
        self.tuning = None

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.L.pdg_batch_destroy(self.handle)
        except Exception:
            pass

    # -- schedule
    def info(self):
        n, na, gr, th, sm, ti = (ctypes.c_int() for _ in range(6))
        nd = ctypes.c_longlong()
        _native.check(self.L.pdg_batch_info(self.handle, ctypes.byref(n), ctypes.byref(na), ctypes.byref(nd), ctypes.byref(gr),
                                            ctypes.byref(th), ctypes.byref(sm), ctypes.byref(ti)), "pdg_batch_info")
        return {"items": n.value, "atoms": na.value, "density_doubles": nd.value, "scf_ctas": gr.value, "scf_threads": th.value,
                "scf_shared_bytes": sm.value, "tensor_items": ti.value}

    def schedule(self, threads=256, ctas_per_sm=2, order=0):
        _native.check(self.L.pdg_batch_schedule(self.handle, int(threads), int(ctas_per_sm), int(order)), "pdg_batch_schedule")

    # -- buffers and calls
    def coordinates(self, frames):
        """Concatenate per-molecule coordinates [n_k, 3] (Angstrom) into one device tensor [sum n_k, 3]."""
        X = np.concatenate([np.asarray(f[1] if isinstance(f, tuple) else f, dtype=np.float64).reshape(-1, 3) for f in frames])
        if X.shape[0] != self.atom_offsets[-1]:
            raise ValueError("coordinates do not match the batch's atoms")
        return torch.as_tensor(X, device=self.device)

    def _buffers(self, gradients):
        dev, n, na = self.device, self.n, int(self.atom_offsets[-1])
        return {"density": torch.empty(int(self.density_offsets[-1]), dtype=torch.float64, device=dev),
                "energies": torch.empty((n, _native.NENERGY), dtype=torch.float64, device=dev),
                "gradients": torch.empty((na, 3), dtype=torch.float64, device=dev) if gradients else None,
                "charges": torch.empty(na, dtype=torch.float64, device=dev),
                "status": torch.empty(n, dtype=torch.int32, device=dev),
                "ncycles": torch.empty(n, dtype=torch.int32, device=dev)}

    def _args(self, xyz_bohr, converger, b, use_density=0):
        P_ = _native.ptr
        opts = converger.options()
        return (self.handle, P_(xyz_bohr), None, ctypes.byref(opts), P_(b["density"]), int(use_density), P_(b["energies"]),
                P_(b["gradients"]), P_(b["charges"]), P_(b["status"]), P_(b["ncycles"]), P_(self.ws), self.ws.numel()), opts

    def run(self, xyz, converger, gradients=True, buffers=None):
        """xyz [sum n_k, 3] device float64 in Angstrom.  Returns the device buffers: energies [n, NENERGY] and
        gradients [sum n_k, 3] in Hartree and Hartree/Bohr, Lowdin charges, status, SCF cycles, densities."""
        b = buffers or self._buffers(gradients)
        b["xyz_bohr"] = (xyz * ANGSTROMS_TO_BOHRS).contiguous()
        args, opts = self._args(b["xyz_bohr"], converger, b)
        _native.check(self.L.pdg_batch_energy_gradients(*args, _native.stream_handle(torch.cuda.current_stream(self.device))),
                      "pdg_batch_energy_gradients")
        return b

    def capture(self, xyz, converger, gradients=True):
        """Capture one evaluation on fixed buffers into a CUDA graph (BatchGraph); replays recompute from
        the coordinates in the returned buffers' "xyz_bohr"."""
        b = self._buffers(gradients)
        b["xyz_bohr"] = (xyz * ANGSTROMS_TO_BOHRS).contiguous()
        args, opts = self._args(b["xyz_bohr"], converger, b)
        g = ctypes.c_void_p()
        torch.cuda.synchronize(self.device)
        _native.check(self.L.pdg_batch_graph_create(*args, ctypes.byref(g)), "pdg_batch_graph_create")
        return BatchGraph(self, g, b)

    def autotune(self, xyz, converger, gradients=True, repeats=2, schedules=SCHEDULES):
        """Time each SCF schedule on this batch (CUDA events, after one untimed call) and keep the fastest.
        Returns {schedule: ms} and leaves the best schedule set."""
        times = {}
        b = self._buffers(gradients)
        st = torch.cuda.current_stream(self.device)
        for sch in schedules:
            self.schedule(*sch)
            self.run(xyz, converger, gradients, b)
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(st)
            for _ in range(repeats):
                self.run(xyz, converger, gradients, b)
            t1.record(st)
            t1.synchronize()
            times[sch] = t0.elapsed_time(t1) / repeats
        best = min(times, key=times.get)
        self.schedule(*best)
        self.tuning = {"schedules_ms": {"%d_threads_%d_ctas_per_sm_order_%d" % k: v for k, v in times.items()},
                       "best": {"threads": best[0], "ctas_per_sm": best[1], "order": "largest first" if best[2] == 0 else "item order"}}
        return times

    def timings(self):
        """Per-molecule SCF phase timings of the last call, as {name: array [n]} (names as QCEngine.timings)."""
        out = torch.empty((self.n, len(_native.TIMERS)), dtype=torch.float64, device=self.device)
        _native.check(self.L.pdg_batch_timings(self.handle, _native.ptr(self.ws), self.ws.numel(), _native.ptr(out),
                                               _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_batch_timings")
        t = out.cpu().numpy()
        return {name: t[:, k] for k, name in enumerate(_native.TIMERS)}

    # -- results
    def results(self, b):
        """Host results: Pure QC energies (kJ/mol) [n], gradients (kJ/mol/A) per molecule, status, cycles."""
        E = b["energies"].cpu().numpy()
        pure = HARTREES_TO_KJ * (E[:, _native.EN_ELECTRONIC] + E[:, _native.EN_NUCLEAR] + E[:, _native.EN_BASELINE])
        G = None
        if b.get("gradients") is not None:
            g = b["gradients"].cpu().numpy() * GRADIENT_TO_KJ_PER_A
            G = [g[self.atom_offsets[k]:self.atom_offsets[k + 1]] for k in range(self.n)]
        return pure, G, b["status"].cpu().numpy(), b["ncycles"].cpu().numpy()

    def density(self, b, k):
        N = self.n_basis[k]
        return b["density"][self.density_offsets[k]:self.density_offsets[k + 1]].view(N, N)
