"""Device orchestration of one QC region: the call sequence of one System.Energy(doGradients=True).

For a batch of frames (configurations of the same QC region and MM environment) the engine queues, on one
CUDA stream:
  1. QC/MM potentials at the QC atoms              pdg_qcmm_potentials   (NBModel.QCMMPotentials)
  2. integrals, the complete SCF, QC gradients     pdg_energy_gradients  (QCModel.Energy + EnergyGradients)
  3. QC/MM gradients with the final Lowdin charges pdg_qcmm_gradients    (NBModel.QCMMGradients)
(pMolecule/System.py:309-312).  Torch supplies device memory and the stream only.
"""

import contextlib, ctypes

import numpy as np
import torch

from . import _native
from .parameters import ANGSTROMS_TO_BOHRS, HARTREES_TO_KJ, element_table

GRADIENT_TO_KJ_PER_A = ANGSTROMS_TO_BOHRS * HARTREES_TO_KJ   # QCAtomContainer.c:632 CONVERSION_FACTOR


def require_cuda():
    if not torch.cuda.is_available():
        raise _native.NativeError("a CUDA device is required: the GB300 kernels are the only compute path")


# Basis size above which one frame's SCF is spread over the whole GPU (pdg_wide_*) instead of one CTA per frame.
WIDE_BASIS = 384


class QCEngine:
    """A pdg_system plus the device buffers of a batch.

    Regions of more than WIDE_BASIS basis functions (or wide=True) run every frame's SCF over the whole GPU
    (pdg_wide_energy_gradients, one frame after another); smaller ones give each frame one CTA
    (pdg_energy_gradients, all frames in one launch)."""

    def __init__(self, hamiltonian, atomic_numbers, charge, device=None, wide=None):
        require_cuda()
        self.L = _native.load()
        self.device = torch.device(device or "cuda")
        self.atomic_numbers = [int(z) for z in atomic_numbers]
        self.elements, records, index = element_table(hamiltonian, self.atomic_numbers)
        self._records = np.ascontiguousarray(records)
        self._index = np.ascontiguousarray(index)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(self.L.pdg_system_create(self._records.ctypes.data_as(ctypes.c_void_p), len(self.elements),
                                                   len(self.atomic_numbers), self._index.ctypes.data_as(ctypes.c_void_p),
                                                   int(charge), ctypes.byref(h)), "pdg_system_create")
        self.handle = h
        nb, no, npair = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _native.check(self.L.pdg_system_info(h, ctypes.byref(nb), ctypes.byref(no), ctypes.byref(npair)), "pdg_system_info")
        self.n_atoms, self.n_basis, self.n_occupied, self.n_pairs = len(self.atomic_numbers), nb.value, no.value, npair.value
        from .parameters import E_ZCORE
        self.n_electrons = int(round(sum(self._records[k][E_ZCORE] for k in self._index))) - int(charge)
        self.density_open = None     # device [F, n_sets, N, N] of the last open-shell / fractional-occupancy run
        self._ws, self._ws_frames = None, 0
        self._qcmm_ws = None
        self.wide = (self.n_basis > WIDE_BASIS) if wide is None else bool(wide)
        self._wide = None
        if self.wide:
            w = ctypes.c_void_p()
            with torch.cuda.device(self.device):
                _native.check(self.L.pdg_wide_create(h, ctypes.byref(w)), "pdg_wide_create")
            self._wide = w
        self.density = None          # device [F, N, N], kept between calls as the reference keeps its state
        self._knots = {}
        self._base, self._base_on = None, False   # shared base of the mixed method's perturbative steps

    def __del__(self):
        try:
            if getattr(self, "_wide", None):
                self.L.pdg_wide_destroy(self._wide)
            if getattr(self, "handle", None):
                self.L.pdg_system_destroy(self.handle)
        except Exception:
            pass

    def workspace(self, n_frames):
        if self.wide:
            n_frames = 1   # the wide path computes one frame at a time
        if self._ws is None or self._ws_frames < n_frames:
            nbytes = int(self.L.pdg_wide_workspace_bytes(self.handle)) if self.wide else int(self.L.pdg_workspace_bytes(self.handle, n_frames))
            self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._ws_frames = n_frames
        return self._ws

    def qcmm_workspace(self, n_frames, n_mm):
        """The device workspace of pdg_qcmm_potentials / pdg_qcmm_gradients (the per-frame near lists), grown as
        needed: (tensor, bytes)."""
        need = int(self.L.pdg_qcmm_workspace_bytes(int(n_frames), int(n_mm)))
        if self._qcmm_ws is None or self._qcmm_ws.numel() < need:
            self._qcmm_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._qcmm_ws, self._qcmm_ws.numel()

    def knots(self, nbmodel):
        k = id(nbmodel)
        if k not in self._knots:
            self._knots[k] = torch.as_tensor(nbmodel.knots(), dtype=torch.float64, device=self.device)
        return self._knots[k]

    def run(self, qc_xyz, converger, mm_xyz=None, mm_charges=None, nbmodel=None, gradients=True, warm_start=True, guess=None,
            mm_gradients=True, events=False):
        """qc_xyz [F, n, 3] and mm_xyz [F, m, 3] in Angstrom (device float64), mm_charges [m].  The SCF starts
        from the previous density (warm_start, same batch shape), else from guess.predict (a
        LearnedDensityGuess, unless its validation disabled it), else from the diagonal guess.  mm_gradients=False skips the
        MM-side QC/MM gradients (fixed MM atoms).  Returns a dict of device tensors in Hartree / Hartree per Bohr.
        events=True also returns "events": four CUDA events on the stream, before the QC/MM potentials, after them,
        after pdg_energy_gradients and after the QC/MM gradients (for profiling)."""
        F = qc_xyz.shape[0]
        n, N = self.n_atoms, self.n_basis
        dev = self.device
        stream = torch.cuda.current_stream(dev)
        sh = _native.stream_handle(stream)
        ws = self.workspace(F)
        out = {}
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if events else None

        def mark(k):
            if ev:
                ev[k].record(stream)
        phi = None
        qcmm = nbmodel is not None and mm_xyz is not None and mm_xyz.shape[1] > 0
        # the QC/MM kernels on a side stream, beside the integrals and the pair gradients (pdg_set_side_stream),
        # except when phase events are wanted (their intervals assume one stream) and on the wide path
        side = self._side_stream() if (qcmm and not events and not self.wide) else None
        qsh = sh
        if side is not None:
            side.wait_stream(stream)
            qsh = _native.stream_handle(side)

        def on_side():
            # tensors the side stream writes come from its own pool
            return torch.cuda.stream(side) if side is not None else contextlib.nullcontext()
        mark(0)
        if qcmm:
            knots = self.knots(nbmodel) if nbmodel.model_id == 1 else None
            nk = 0 if knots is None else knots.numel() // 3
            with on_side():
                phi = torch.empty((F, n), dtype=torch.float64, device=dev)
            qws, qwb = self.qcmm_workspace(F, mm_xyz.shape[1])
            _native.check(self.L.pdg_qcmm_potentials(nbmodel.model_id, F, n, mm_xyz.shape[1], _native.ptr(qc_xyz), _native.ptr(mm_xyz),
                                                     _native.ptr(mm_charges), nk, _native.ptr(knots), float(nbmodel.outerCutoff),
                                                     _native.ptr(phi), _native.ptr(qws), qwb, qsh), "pdg_qcmm_potentials")
        mark(1)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        use = 1 if (warm_start and self.density is not None and self.density.shape[0] == F) else 0
        if not use and guess is not None and guess.enabled:
            # the prediction reads the QC/MM potentials: on the side stream too, before the SCF's wait
            with on_side():
                self.density = guess.predict(qc_xyz, phi)
            use = getattr(guess, "start_mode", 1)
        if not use:
            self.density = torch.empty((F, N, N), dtype=torch.float64, device=dev)
        energies = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=dev)
        grad = torch.empty((F, n, 3), dtype=torch.float64, device=dev) if gradients else None
        charges = torch.empty((F, n), dtype=torch.float64, device=dev)
        status = torch.empty(F, dtype=torch.int32, device=dev)
        ncycles = torch.empty(F, dtype=torch.int32, device=dev)
        opts = converger.options()
        if self.wide:
            # one frame after another, each over the whole GPU
            for f in range(F):
                _native.check(self.L.pdg_wide_energy_gradients(
                    self._wide, _native.ptr(xyz_bohr[f]), _native.ptr(None if phi is None else phi[f]), ctypes.byref(opts),
                    _native.ptr(self.density[f]), use, _native.ptr(energies[f]), _native.ptr(None if grad is None else grad[f]),
                    _native.ptr(charges[f]), _native.ptr(status[f:f + 1]), _native.ptr(ncycles[f:f + 1]), _native.ptr(ws), ws.numel(), sh),
                    "pdg_wide_energy_gradients")
        else:
            shared = opts.density_step != 0 and bool(getattr(converger, "sharedBase", False))
            self._attach_base(shared and self._base is not None)
            self._attach_side(side)
            _native.check(self.L.pdg_energy_gradients(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(phi), ctypes.byref(opts),
                                                      _native.ptr(self.density), use, _native.ptr(energies), _native.ptr(grad),
                                                      _native.ptr(charges), _native.ptr(status), _native.ptr(ncycles),
                                                      _native.ptr(ws), ws.numel(), sh), "pdg_energy_gradients")
            if shared and self._base is None:
                self.capture_base(F, 0)
        out.update(energies=energies, qc_gradients=grad, charges=charges, status=status, ncycles=ncycles, phi=phi)
        mark(2)
        if qcmm and gradients:
            with on_side():
                gqc = torch.empty((F, n, 3), dtype=torch.float64, device=dev)
                gmm = torch.empty((F, mm_xyz.shape[1], 3), dtype=torch.float64, device=dev) if mm_gradients else None
            # the mixed method takes the QC/MM gradient pair terms in FP32 (per-atom sums in FP64); plain FP64 keeps FP64
            gmodel = nbmodel.model_id | (_native.QCMM_FP32_PAIRS if opts.density_step != 0 else 0)
            _native.check(self.L.pdg_qcmm_gradients(gmodel, F, n, mm_xyz.shape[1], _native.ptr(qc_xyz), _native.ptr(mm_xyz),
                                                    _native.ptr(mm_charges), _native.ptr(charges), nk, _native.ptr(knots),
                                                    float(nbmodel.outerCutoff), _native.ptr(gqc), _native.ptr(gmm), _native.ptr(qws), qwb, qsh),
                          "pdg_qcmm_gradients")
            out.update(qcmm_qc_gradients=gqc, qcmm_mm_gradients=gmm)
        if side is not None:
            stream.wait_stream(side)
        mark(3)
        if ev:
            out["events"] = ev
        return out

    def run_uhf(self, qc_xyz, converger, n_alpha, n_beta, mm_xyz=None, mm_charges=None, nbmodel=None, gradients=True, warm_start=True,
                mm_gradients=True):
        """The spin-unrestricted E + gradient with n_alpha and n_beta electrons in cardinal occupancies: run_open."""
        occ = _native.Occupancy(spin_restricted=0, occupancy_type=0, alpha_charge=float(n_alpha), beta_charge=float(n_beta))
        return self.run_open(qc_xyz, converger, occ, mm_xyz, mm_charges, nbmodel, gradients, warm_start, mm_gradients)

    def run_open(self, qc_xyz, converger, occupancy, mm_xyz=None, mm_charges=None, nbmodel=None, gradients=True, warm_start=True,
                 mm_gradients=True):
        """The open-shell or fractional-occupancy E + gradient of frames qc_xyz [F, n, 3] (A) with the density sets and
        occupancies of occupancy (a _native.Occupancy; pdg_energy_gradients_open, the FP64 method), starting from the
        previous run's densities when warm_start and the shapes match, else from the diagonal guess.  Returns run()'s
        dict plus "density_sets" (device [F, n_sets, N, N]: the total density, or alpha and beta), "density" (total)
        and, for two sets, "density_alpha", "density_beta" and "spin_density" (the last with gradients)."""
        F = qc_xyz.shape[0]
        n, N = self.n_atoms, self.n_basis
        ns = 1 if occupancy.spin_restricted else 2
        dev = self.device
        stream = torch.cuda.current_stream(dev)
        sh = _native.stream_handle(stream)
        opts = converger.options()
        if opts.density_step != 0:
            raise ValueError("Open-shell and fractional-occupancy states run the FP64 density step (densityStep 'fp64').")
        if self.wide:
            raise ValueError("Open-shell and fractional-occupancy states run one CTA per frame (at most %d basis functions)." % WIDE_BASIS)
        phi = None
        qcmm = nbmodel is not None and mm_xyz is not None and mm_xyz.shape[1] > 0
        if qcmm:
            knots = self.knots(nbmodel) if nbmodel.model_id == 1 else None
            nk = 0 if knots is None else knots.numel() // 3
            phi = torch.empty((F, n), dtype=torch.float64, device=dev)
            qws, qwb = self.qcmm_workspace(F, mm_xyz.shape[1])
            _native.check(self.L.pdg_qcmm_potentials(nbmodel.model_id, F, n, mm_xyz.shape[1], _native.ptr(qc_xyz), _native.ptr(mm_xyz),
                                                     _native.ptr(mm_charges), nk, _native.ptr(knots), float(nbmodel.outerCutoff),
                                                     _native.ptr(phi), _native.ptr(qws), qwb, sh), "pdg_qcmm_potentials")
        need = int(self.L.pdg_open_workspace_bytes(self.handle, F))
        if getattr(self, "_open_ws", None) is None or self._open_ws.numel() < need:
            self._open_ws = torch.empty(need, dtype=torch.uint8, device=dev)
        ws = self._open_ws
        use = 1 if (warm_start and self.density_open is not None and tuple(self.density_open.shape[:2]) == (F, ns)) else 0
        if not use:
            self.density_open = torch.empty((F, ns, N, N), dtype=torch.float64, device=dev)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        energies = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=dev)
        grad = torch.empty((F, n, 3), dtype=torch.float64, device=dev) if gradients else None
        ts = torch.empty((2, F, N, N), dtype=torch.float64, device=dev) if (gradients and ns == 2) else None
        charges = torch.empty((F, n), dtype=torch.float64, device=dev)
        status = torch.empty(F, dtype=torch.int32, device=dev)
        ncycles = torch.empty(F, dtype=torch.int32, device=dev)
        self._attach_side(None)
        _native.check(self.L.pdg_energy_gradients_open(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(phi), ctypes.byref(opts),
                                                       ctypes.byref(occupancy), _native.ptr(self.density_open), use, _native.ptr(energies),
                                                       _native.ptr(grad), _native.ptr(charges), _native.ptr(status), _native.ptr(ncycles),
                                                       _native.ptr(ts), _native.ptr(ws), ws.numel(), sh), "pdg_energy_gradients_open")
        D = self.density_open
        out = dict(energies=energies, qc_gradients=grad, charges=charges, status=status, ncycles=ncycles, phi=phi, density_sets=D)
        if ns == 1:
            out.update(density=D[:, 0], spin_populations=torch.zeros((F, n), dtype=torch.float64, device=dev))
        else:
            # Lowdin spin populations of the QC atoms: sum over each atom's orbitals of (P_alpha - P_beta)_mm
            sd = D[:, 0].diagonal(dim1=-2, dim2=-1) - D[:, 1].diagonal(dim1=-2, dim2=-1)
            out.update(density_alpha=D[:, 0], density_beta=D[:, 1],
                       spin_populations=torch.zeros((F, n), dtype=torch.float64, device=dev).index_add_(1, self.basis_atom(), sd))
            if gradients:
                out.update(density=ts[0], spin_density=ts[1])
            else:
                out.update(density=D[:, 0] + D[:, 1])
        if qcmm and gradients:
            gqc = torch.empty((F, n, 3), dtype=torch.float64, device=dev)
            gmm = torch.empty((F, mm_xyz.shape[1], 3), dtype=torch.float64, device=dev) if mm_gradients else None
            _native.check(self.L.pdg_qcmm_gradients(nbmodel.model_id, F, n, mm_xyz.shape[1], _native.ptr(qc_xyz), _native.ptr(mm_xyz),
                                                    _native.ptr(mm_charges), _native.ptr(charges), nk, _native.ptr(knots),
                                                    float(nbmodel.outerCutoff), _native.ptr(gqc), _native.ptr(gmm), _native.ptr(qws), qwb, sh),
                          "pdg_qcmm_gradients")
            out.update(qcmm_qc_gradients=gqc, qcmm_mm_gradients=gmm)
        return out

    def basis_atom(self):
        """Device index of the atom of every basis function (the atoms' orbitals in atom order)."""
        if getattr(self, "_basis_atom", None) is None:
            from .parameters import E_NORB
            norb = [int(self._records[k][E_NORB]) for k in self._index]
            self._basis_atom = torch.as_tensor(np.repeat(np.arange(self.n_atoms), norb), dtype=torch.long, device=self.device)
        return self._basis_atom

    def _side_stream(self):
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(device=self.device)
        return self._side

    def _attach_side(self, side):
        h = None if side is None else side.cuda_stream
        if h != getattr(self, "_side_on", None):
            _native.check(self.L.pdg_set_side_stream(self.handle, None if h is None else ctypes.c_void_p(h)), "pdg_set_side_stream")
            self._side_on = h

    def _attach_base(self, on):
        if on != self._base_on:
            _native.check(self.L.pdg_set_shared_base(self.handle, _native.ptr(self._base) if on else None), "pdg_set_shared_base")
            self._base_on = on

    def capture_base(self, n_frames, frame=0):
        """Keep frame `frame`'s perturbative base from the last mixed-method run of n_frames frames
        (pdg_base_capture) as the shared base of later runs with a sharedBase converger."""
        if self._base is None:
            self._base = torch.empty(int(self.L.pdg_base_bytes(self.handle)), dtype=torch.uint8, device=self.device)
        ws = self.workspace(n_frames)
        _native.check(self.L.pdg_base_capture(self.handle, int(n_frames), int(frame), _native.ptr(ws), ws.numel(), _native.ptr(self._base),
                                              _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_base_capture")

    def reset_base(self):
        """Forget the shared base: the next sharedBase run takes the full mixed path and captures a new one."""
        self._attach_base(False)
        self._base = None

    def scf(self, converger, phi=None, use_density=False):
        """pdg_scf: the SCF alone on the integrals of the last run (same frames); returns (energies, status,
        ncycles) device tensors and updates self.density."""
        F = self.density.shape[0]
        ws = self.workspace(F)
        energies = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=self.device)
        status = torch.empty(F, dtype=torch.int32, device=self.device)
        ncycles = torch.empty(F, dtype=torch.int32, device=self.device)
        opts = converger.options()
        self._attach_base(opts.density_step != 0 and bool(getattr(converger, "sharedBase", False)) and self._base is not None)
        _native.check(self.L.pdg_scf(self.handle, F, _native.ptr(phi), ctypes.byref(opts), _native.ptr(self.density), 1 if use_density else 0,
                                     _native.ptr(energies), None, _native.ptr(status), _native.ptr(ncycles), _native.ptr(ws), ws.numel(),
                                     _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_scf")
        return energies, status, ncycles

    def density_step(self, fock, density_step=0, previous=None):
        """pdg_density: one density step for Fock matrices fock [F, N, N] (device float64)."""
        F = fock.shape[0]
        ws = self.workspace(F)
        P = previous.clone() if previous is not None else torch.zeros_like(fock)
        en = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=self.device)
        st = torch.empty(F, dtype=torch.int32, device=self.device)
        _native.check(self.L.pdg_density(self.handle, F, _native.ptr(fock.contiguous()), int(density_step), _native.ptr(P), _native.ptr(en),
                                         _native.ptr(st), _native.ptr(ws), ws.numel(), _native.stream_handle(torch.cuda.current_stream(self.device))),
                      "pdg_density")
        return P, en, st

    def phase_events(self, enable=True):
        """Record CUDA events around the integral, SCF and gradient kernels of every later run (pdg_phase_events)."""
        _native.check(self.L.pdg_phase_events(self.handle, 1 if enable else 0), "pdg_phase_events")

    def phase_times(self):
        """Device milliseconds of the last run's integrals, SCF and gradients (pdg_phase_times; waits for them)."""
        out = (ctypes.c_float * 3)()
        _native.check(self.L.pdg_phase_times(self.handle, out), "pdg_phase_times")
        return {"integrals": out[0], "scf": out[1], "gradients": out[2]}

    def wide_phase_events(self, enable=True):
        """Per-phase device timing of the wide path's later calls (pdg_wide_phase_events)."""
        _native.check(self.L.pdg_wide_phase_events(self._wide, 1 if enable else 0), "pdg_wide_phase_events")

    def wide_phase_times(self):
        """Device milliseconds per phase of the last wide call (pdg_wide_phase_times), as {phase: ms}."""
        out = (ctypes.c_float * len(_native.WIDE_PHASES))()
        _native.check(self.L.pdg_wide_phase_times(self._wide, out), "pdg_wide_phase_times")
        return dict(zip(_native.WIDE_PHASES, list(out)))

    def occupancy(self):
        """(threads per SCF CTA, dynamic shared bytes, resident SCF CTAs per SM)."""
        t, b, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _native.check(self.L.pdg_scf_occupancy(self.handle, ctypes.byref(t), ctypes.byref(b), ctypes.byref(n)), "pdg_scf_occupancy")
        return t.value, b.value, n.value

    def timings(self, n_frames):
        """Per-frame SCF phase timings (GPU clock cycles) of the last run, as {name: array}."""
        out = torch.empty((n_frames, len(_native.TIMERS)), dtype=torch.float64, device=self.device)
        ws = self.workspace(n_frames)
        _native.check(self.L.pdg_scf_timings(self.handle, n_frames, _native.ptr(ws), ws.numel(), _native.ptr(out),
                                             _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_scf_timings")
        t = out.cpu().numpy()
        return {name: t[:, k] for k, name in enumerate(_native.TIMERS)}

    # diagnostics used by the parity tests
    def one_electron(self, qc_xyz):
        F = qc_xyz.shape[0]
        ws = self.workspace(F)
        H = torch.empty((F, self.n_basis, self.n_basis), dtype=torch.float64, device=self.device)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        _native.check(self.L.pdg_one_electron(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(H), _native.ptr(ws), ws.numel(),
                                              _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_one_electron")
        return H

    def fock(self, qc_xyz, density, phi=None):
        F = qc_xyz.shape[0]
        ws = self.workspace(F)
        Fm = torch.empty((F, self.n_basis, self.n_basis), dtype=torch.float64, device=self.device)
        en = torch.empty((F, _native.NENERGY), dtype=torch.float64, device=self.device)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        _native.check(self.L.pdg_fock(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(phi), _native.ptr(density.contiguous()),
                                      _native.ptr(Fm), _native.ptr(en), _native.ptr(ws), ws.numel(),
                                      _native.stream_handle(torch.cuda.current_stream(self.device))), "pdg_fock")
        return Fm, en

    def gradients(self, qc_xyz, density):
        F = qc_xyz.shape[0]
        ws = self.workspace(F)
        g = torch.empty((F, self.n_atoms, 3), dtype=torch.float64, device=self.device)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        _native.check(self.L.pdg_gradients(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(density.contiguous()), _native.ptr(g),
                                           _native.ptr(ws), ws.numel(), _native.stream_handle(torch.cuda.current_stream(self.device))),
                      "pdg_gradients")
        return g

    def gradients_static_scratch(self, qc_xyz, density):
        """Gradients for given densities through pdg_gradients_static_scratch (no workspace, no allocation
        inside the library)."""
        F = qc_xyz.shape[0]
        g = torch.empty((F, self.n_atoms, 3), dtype=torch.float64, device=self.device)
        xyz_bohr = (qc_xyz * ANGSTROMS_TO_BOHRS).contiguous()
        _native.check(self.L.pdg_gradients_static_scratch(self.handle, F, _native.ptr(xyz_bohr), _native.ptr(density.contiguous()),
                                                          _native.ptr(g), _native.stream_handle(torch.cuda.current_stream(self.device))),
                      "pdg_gradients_static_scratch")
        return g
