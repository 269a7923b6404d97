"""Langevin dynamics of the QC atoms of a System, as many independent replicas on one GPU.

Restates pDynamo's LangevinVelocityVerletIntegrator (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py) and
the script function LangevinDynamics_SystemGeometry (pMoleculeScripts-1.9.0/pMoleculeScripts/MolecularDynamics.py:42-48).
Every step is one energy + gradient of every replica (System.Energy's path: QC/MM potentials, integrals, SCF,
QC and QC/MM gradients) between the two halves of the velocity Verlet update (csrc/dynamics.cu).  MM atoms
must be fixed (System.DefineFixedAtoms): this library has no MM force field, and with fixed atoms pDynamo removes
no rotation or translation (SystemGeometryObjectiveFunction.py:213-222).

Start density of each step's SCF (`densityGuess`):
  "diagonal"     the reference's cold guess every step (QCOnePDM.c:280);
  "previous"     the previous step's converged density: the reference's behaviour in dynamics, where the QC state
                 persists on the configuration between Energy calls (pMolecule.QCModel.pyx:153);
  "extrapolate"  2 P(t-1) - P(t-2) (linear extrapolation of the converged densities);
  a LearnedDensityGuess  the extrapolation corrected by the model's own change between the steps:
                 2 P(t-1) - P(t-2) + M(t) - 2 M(t-1) + M(t-2), M the model's prediction (not in the reference).
"""

import ctypes, math

import numpy as np
import torch

from . import _native
from .engine import GRADIENT_TO_KJ_PER_A
from .parameters import atomic_mass

# pCore-1.9.0/pCore/Units.py:15,17; SystemGeometryObjectiveFunction.py:19-28
CONSTANT_ATOMIC_MASS = 1.66053886e-27
CONSTANT_BOLTZMANN = 1.3806505e-23
MS_TO_APS = 1.0e-2
AMUA2PS2_TO_K = CONSTANT_ATOMIC_MASS / (CONSTANT_BOLTZMANN * MS_TO_APS ** 2)
AMUA2PS2_TO_KJMOL = 1.0e-2

GUESS_MODES = ("diagonal", "previous", "extrapolate")


class LangevinVelocityVerletIntegrator:
    """Integration constants of the reference integrator (collisionFrequency ps^-1, timeStep ps, temperature K)."""

    def __init__(self, collisionFrequency=25.0, temperature=300.0, timeStep=0.001):
        if collisionFrequency <= 0.0 or temperature < 0.0:
            raise ValueError("Invalid temperature handling options.")   # TemperatureHandlingOptions (:159-163)
        if timeStep <= 0.0:
            raise ValueError("Invalid time step.")
        self.collisionFrequency, self.temperature, self.timeStep = float(collisionFrequency), float(temperature), float(timeStep)
        self.constants = self._constants()

    def _constants(self):
        """CalculateIntegrationConstants (:63-112): exponential forms when gamma dt > 0.009, else the series."""
        f, dt = self.collisionFrequency * self.timeStep, self.timeStep
        if f > 0.009:
            c0 = math.exp(-f)
            c1 = (1.0 - c0) / f
            c2 = (1.0 - c1) / f
            sdR = math.sqrt(dt * dt * (2.0 - (3.0 - 4.0 * c0 + c0 * c0) / f) / f)
            sdV = math.sqrt(1.0 - c0 * c0)
            cRV1 = dt * (1.0 - c0) ** 2 / (f * sdR * sdV)
            cRV2 = math.sqrt(1.0 - cRV1 * cRV1)
        else:
            p = [f ** k for k in range(6)]
            c0 = p[0] - p[1] + p[2] / 2.0 - p[3] / 6.0 + p[4] / 24.0 - p[5] / 120.0
            c1 = p[0] - p[1] / 2.0 + p[2] / 6.0 - p[3] / 24.0 + p[4] / 120.0 - p[5] / 720.0
            c2 = 0.5 - p[1] / 6.0 + p[2] / 24.0 - p[3] / 120.0 + p[4] / 720.0 - p[5] / 5040.0
            sdR = (2.0 - 3.0 * p[1] / 4.0 + 67.0 * p[2] / 320.0 - 119.0 * p[3] / 2560.0) * math.sqrt(f / 6.0) * dt
            sdV = (2.0 - p[1] + 5.0 * p[2] / 12.0 - p[3] / 8.0 + 79.0 * p[4] / 2880.0) * math.sqrt(f / 2.0)
            cRV1 = (1.5 - 3.0 * p[1] / 16.0 - 51.0 * p[2] / 1280.0 + 17.0 * p[3] / 2048.0 + 40967.0 * p[4] / 11468800.0
                    - 57203.0 * p[5] / 91750400.0) / math.sqrt(3.0)
            cRV2 = (0.5 + 3.0 * p[1] / 16.0 - 9.0 * p[2] / 1280.0 - 109.0 * p[3] / 10240.0 + 10077.0 * p[4] / 11468800.0
                    + 14887.0 * p[5] / 18350080.0)
        t = math.sqrt(self.temperature / AMUA2PS2_TO_K)   # TemperatureConversionFactor (:262-265)
        return {"facR1": c1 * dt, "facR2": c2 * dt * dt, "facV1": c0, "facV2": (c1 - c2) * dt, "facV3": c2 * dt,
                "sdR": sdR * t, "sdV1": cRV1 * sdV * t, "sdV2": cRV2 * sdV * t}

    def factors(self):
        c = self.constants
        return (ctypes.c_double * 7)(c["facR1"], c["facR2"], c["facV1"], c["facV2"], c["sdR"], c["sdV1"], c["sdV2"])


class LangevinDynamics:
    """Langevin dynamics of `replicas` independent copies of a System's QC region in its fixed MM environment.

    Coordinates, velocities, accelerations and densities stay on the device; `step()` queues, on one stream:
    the position half-step, the energy + gradient of every replica, the velocity half-step."""

    def __init__(self, system, replicas=1, timeStep=0.001, temperature=300.0, collisionFrequency=25.0, seed=0,
                 densityGuess="previous", coordinates=None):
        if system.qcModel is None:
            raise ValueError("No QC model defined.")
        fixed = set(system.fixedAtoms or [])
        mm = system.mm_indices()
        if any(i not in fixed for i in mm):
            raise ValueError("MM atoms must be fixed (System.DefineFixedAtoms): there is no MM force field on this path.")
        if getattr(system, "mmModel", None) is not None:
            raise ValueError("The dynamics driver does not include the MM model's LJ terms yet: remove the MM model "
                             "(System.DefineMMModel(None)) to run QC/MM electrostatics only.")
        self.system = system
        self.eng = eng = system.engine()
        self.dev = eng.device
        self.integrator = LangevinVelocityVerletIntegrator(collisionFrequency, temperature, timeStep)
        self.R = int(replicas)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        qc = system.qcSelection
        self.free_qc = [k for k, i in enumerate(qc) if i not in fixed]
        if not self.free_qc:
            raise ValueError("No free atoms.")
        nf = len(self.free_qc)
        self.dof = 3 * nf
        masses = np.array([atomic_mass(system.atomicNumbers[qc[k]]) for k in self.free_qc])
        dev = self.dev
        self.d_free = torch.as_tensor(self.free_qc, dtype=torch.int32, device=dev)
        self.d_mass = torch.as_tensor(masses, dtype=torch.float64, device=dev)
        self.d_isqm = torch.as_tensor(1.0 / np.sqrt(masses), dtype=torch.float64, device=dev)
        X = system.coordinates3 if coordinates is None else np.asarray(coordinates, dtype=np.float64)
        X = np.broadcast_to(X, (self.R,) + system.coordinates3.shape) if X.ndim == 2 else X
        qc_x, mm_x, q, _ = system._device_inputs(np.ascontiguousarray(X))
        self.xyz = qc_x.contiguous()                   # [R, n_qc, 3] Angstrom, moved in place
        self.mm_xyz, self.mm_q = mm_x, q               # fixed
        self.nb = system.nbModel if mm_x is not None else None
        self.vel = torch.zeros((self.R, nf, 3), dtype=torch.float64, device=dev)
        self.acc = torch.zeros_like(self.vel)
        self.mv2 = torch.zeros(self.R, dtype=torch.float64, device=dev)
        self.n_step = 0
        self.guess = densityGuess
        if not isinstance(densityGuess, str):
            self.mode = "learned"
        elif densityGuess in GUESS_MODES:
            self.mode = densityGuess
        else:
            raise ValueError("Unknown densityGuess: %r" % (densityGuess,))
        self.history, self.model_history = [], []
        self.last = None
        self._assign_velocities(temperature)

    # -- set-up
    def _sh(self):
        return _native.stream_handle(torch.cuda.current_stream(self.dev))

    def _assign_velocities(self, temperature):
        """VelocitiesAssign (SystemGeometryObjectiveFunction.py:317-345): Gaussian mass-weighted velocities of width
        sqrt(kT/amu), scaled per replica to the exact temperature; deviates from the device generator (stream 1)."""
        n = self.vel.numel()
        w = torch.empty(2 * ((n + 1) // 2), dtype=torch.float64, device=self.dev)
        _native.check(self.eng.L.pdg_normal_deviates((n + 1) // 2, self.seed, 0, 1, _native.ptr(w), self._sh()), "pdg_normal_deviates")
        sigma = MS_TO_APS * math.sqrt(CONSTANT_BOLTZMANN * max(temperature, 0.0) / CONSTANT_ATOMIC_MASS)
        v = w[:n].view_as(self.vel) * sigma * self.d_isqm[None, :, None]
        if temperature > 0.0:
            t = AMUA2PS2_TO_K * (self.d_mass[None, :, None] * v * v).sum(dim=(1, 2)) / self.dof
            v = v * torch.sqrt(temperature / t)[:, None, None]
        self.vel.copy_(v)

    # -- start densities
    def _start_density(self):
        """Density for the next SCF per densityGuess, or None for the diagonal guess."""
        H = self.history
        if self.mode == "diagonal" or not H:
            return None
        if self.mode == "previous" or len(H) < 2:
            return H[-1]
        terms, coef = [H[-1], H[-2]], [2.0, -1.0]
        if self.mode == "learned":
            M = self.model_history
            terms += [M[-1], M[-2], M[-3]]
            coef += [1.0, -2.0, 1.0]
        out = torch.empty_like(H[-1])
        arr = (ctypes.c_void_p * len(terms))(*[t.data_ptr() for t in terms])
        cf = (ctypes.c_double * len(coef))(*coef)
        _native.check(self.eng.L.pdg_density_combine(out.numel(), len(terms), arr, cf, _native.ptr(out), self._sh()), "pdg_density_combine")
        return out

    def _evaluate(self):
        eng, conv = self.eng, self.system.qcModel.converger
        if self.mode == "learned":
            phi = None
            if self.nb is not None:
                phi = torch.empty((self.R, eng.n_atoms), dtype=torch.float64, device=self.dev)
                knots = eng.knots(self.nb) if self.nb.model_id == 1 else None
                nk = 0 if knots is None else knots.numel() // 3
                qws, qwb = eng.qcmm_workspace(self.R, self.mm_xyz.shape[1])
                _native.check(eng.L.pdg_qcmm_potentials(self.nb.model_id, self.R, eng.n_atoms, self.mm_xyz.shape[1], _native.ptr(self.xyz),
                                                        _native.ptr(self.mm_xyz), _native.ptr(self.mm_q), nk, _native.ptr(knots),
                                                        float(self.nb.outerCutoff), _native.ptr(phi), _native.ptr(qws), qwb, self._sh()),
                              "pdg_qcmm_potentials")
            self.model_history = (self.model_history + [self.guess.predict(self.xyz, phi)])[-3:]
        warm = False
        if self.mode != "diagonal" and self.history:
            if self.mode == "learned" and len(self.model_history) < 3:
                P0 = self.history[-1]
            else:
                P0 = self._start_density()
            # the SCF overwrites its start density with the converged one: never hand it a history entry
            eng.density = P0.clone() if any(P0 is h for h in self.history) else P0
            warm = True
        r = eng.run(self.xyz, conv, self.mm_xyz, self.mm_q, self.nb, gradients=True, warm_start=warm, mm_gradients=False)
        if (r["status"] != _native.PDG_OK).any():
            raise _native.NativeError("SCF procedure not converged in dynamics step %d." % self.n_step)
        if self.mode != "diagonal":
            self.history = (self.history + [eng.density])[-2:]
            eng.density = None
        self.last = r
        return r

    def _accelerations(self, r, facV3):
        g_b = r.get("qcmm_qc_gradients")
        _native.check(self.eng.L.pdg_langevin_velocities(self.R, len(self.free_qc), self.eng.n_atoms, _native.ptr(self.d_free),
                                                         _native.ptr(self.d_mass), _native.ptr(r["qc_gradients"]), _native.ptr(g_b),
                                                         GRADIENT_TO_KJ_PER_A, facV3, _native.ptr(self.vel), _native.ptr(self.acc),
                                                         _native.ptr(self.mv2), self._sh()), "pdg_langevin_velocities")

    def initialize(self):
        """Function and accelerations at the starting point (MultiDimensionalDynamics's initial evaluation)."""
        r = self._evaluate()
        # a = -100 g / m with no velocity change (facV3 = 0)
        self._accelerations(r, 0.0)
        return r

    def step(self, deviates=None, random=True):
        """One Iteration (LangevinVelocityVerletIntegrator.py:126-145) of every replica.  deviates: optional device
        buffer [R, n_free, 3, 2] that receives the random deviates (w1, w2)."""
        if self.last is None:
            self.initialize()
        self.n_step += 1
        eng = self.eng
        _native.check(eng.L.pdg_langevin_positions(self.R, eng.n_atoms, len(self.free_qc), _native.ptr(self.d_free), _native.ptr(self.d_isqm),
                                                   _native.ptr(self.xyz), _native.ptr(self.vel), _native.ptr(self.acc), self.integrator.factors(),
                                                   1 if random else 0, self.seed, self.n_step, _native.ptr(deviates), self._sh()),
                      "pdg_langevin_positions")
        r = self._evaluate()
        self._accelerations(r, self.integrator.constants["facV3"])
        return r

    def set_bath(self, collisionFrequency=None, temperature=None):
        """Change the bath (collision frequency ps^-1, temperature K) for the following steps, e.g. a strongly
        damped equilibration before production."""
        it = self.integrator
        self.integrator = LangevinVelocityVerletIntegrator(it.collisionFrequency if collisionFrequency is None else collisionFrequency,
                                                           it.temperature if temperature is None else temperature, it.timeStep)

    def temperatures(self):
        """Kinetic energy (kJ/mol) and temperature (K) per replica, host arrays (Temperature, :255-260)."""
        mv2 = self.mv2.cpu().numpy()
        return 0.5 * AMUA2PS2_TO_KJMOL * mv2, AMUA2PS2_TO_K * mv2 / self.dof

    def replica_coordinates(self, replica=0):
        """All atoms of one replica (host, Angstrom): the system's coordinates with that replica's QC atoms."""
        X = np.array(self.system.coordinates3, dtype=np.float64)
        X[self.system.qcSelection] = self.xyz[replica].cpu().numpy()
        if self.mm_xyz is not None:   # the replica's fixed atoms, as it was given them
            X[self.system.mm_indices()] = self.mm_xyz[replica].cpu().numpy()
        return X

    def run(self, steps, callback=None, trajectories=None, replica=0):
        """steps Iterations; callback(self, r) after each.  trajectories: [(writer, saveFrequency)], e.g. a
        DCDTrajectoryFileWriter, written with the coordinates of `replica` at iteration 0 and at every multiple of
        saveFrequency, as the reference's objective function logs them (pCore-1.9.0/pCore/ObjectiveFunction.py:274-295).
        Returns the SCF cycles per step (device tensors)."""
        trajectories = [(t, int(f)) for (t, f) in (trajectories or []) if t is not None and int(f) > 0]
        if trajectories and self.last is None:
            self.initialize()
        for t, f in trajectories:
            if len(t) == 0:
                t.WriteHeader()
            if self.n_step % f == 0:
                t.WriteFrame(self.replica_coordinates(replica))
        cycles = []
        for _ in range(int(steps)):
            r = self.step()
            cycles.append(r["ncycles"])
            for t, f in trajectories:
                if self.n_step % f == 0:
                    t.WriteFrame(self.replica_coordinates(replica))
            if callback is not None:
                callback(self, r)
        return cycles


def LangevinDynamics_SystemGeometry(system, steps=1000, timeStep=0.001, temperature=300.0, collisionFrequency=25.0, seed=0,
                                    densityGuess="previous", replicas=1, callback=None, trajectories=None):
    """Langevin dynamics of the system's free atoms (MolecularDynamics.py:42-48 keywords: steps, timeStep in ps,
    temperature, collisionFrequency, trajectories = [(trajectory, saveFrequency)] of replica 0).  Leaves the last
    coordinates of replica 0 on system.coordinates3 and its velocities on system.configuration.velocities; returns
    the LangevinDynamics object."""
    md = LangevinDynamics(system, replicas=replicas, timeStep=timeStep, temperature=temperature,
                          collisionFrequency=collisionFrequency, seed=seed, densityGuess=densityGuess)
    md.run(steps, callback, trajectories=trajectories)
    X = md.xyz[0].cpu().numpy()
    for k, i in enumerate(system.qcSelection):
        system.coordinates3[i] = X[k]
    system.configuration.velocities = md.vel[0].cpu().numpy()
    return md
