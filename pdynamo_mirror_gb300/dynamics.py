"""Langevin dynamics of a System (QC atoms, and MM atoms where they are free), as many independent replicas on one GPU.

Restates pDynamo's LangevinVelocityVerletIntegrator (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py) and
the script function LangevinDynamics_SystemGeometry (pMoleculeScripts-1.9.0/pMoleculeScripts/MolecularDynamics.py:42-48).
Every step is one energy + gradient of every replica (System.Energy's path: QC/MM potentials, integrals, SCF,
QC and QC/MM gradients, the MM model's non-bonded and harmonic terms) between the two halves of the velocity Verlet
update (csrc/dynamics.cu).  The free atoms are the atoms that System.DefineFixedAtoms did not fix, QC or MM
(SystemGeometryObjectiveFunction.py:138-152).  With no fixed atoms, rotation and translation are removed as the
reference's script does by default (removeRotationTranslation, MolecularDynamics.py:27-32;
SystemGeometryObjectiveFunction.RemoveRotationTranslation, :213-240): mass-weighted vectors from each replica's
starting coordinates are projected out of the assigned velocities, the random deviates and the gradients, and the
temperature counts 3 n_free - 6 degrees of freedom.  With fixed atoms nothing is removed.

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
from .engine import GRADIENT_TO_KJ_PER_A, HARTREES_TO_KJ
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


def rotation_translation_vectors(coordinates3, masses):
    """Orthonormal mass-weighted translation and rotation vectors [K, n, 3], K <= 6, as
    Coordinates3_RotationTranslationVectors builds them with the atoms' masses as weights
    (pCore-1.9.0/extensions/csource/Coordinates3.c:1315-1385): Tx, Ty, Tz, Rx, Ry, Rz in that order, weighted by
    sqrt(m), the rotations about the centre of mass; then one Gram-Schmidt pass that keeps a vector only if its
    norm after orthogonalisation exceeds 1e-10 sqrt(3 n) (Real2DArray_GramSchmidtOrthogonalize, Real2DArray.c:487-545)."""
    X = np.asarray(coordinates3, dtype=np.float64).reshape(-1, 3)
    m = np.asarray(masses, dtype=np.float64).ravel()
    n = len(m)
    w = np.sqrt(m)
    d = X - (m[:, None] * X).sum(0) / m.sum()
    raw = []
    for a in range(3):
        v = np.zeros((n, 3)); v[:, a] = w
        raw.append(v)
    for a, (p, q) in enumerate([(2, 1), (0, 2), (1, 0)]):   # R_x: (z, y), R_y: (x, z), R_z: (y, x)
        v = np.zeros((n, 3))
        v[:, p] = w * d[:, q]
        v[:, q] = -w * d[:, p]
        raw.append(v)
    delta = 1.0e-10 * math.sqrt(3 * n)
    out = []
    for v in raw:
        v = v.ravel().copy()
        for u in out:
            v -= (v @ u) * u
        nrm = math.sqrt(v @ v)
        if nrm > delta:
            out.append(v / nrm)
    return np.array(out).reshape(len(out), n, 3)


class LangevinDynamics:
    """Langevin dynamics of `replicas` independent copies of a System: its free atoms move, its fixed atoms stay.

    Coordinates of all atoms (`X`, [R, n_atoms, 3] Angstrom), velocities and accelerations of the free atoms and the
    SCF densities stay on the device; `step()` queues, on one stream: the position half-step, the energy + gradient
    of every replica, the velocity half-step."""

    def __init__(self, system, replicas=1, timeStep=0.001, temperature=300.0, collisionFrequency=25.0, seed=0,
                 densityGuess="previous", coordinates=None, removeRotationTranslation=True):
        if system.qcModel is None:
            raise ValueError("No QC model defined.")
        n = len(system.atomicNumbers)
        fixed = set(system.fixedAtoms or [])
        self.free = [i for i in range(n) if i not in fixed]
        if not self.free:
            raise ValueError("No free atoms.")
        if not isinstance(densityGuess, str):
            self.mode = "learned"
        elif densityGuess in GUESS_MODES:
            self.mode = densityGuess
        else:
            raise ValueError("Unknown densityGuess: %r" % (densityGuess,))
        self.guess = densityGuess
        self.system = system
        self.eng = eng = system.engine()
        self.dev = dev = eng.device
        self.integrator = LangevinVelocityVerletIntegrator(collisionFrequency, temperature, timeStep)
        self.R = int(replicas)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.n_atoms = n
        nf = len(self.free)
        masses = np.array([atomic_mass(system.atomicNumbers[i]) for i in self.free])
        self.d_free = torch.as_tensor(self.free, dtype=torch.int32, device=dev)
        self.d_mass = torch.as_tensor(masses, dtype=torch.float64, device=dev)
        self.d_isqm = torch.as_tensor(1.0 / np.sqrt(masses), dtype=torch.float64, device=dev)
        self.d_sqm = torch.as_tensor(np.sqrt(masses), dtype=torch.float64, device=dev)
        X = system.coordinates3 if coordinates is None else np.asarray(coordinates, dtype=np.float64)
        X = np.ascontiguousarray(np.broadcast_to(X, (self.R,) + system.coordinates3.shape) if X.ndim == 2 else X)
        self.X = system._device_frames(X).contiguous()          # [R, n, 3] Angstrom, free rows moved in place
        self._qs, self._ms, self.mm_q, mm_idx = system._selections()
        self.nb = system.nbModel if self._ms is not None else None
        self.mm_gradients = self.nb is not None and any(i not in fixed for i in mm_idx)
        self.mmi = system._mm_interactions() if getattr(system, "mmModel", None) is not None else None
        # rotation and translation removed only when no atom is fixed (SystemGeometryObjectiveFunction.py:213-240)
        self.V, self.n_constraints = None, 0
        if removeRotationTranslation and not fixed:
            allm = np.array([atomic_mass(z) for z in system.atomicNumbers])
            Vs = [rotation_translation_vectors(X[r], allm) for r in range(self.R)]
            if len({len(v) for v in Vs}) != 1:
                raise ValueError("The replicas' starting geometries give different numbers of rotation and translation vectors.")
            self.n_constraints = len(Vs[0])
            self.V = torch.as_tensor(np.ascontiguousarray(np.array(Vs)), dtype=torch.float64, device=dev)
        self.dof = 3 * nf - self.n_constraints
        if self.dof <= 0:
            raise ValueError("No degrees of freedom left after removing rotation and translation.")
        self.vel = torch.zeros((self.R, nf, 3), dtype=torch.float64, device=dev)
        self.acc = torch.zeros_like(self.vel)
        self.mv2 = torch.zeros(self.R, dtype=torch.float64, device=dev)
        self.G = torch.zeros((self.R, n, 3), dtype=torch.float64, device=dev)
        self.potential = torch.zeros(self.R, dtype=torch.float64, device=dev)
        self._dev = torch.empty((self.R, nf, 3, 2), dtype=torch.float64, device=dev) if self.V is not None else None
        self.n_step = 0
        self.history, self.model_history = [], []
        self.last = None
        self._assign_velocities(temperature)

    # -- coordinates of the QC and MM atoms (copies gathered from X)
    @property
    def xyz(self):
        """QC atoms' coordinates [R, n_qc, 3] (a copy)."""
        return self.system._take(self.X, self._qs)

    @property
    def mm_xyz(self):
        """Coordinates [R, n_mm, 3] of the MM atoms the QC region sees (a copy), None without them."""
        return None if self._ms is None else self.system._take(self.X, self._ms)

    @property
    def free_qc(self):
        qc = set(self.system.qcSelection)
        return [i for i in self.free if i in qc]

    # -- set-up
    def _sh(self):
        return _native.stream_handle(torch.cuda.current_stream(self.dev))

    def _project(self, arr, rows, n_rows, scale, width):
        _native.check(self.eng.L.pdg_linear_constraints_project(self.R, len(self.free), n_rows, _native.ptr(rows), self.n_constraints,
                                                                _native.ptr(self.V), _native.ptr(scale), width, _native.ptr(arr), self._sh()),
                      "pdg_linear_constraints_project")

    def _assign_velocities(self, temperature):
        """VelocitiesAssign (SystemGeometryObjectiveFunction.py:317-345): Gaussian mass-weighted velocities of width
        sqrt(kT/amu), rotation and translation projected out when they are removed, scaled per replica to the exact
        temperature; deviates from the device generator (stream 1)."""
        n = self.vel.numel()
        w = torch.empty(2 * ((n + 1) // 2), dtype=torch.float64, device=self.dev)
        _native.check(self.eng.L.pdg_normal_deviates((n + 1) // 2, self.seed, 0, 1, _native.ptr(w), self._sh()), "pdg_normal_deviates")
        sigma = MS_TO_APS * math.sqrt(CONSTANT_BOLTZMANN * max(temperature, 0.0) / CONSTANT_ATOMIC_MASS)
        v = (w[:n].view_as(self.vel) * sigma * self.d_isqm[None, :, None]).contiguous()
        if self.V is not None:
            self._project(v, None, len(self.free), self.d_sqm, 1)
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
        qc, mm = self.xyz, self.mm_xyz
        if self.mode == "learned":
            phi = None
            if self.nb is not None:
                phi = torch.empty((self.R, eng.n_atoms), dtype=torch.float64, device=self.dev)
                knots = eng.knots(self.nb) if self.nb.model_id == 1 else None
                nk = 0 if knots is None else knots.numel() // 3
                qws, qwb = eng.qcmm_workspace(self.R, mm.shape[1])
                _native.check(eng.L.pdg_qcmm_potentials(self.nb.model_id, self.R, eng.n_atoms, mm.shape[1], _native.ptr(qc),
                                                        _native.ptr(mm), _native.ptr(self.mm_q), nk, _native.ptr(knots),
                                                        float(self.nb.outerCutoff), _native.ptr(phi), _native.ptr(qws), qwb, self._sh()),
                              "pdg_qcmm_potentials")
            self.model_history = (self.model_history + [self.guess.predict(qc, phi)])[-3:]
        warm = False
        if self.mode != "diagonal" and self.history:
            if self.mode == "learned" and len(self.model_history) < 3:
                P0 = self.history[-1]
            else:
                P0 = self._start_density()
            # the SCF overwrites its start density with the converged one: never hand it a history entry
            eng.density = P0.clone() if any(P0 is h for h in self.history) else P0
            warm = True
        r = eng.run(qc, conv, mm, self.mm_q, self.nb, gradients=True, warm_start=warm, mm_gradients=self.mm_gradients)
        if (r["status"] != _native.PDG_OK).any():
            raise _native.NativeError("SCF procedure not converged in dynamics step %d." % self.n_step)
        if self.mode != "diagonal":
            self.history = (self.history + [eng.density])[-2:]
            eng.density = None
        # gradients of all atoms (kJ/mol/A) and the potential energy (kJ/mol) of each replica
        E = r["energies"]
        pot = E[:, _native.EN_ELECTRONIC] + E[:, _native.EN_NUCLEAR] + E[:, _native.EN_BASELINE]
        G = self.G
        G.zero_()
        gq = r["qc_gradients"]
        if "qcmm_qc_gradients" in r:
            gq = gq + r["qcmm_qc_gradients"]
            pot = pot + E[:, _native.EN_QCMM]
        G[:, self._qs] = gq * GRADIENT_TO_KJ_PER_A
        if self.mm_gradients:
            G[:, self._ms] = r["qcmm_mm_gradients"] * GRADIENT_TO_KJ_PER_A
        pot = pot * HARTREES_TO_KJ
        if self.mmi is not None:
            Emm, Gmm = self.mmi.run(self.X, gradients=True)
            G += Gmm
            pot = pot + Emm.sum(1)
            r["mm_energies"] = Emm
        if self.V is not None:
            self._project(G, self.d_free, self.n_atoms, self.d_isqm, 1)
        self.potential = pot
        self.last = r
        return r

    def _accelerations(self, r, facV3):
        _native.check(self.eng.L.pdg_langevin_velocities(self.R, len(self.free), self.n_atoms, _native.ptr(self.d_free),
                                                         _native.ptr(self.d_mass), _native.ptr(self.G), None, 1.0, facV3,
                                                         _native.ptr(self.vel), _native.ptr(self.acc), _native.ptr(self.mv2), self._sh()),
                      "pdg_langevin_velocities")

    def initialize(self):
        """Function and accelerations at the starting point (MultiDimensionalDynamics's initial evaluation)."""
        r = self._evaluate()
        # a = -100 g / m with no velocity change (facV3 = 0)
        self._accelerations(r, 0.0)
        return r

    def step(self, deviates=None, random=True):
        """One Iteration (LangevinVelocityVerletIntegrator.py:126-145) of every replica.  deviates: optional device
        buffer [R, n_free, 3, 2] that receives the random deviates (w1, w2) as applied (projected, where rotation and
        translation are removed).  random=False: no random forces (with a small collision frequency, plain velocity
        Verlet)."""
        if self.last is None:
            self.initialize()
        self.n_step += 1
        eng = self.eng
        mode = 1 if random else 0
        if random and self.V is not None:
            # RandomForces with ApplyLinearConstraints on both deviate vectors (:147-157): the same counter-based
            # deviates as mode 1, projected, then read by the position kernel
            D = self._dev
            nf = len(self.free)
            _native.check(eng.L.pdg_normal_deviates(self.R * nf * 3, self.seed, self.n_step, 0, _native.ptr(D), self._sh()),
                          "pdg_normal_deviates")
            self._project(D, None, nf, None, 2)
            if deviates is not None:
                deviates.copy_(D.view_as(deviates))
            deviates, mode = D, 2
        _native.check(eng.L.pdg_langevin_positions(self.R, self.n_atoms, len(self.free), _native.ptr(self.d_free), _native.ptr(self.d_isqm),
                                                   _native.ptr(self.X), _native.ptr(self.vel), _native.ptr(self.acc), self.integrator.factors(),
                                                   mode, self.seed, self.n_step, _native.ptr(deviates), self._sh()),
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

    def potential_energies(self):
        """Potential energy (kJ/mol) per replica at the last evaluation, host array: the total of System.Energy
        (Pure QC, QC/MM Elect. and the MM model's terms)."""
        return self.potential.cpu().numpy()

    def total_energies(self):
        """Potential plus kinetic energy (kJ/mol) per replica (the integrator's state.totalEnergy, :135)."""
        return self.potential_energies() + self.temperatures()[0]

    def replica_coordinates(self, replica=0):
        """All atoms of one replica (host, Angstrom)."""
        return self.X[replica].cpu().numpy()

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
                                    densityGuess="previous", replicas=1, callback=None, trajectories=None, removeRotationTranslation=True):
    """Langevin dynamics of the system's free atoms (MolecularDynamics.py:42-48 keywords: steps, timeStep in ps,
    temperature, collisionFrequency, removeRotationTranslation, trajectories = [(trajectory, saveFrequency)] of
    replica 0).  Leaves the last coordinates of replica 0 on system.coordinates3 and its velocities on
    system.configuration.velocities; returns the LangevinDynamics object."""
    md = LangevinDynamics(system, replicas=replicas, timeStep=timeStep, temperature=temperature,
                          collisionFrequency=collisionFrequency, seed=seed, densityGuess=densityGuess,
                          removeRotationTranslation=removeRotationTranslation)
    md.run(steps, callback, trajectories=trajectories)
    system.coordinates3[...] = md.X[0].cpu().numpy()
    system.configuration.velocities = md.vel[0].cpu().numpy()
    return md
