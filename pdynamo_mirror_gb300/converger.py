"""DIISSCFConverger: the keyword surface of pDynamo's DIIS/ODA SCF converger.

Options and defaults follow ``pMolecule.DIISSCFConverger.pyx:140-150`` and ``DIISSCFConverger.c:27-32``.
The iteration itself runs on the device inside the SCF kernel (csrc/scf.cu).
"""

from . import _native

# The mixed method (the metric's "mixed"): split-BF16 purification with six partial products until the RMS
# density change falls below 1e-5, then FP64 and perturbative density steps to the reference's convergence test.
# DIISSCFConverger(**MIXED_METHOD).
MIXED_METHOD = {"densityStep": "purification", "purificationProducts": 6, "purificationSwitch": 1.0e-5}

# The mixed method with a shared base, as the benchmark times it for batches of frames of one QC region: the first
# batch runs MIXED_METHOD and leaves the base of one frame's FP64 step; every later batch starts each frame from
# that base's density and takes perturbative density steps around it (no purification, no FP64 eigensolve) until
# the reference's convergence test, falling back to FP64 steps for a frame the base no longer carries.
SHARED_BASE_METHOD = dict(MIXED_METHOD, sharedBase=True)


class DIISSCFConverger:
    """DIIS with ODA (RCA) start-up, as pDynamo's default converger.

    Two keywords beyond the reference's select the density step of the early cycles:
    densityStep "fp64" (default: the FP64 eigensolve every cycle, as the reference) or "purification"
    (split-BF16 SP2 purification on the tensor cores until the RMS density change falls below
    purificationSwitch, then the FP64 eigensolve to convergence); purificationProducts 3 or 6 is the
    number of BF16 partial products accumulated in FP32.  The converged result is that of the FP64 step.
    sharedBase (with "purification", one CTA per frame) keeps the base of the perturbative steps of one frame
    of the first call and starts every frame of later calls from it (pdg_set_shared_base): the same fixed
    point by a path of perturbative steps only.
    """

    _DEFAULTS = {"densityTolerance": 1.0e-8, "diisOnset": 0.2, "energyTolerance": 2.0e-4, "history": 10,
                 "maximumSCFCycles": 100, "useRCA": True, "densityStep": "fp64", "purificationSwitch": 1.0e-4,
                 "purificationProducts": 3, "sharedBase": False}

    def __init__(self, **options):
        for k, v in self._DEFAULTS.items():
            setattr(self, k, v)
        self.SetOptions(**options)

    def SetOptions(self, **options):
        for k in list(options):
            if k in self._DEFAULTS:
                setattr(self, k, options.pop(k))
        if options:
            raise ValueError("Invalid options: " + ", ".join(sorted(options)) + ".")
        if not (1 <= int(self.history) <= _native.MAX_HISTORY):
            raise ValueError("history must be between 1 and %d." % _native.MAX_HISTORY)
        if self.densityStep not in ("fp64", "purification"):
            raise ValueError("densityStep must be 'fp64' or 'purification'.")
        if int(self.purificationProducts) not in (3, 6):
            raise ValueError("purificationProducts must be 3 or 6.")
        if self.sharedBase and self.densityStep != "purification":
            raise ValueError("sharedBase needs the mixed method (densityStep 'purification').")

    def options(self):
        step = 0 if self.densityStep == "fp64" else int(self.purificationProducts)
        return _native.SCFOptions(float(self.densityTolerance), float(self.energyTolerance), float(self.diisOnset),
                                  int(self.maximumSCFCycles), int(self.history), 1 if self.useRCA else 0, step,
                                  float(self.purificationSwitch))

    def __getstate__(self):
        return {k: getattr(self, k) for k in self._DEFAULTS}
