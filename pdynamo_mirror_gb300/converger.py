"""DIISSCFConverger: the keyword surface of pDynamo's DIIS/ODA SCF converger.

Options and defaults follow ``pMolecule.DIISSCFConverger.pyx:140-150`` and ``DIISSCFConverger.c:27-32``.
The iteration itself runs on the device inside the SCF kernel (csrc/scf.cu).
"""

from . import _native


class DIISSCFConverger:
    """DIIS with ODA (RCA) start-up, as pDynamo's default converger."""

    _DEFAULTS = {"densityTolerance": 1.0e-8, "diisOnset": 0.2, "energyTolerance": 2.0e-4, "history": 10,
                 "maximumSCFCycles": 100, "useRCA": True}

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

    def options(self):
        return _native.SCFOptions(float(self.densityTolerance), float(self.energyTolerance), float(self.diisOnset),
                                  int(self.maximumSCFCycles), int(self.history), 1 if self.useRCA else 0, 0)

    def __getstate__(self):
        return {k: getattr(self, k) for k in self._DEFAULTS}
