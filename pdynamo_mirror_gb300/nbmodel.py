"""Non-bonding models for the QC/MM electrostatics: NBModelABFS and NBModelFull.

Only the QC/MM electrostatic part of pDynamo's NB models is on this path (the MM charges polarise the
QC region through Lowdin-charge embedding):

* ``NBModelFull``: plain 1/r between every QC atom and every MM point charge (NBModelFull.c:392,604).
* ``NBModelABFS``: the atom-based force-switching model with pDynamo's default QC/MM interaction, a
  Delta/Gaussian Coulomb of width 2 Bohr switched between the inner and outer cutoffs and tabulated as a
  cubic spline in r^2 (pMolecule.NBModelABFS.pyx:59-99, pMolecule.PairwiseInteraction.pyx:27-112,183-215).

The spline tabulation is restated here from the reference's Python (its Integrate function and
pCore/NumericalIntegration.py:21 AdaptiveSimpsonsRule); the spline's second derivatives solve the same
clamped tridiagonal system as CubicSpline_MakeFromReal1DArrays (pCore CubicSpline.c).
"""

import heapq, math

import numpy as np

from .parameters import ANGSTROMS_TO_BOHRS, BOHRS_TO_ANGSTROMS


def _f_gaussian(p):
    def F(r):
        x = p * r
        x2 = x * x
        if x > 1.0e-2:
            f = math.erf(x) / x
        else:
            f = (2.0 - x2 * (2.0 / 3.0 - x2 * (0.2 - x2 * (1.0 / 21.0 - x2 * (1.0 / 108.0 - x2 / 660.0))))) / math.sqrt(math.pi)
        return f * p
    return F


def _g_gaussian(p):
    def G(r):
        sp = math.sqrt(math.pi)
        x = p * r
        x2 = x * x
        if x > 1.0e-2:
            g = 2.0 * math.exp(-x2) / (sp * x) - math.erf(x) / x2
        else:
            g = -x * (4.0 / 3.0 - x2 * (0.8 - x2 * (2.0 / 7.0 - x2 * (2.0 / 27.0 - x2 / 66.0)))) / sp
        return g * p * p
    return G


def _switch(r, on, off):
    return (off ** 2 - r ** 2) ** 2 * (off ** 2 + 2.0 * r ** 2 - 3.0 * on ** 2) / (off ** 2 - on ** 2) ** 3


def adaptive_simpson(F, a, b, tolerance, maximum_iterations):
    """Priority-queue adaptive Simpson's rule (pCore/NumericalIntegration.py:21-65)."""
    h0 = abs(a - b)
    eps = tolerance / h0
    integral, heap, it = 0.0, [], 0
    p1 = 0.5 * (a + b)
    f0, f1, f2 = F(a), F(p1), F(b)
    heapq.heappush(heap, (0.0, h0, a, p1, b, f0, f1, f2, (f0 + 4.0 * f1 + f2) * h0 / 6.0))
    while it < maximum_iterations and heap:
        (err, h, p0, p2, p4, f0, f2, f4, whole) = heapq.heappop(heap)
        q1, q3 = 0.5 * (p0 + p2), 0.5 * (p2 + p4)
        g1, g3 = F(q1), F(q3)
        left = (f0 + 4.0 * g1 + f2) * h / 12.0
        right = (f2 + 4.0 * g3 + f4) * h / 12.0
        lrw = left + right - whole
        err = abs(lrw)
        if err < 15.0 * h * eps:
            integral += left + right + lrw / 15.0
        else:
            h *= 0.5
            heapq.heappush(heap, (-err, h, p0, q1, p2, f0, g1, f2, left))
            heapq.heappush(heap, (-err, h, p2, q3, p4, f2, g3, f4, right))
        it += 1
    for item in heap:
        integral += item[-1]
    return -integral if a > b else integral


def abfs_knots(inner, outer, width2=2.0 * BOHRS_TO_ANGSTROMS, point_density=50, damping=0.0):
    """Knots (x = r^2 in A^2, y in atomic units) of the QC/MM Delta/Gaussian ABFS spline."""
    p = (2.0 / math.sqrt(math.pi)) / width2
    F, G = _f_gaussian(p), _g_gaussian(p)
    GS = lambda r: G(r) * _switch(r, inner, outer)
    n = int(math.ceil(float(point_density) * outer + 1.0))
    x = np.zeros(n); y = np.zeros(n)
    inc = outer / float(n - 1)
    for i in range(1, n - 1):
        x[i] = inc * float(i)
    x[-1] = outer
    integral, iupper = 0.0, n - 2
    for i in range(n - 2, -1, -1):
        lo, up = x[i], x[i + 1]
        if lo < inner:
            iupper = i
            if up > inner:
                integral -= adaptive_simpson(GS, inner, up, 1.0e-15, 1000)
            break
        integral -= adaptive_simpson(GS, lo, up, 1.0e-15, 1000)
        y[i] = integral
    offset = integral - F(inner)
    if damping > 0.0:
        raise ValueError("QC/MM ABFS damping is not used by pDynamo's default QC/MM interaction.")
    for i in range(iupper + 1):
        y[i] = F(x[i]) + offset
    return x * x, y / ANGSTROMS_TO_BOHRS


def spline_second_derivatives(x, y):
    """Clamped cubic spline (zero end slopes) second derivatives by a tridiagonal solve."""
    n = len(x)
    dg, sub, sup, h = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
    dl = x[1] - x[0]
    dg[0], sup[0], h[0] = dl / 3.0, dl / 6.0, (y[1] - y[0]) / dl
    for i in range(1, n - 1):
        dl, du = x[i] - x[i - 1], x[i + 1] - x[i]
        sub[i - 1], dg[i], sup[i] = dl / 6.0, (dl + du) / 3.0, du / 6.0
        h[i] = (y[i + 1] - y[i]) / du + (y[i - 1] - y[i]) / dl
    du = x[n - 1] - x[n - 2]
    sub[n - 2], dg[n - 1], h[n - 1] = du / 6.0, du / 3.0, -(y[n - 1] - y[n - 2]) / du
    for i in range(1, n):
        m = sub[i - 1] / dg[i - 1]
        dg[i] -= m * sup[i - 1]
        h[i] -= m * h[i - 1]
    h[n - 1] /= dg[n - 1]
    for i in range(n - 2, -1, -1):
        h[i] = (h[i] - sup[i] * h[i + 1]) / dg[i]
    return h


class NBModelFull:
    """All QC/MM pairs with plain 1/r (the model of pDynamo's QC/MM tests)."""

    model_id = 0

    def __init__(self, dielectric=1.0):
        if dielectric != 1.0:
            raise ValueError("Only dielectric 1 is supported.")
        self.outerCutoff = 0.0

    def knots(self):
        return None


class NBModelABFS:
    """Atom-based force switching; QC/MM electrostatics via the Delta/Gaussian spline."""

    model_id = 1

    def __init__(self, innerCutoff=8.0, outerCutoff=12.0, listCutoff=13.5, dielectric=1.0, dampingCutoff=0.5,
                 electrostaticScale14=1.0, **options):
        # defaults as NBModelABFS.c:29-36; dampingCutoff and electrostaticScale14 act on the MM/MM terms (mmmodel.py)
        if options:
            raise ValueError("Invalid options: " + ", ".join(sorted(options)) + ".")
        if dielectric != 1.0:
            raise ValueError("Only dielectric 1 is supported.")
        if not (0.0 < innerCutoff < outerCutoff <= listCutoff):
            raise ValueError("Cutoffs must satisfy 0 < inner < outer <= list.")
        if not (0.0 <= dampingCutoff < innerCutoff):
            raise ValueError("The damping cutoff must satisfy 0 <= damping < inner.")
        self.innerCutoff, self.outerCutoff, self.listCutoff = float(innerCutoff), float(outerCutoff), float(listCutoff)
        self.dielectric, self.dampingCutoff, self.electrostaticScale14 = float(dielectric), float(dampingCutoff), float(electrostaticScale14)
        self._knots = None

    def knots(self):
        """[x | y | y''] flattened, as pdg_qcmm_potentials expects."""
        if self._knots is None:
            x, y = abfs_knots(self.innerCutoff, self.outerCutoff)
            self._knots = np.concatenate([x, y, spline_second_derivatives(x, y)])
        return self._knots
