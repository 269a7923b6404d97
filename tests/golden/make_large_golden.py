"""Generate tests/golden/large_qcmm_reference.json: the oracle's energy + gradient of the large QC/MM system (200 QC
waters, 600 atoms, N = 1200, AM1, in 20000 TIP3P waters in an 85 A cube, NBModelABFS 8/12 A; workloads.large_qcmm,
seed 4), the configuration whose SCF runs over the whole GPU.  The oracle (oracle/mndo_oracle.c) is itself pinned to
the reference core and to the reference's stored energies (tests/test_oracle.py); one evaluation takes about a minute
here, too long for every test run, hence the fixture.

    python tests/golden/make_large_golden.py

Stored: the energy terms (Hartree), the QC gradients (Hartree/Bohr, QC/MM part included), the SCF cycle count, and the
MM gradients of the 400 MM atoms nearest the QC region's centre (the whole MM gradient array would be 60000 x 3)."""

import json, os, sys, time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from pdynamo_mirror_gb300 import workloads  # noqa: E402


def main():
    Z, X, Q, sel, charge = workloads.large_qcmm()
    nq = len(sel)
    t0 = time.time()
    knots = O.abfs_knots(8.0, 12.0)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    r = O.System(O.Hamiltonian("am1", list(Z[:nq])), list(Z[:nq]), charge=charge).energy(X[:nq], phi=phi)
    _, gq, gm = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=knots)
    centre = X[:nq].mean(axis=0)
    near = np.argsort(np.linalg.norm(X[nq:] - centre, axis=1))[:400]
    out = {"system": "workloads.large_qcmm(seed=4)", "hamiltonian": "am1", "nbmodel": "NBModelABFS(8, 12)",
           "converged": bool(r["converged"]), "ncycles": int(r["ncycles"]),
           "eelectronic": r["eelectronic"], "enuclear": r["enuclear"], "baseline": r["baseline"], "eqcmm": r["eqcmm"],
           "qc_gradients": (r["gradients"] + gq).tolist(), "charges": r["charges"].tolist(),
           "mm_sample": near.tolist(), "mm_gradients_sample": gm[near].tolist(),
           "mm_gradient_sum": gm.sum(axis=0).tolist(), "seconds": time.time() - t0}
    with open(os.path.join(HERE, "large_qcmm_reference.json"), "w") as f:
        json.dump(out, f)
    print("written; %.1f s, %d cycles" % (out["seconds"], out["ncycles"]))


if __name__ == "__main__":
    main()
