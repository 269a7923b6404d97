/*
 * mndo_oracle.h - test infrastructure: plain-C CPU restatement of pDynamo 1.9.0's NDDO (MNDO-family)
 * closed-shell RHF energy + analytic gradient path with Lowdin-charge QC/MM embedding.
 *
 * This is the checker for the CUDA path, never the product: only tests, smoke() and bench.py's
 * CPU-baseline leg load it.  Each function in mndo_oracle.c cites the reference file:line it follows.
 * Parity is pinned against pDynamo's own compiled C core (oracle/_ref, built from the reference tree
 * where it exists) and against the golden fixtures under tests/golden/.
 *
 * Inputs use the same raw (file-unit) parameter layout as ref_shim.c so that the same arrays drive both.
 */
#ifndef MNDO_ORACLE_H
#define MNDO_ORACLE_H

#define ORACLE_NRAW     40
#define ORACLE_MAXGAUSS 4
#define ORACLE_MAXPDDG  4
#define ORACLE_MAXPRIM  6
#define ORACLE_MAXDIATOMIC 100   /* PM6 diatomic pairs per element, by partner atomic number */

typedef struct {
    double densityTolerance;   /* DIISSCFConverger.c:27 default 1e-8 */
    double diisOnset;          /* 0.2 */
    double energyTolerance;    /* 2e-4 */
    int    maximumSCFCycles;   /* 100 */
    int    history;            /* 10 */
    int    useRCA;             /* 1 */
} OracleSCFOptions;

/* Opaque handles. */
typedef struct OracleHamiltonian OracleHamiltonian;

OracleHamiltonian *oracle_hamiltonian_create(int nElements, const int *atomicNumbers, const int *norbitals,
                                             const double *raw, const int *nGaussians, const double *gaussians,
                                             const int *nPDDG, const double *pddg, const int *nShells,
                                             const int *shellTypes, const int *nPrimitives,
                                             const double *exponents, const double *coefficients,
                                             const int *nDiatomic, const double *diatomic);
void oracle_hamiltonian_free(OracleHamiltonian *h);

/* Derived per-element parameters, same layout as ref_element_derived in ref_shim.c. */
int oracle_element_derived(const OracleHamiltonian *h, int e, double *out);

/* Energy + gradient of one QC region.
 *   xyz            nAtoms*3 Angstrom
 *   phi            nAtoms QC/MM potentials (atomic units) or NULL
 *   density        packed N(N+1)/2 in/out: used as the SCF start when *useDensity, else the diagonal guess
 *   energies[8]    total electronic incl. QC/MM, electronic (QC only), nuclear, baseline, qcmm, eocc(0), eoei, etei  (Eh)
 *   gradients      nAtoms*3 in Eh/Bohr (NULL: none)
 *   charges        nAtoms Lowdin charges of the final density (NULL: none)
 * Returns 0 converged, 1 not converged, 4 bad argument. */
int oracle_energy(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz, int charge,
                  const double *phi, const OracleSCFOptions *options, double *density, int useDensity,
                  double *energies, double *gradients, double *charges, int *ncycles, double *oneElectron);

/* Fock matrix (packed) and energies [total electronic, electronic, nuclear] for a given density, no SCF. */
/* Open-shell and fractional-occupancy states (QC only): restricted (total density) or unrestricted (alpha, beta)
 * densities, occupancyType 0 cardinal, 1 fixed fractional, 2 variable fractional (Fermi), nFractional = (HOOs,
 * LUOs, alpha HOOs, alpha LUOs, beta HOOs, beta LUOs).  energies[5] = occupancy energy.  phi (nullable): QC/MM
 * potentials at the QC atoms (a.u.), charges (nullable): the Lowdin charges of the last Fock build.  startA / startB
 * (nullable, packed): start densities in place of the diagonal guess (alpha and beta; startA alone, the total density,
 * when restricted), valid for the DIIS history from the first cycle. */
int oracle_energy_open(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                       double alphaCharge, double betaCharge, int restricted, int occupancyType, const int *nFractional,
                       double fermiBroadening, const double *phi, const OracleSCFOptions *o, double *energies, double *grad,
                       double *charges, double *densityA, double *densityB, int *ncycles, const double *startA,
                       const double *startB);
int oracle_fock(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                const double *phi, const double *density, double *fock, double *energies);

/* Gradients (Eh/Bohr) for a given density, no SCF. */
int oracle_gradients(const OracleHamiltonian *h, int nAtoms, const int *elementIndex, const double *xyz,
                     const double *density, double *gradients);

/* ABFS Delta/Gaussian QC/MM spline tabulation (pMolecule.PairwiseInteraction.pyx:27-112,183-196):
 * x = r^2 (A^2), y in atomic units; returns the number of knots written (<= maxKnots). */
int oracle_abfs_knots(double innerCutoff, double outerCutoff, double width2, int pointDensity,
                      int maxKnots, double *x, double *y);

/* QC/MM potentials (a.u.) and gradients (Eh/Bohr on QC and MM atoms) for given Lowdin charges.
 * model 0: NBModelFull 1/r (NBModelFull.c:392,604); model 1: ABFS spline (PairwiseInteraction.c:542,612). */
int oracle_qcmm(int model, double innerCutoff, double outerCutoff, int nKnots, const double *x, const double *y,
                int nQC, const double *qcxyz, int nMM, const double *mmxyz, const double *mmCharges,
                const double *qcCharges, double *potentials, double *qcGradients, double *mmGradients);

#endif
