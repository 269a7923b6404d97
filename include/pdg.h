/*
 * pdg.h - C ABI of the GB300 (sm_103a) NDDO QC/MM energy + gradient library (libpdg.so).
 *
 * The library replaces pDynamo 1.9.0's C compute core for one path: closed-shell RHF
 * MNDO/AM1/PM3/PDDG/RM1 energy + analytic gradient with Lowdin-charge QC/MM embedding, as driven by
 * QCModel.Energy (pMolecule-1.9.0/extensions/pyrex/pMolecule.QCModel.pyx:146-185) and System.Energy
 * (pMolecule-1.9.0/pMolecule/System.py:272-318).  One call evaluates a whole batch of configurations
 * ("frames") of the same QC region: integrals, the complete SCF loop, and gradients, on the device.
 *
 * Conventions
 *   - All pointers named d_* are device pointers (cudaMalloc / torch CUDA tensors); h_* are host.
 *   - The library never allocates or frees caller memory.  Scratch lives in a caller-provided
 *     workspace whose size pdg_workspace_bytes() reports.
 *   - Every function returns a pdg_status.  No exception or C++ type crosses this boundary.
 *   - Work is queued on the stream passed in; functions return before it completes unless stated.
 *   - A pdg_system may be used from one host thread at a time.
 *   - Units: coordinates Bohr, energies Hartree, gradients Hartree/Bohr, potentials Hartree/e.
 *   - Matrices are dense row-major N x N doubles per frame (N = basis functions); basis order per atom
 *     is s, pz, px, py as in pDynamo (pMolecule-1.9.0/extensions/cinclude/MNDODefinitions.h:16-19).
 */
#ifndef PDG_H
#define PDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PDG_OK             = 0,   /* converged / success */
    PDG_NOT_CONVERGED  = 1,   /* SCF hit maximumSCFCycles (pMolecule.QCModel.pyx:177 raises ValueError) */
    PDG_NAN            = 2,   /* non-finite energy or density */
    PDG_DIIS_SINGULAR  = 3,   /* reserved: DIIS never recovered a well-conditioned subspace */
    PDG_BAD_ARGUMENT   = 4,
    PDG_CUDA_ERROR     = 5,
    PDG_TOO_LARGE      = 6,   /* a size exceeds a compiled limit */
    PDG_TENSOR_TIMEOUT = 7    /* a tensor-core completion wait ran out (the frame's SCF was stopped) */
} pdg_status;

/* Per-element parameter record: PDG_ELEMENT_STRIDE doubles, all in atomic units, filled by the host
 * from pDynamo's parameter files (restating pMolecule.MNDOParameters.pyx:309-370 and
 * MNDOParameters.c:155-930).  Offsets: */
#define PDG_ELEMENT_STRIDE 128
enum {
    PDG_E_Z = 0, PDG_E_NORB = 1, PDG_E_ZCORE = 2, PDG_E_ALP = 3, PDG_E_GPHOT = 4, PDG_E_NG = 5, PDG_E_NPDDG = 6,
    PDG_E_DD = 7, PDG_E_QQ = 8, PDG_E_PO = 9 /* 9 values */, PDG_E_GSS = 18, PDG_E_GSP = 19, PDG_E_GPP = 20,
    PDG_E_GP2 = 21, PDG_E_HSP = 22, PDG_E_HPP = 23, PDG_E_BETA = 24 /* 4 */, PDG_E_USPD = 28 /* 4 */,
    PDG_E_FN1 = 32 /* 4 */, PDG_E_FN2 = 36 /* 4 */, PDG_E_FN3 = 40 /* 4 */, PDG_E_PDDGC = 44 /* 4 */,
    PDG_E_PDDGE = 48 /* 4 */, PDG_E_EHEAT = 52, PDG_E_EISOL = 53, PDG_E_NSHELL = 54, PDG_E_NPRIM_S = 55,
    PDG_E_NPRIM_P = 56, PDG_E_EXP_S = 57 /* 6 */, PDG_E_CCBF_S = 63 /* 6 */, PDG_E_EXP_P = 69 /* 6 */,
    PDG_E_CCBF_P = 75 /* 6 */,
    /* PM6: 1 when the element has diatomic core-core pairs; the element's index in the system's element list; the
     * pairs' exponent a (1/bohr) and coefficient x by partner index (0 where the pair has no parameters) */
    PDG_E_DIAT = 81, PDG_E_INDEX = 82, PDG_E_DIAT_A = 84 /* PDG_MAX_ELEMENTS */, PDG_E_DIAT_X = 100 /* PDG_MAX_ELEMENTS */
};

#define PDG_MAX_ELEMENTS 16
#define PDG_MAX_ATOMS    1024
#define PDG_MAX_BASIS    2048

/* SCF options: the DIISSCFConverger keywords (pMolecule.DIISSCFConverger.pyx:140-150;
 * defaults DIISSCFConverger.c:27-32). */
typedef struct {
    double density_tolerance;   /* 1e-8 */
    double energy_tolerance;    /* 2e-4 */
    double diis_onset;          /* 0.2  */
    int    maximum_scf_cycles;  /* 100  */
    int    history;             /* 10, at most 16 */
    int    use_rca;             /* 1: ODA/RCA before DIIS, as the reference default */
    int    density_step;        /* 0: FP64 eigensolve every cycle (the reference's method);
                                   3 or 6: split-BF16 SP2 purification on the tensor cores with that many BF16
                                   partial products accumulated in FP32, for the cycles before the density RMS
                                   change falls below mixed_switch, then the FP64 eigensolve to convergence
                                   (N <= 144; larger systems use the FP64 step throughout). Not in the reference.
                                   3 and 6 (the mixed method) also turn on: perturbative density steps after the
                                   first FP64 step (or from the start, around a shared base: pdg_set_shared_base),
                                   FP32 DIIS commutators, and FP32 sp-sp pair gradient terms (assembled and summed
                                   in FP64) in pdg_energy_gradients / pdg_batch_*. */
    double mixed_switch;        /* RMS density change that ends the purification cycles (e.g. 1e-4) */
} pdg_scf_options;

/* Energy terms returned per frame (PDG_NENERGY doubles). */
#define PDG_NENERGY 8
enum {
    PDG_EN_TOTAL_ELECTRONIC = 0,   /* QC electronic + QC/MM (what the SCF minimises) */
    PDG_EN_ELECTRONIC = 1,         /* QCModelMNDOState eelectronic: tr(PH) + tr(PG)/2 */
    PDG_EN_NUCLEAR = 2,            /* core-core */
    PDG_EN_BASELINE = 3,           /* sum (eheat - eisol) */
    PDG_EN_QCMM = 4,               /* q . phi */
    PDG_EN_ONE_ELECTRON = 5,
    PDG_EN_TWO_ELECTRON = 6,
    PDG_EN_RMS_DENSITY = 7         /* final RMS density change */
};

typedef struct pdg_system pdg_system;

/* Library version (major*10000 + minor*100 + patch). */
int pdg_version(void);

/* Create a QC region.  Replaces the set-up that pDynamo performs in QCModelMNDO.SetUp
 * (pMolecule.QCModelMNDO.pyx:623-672 -> QCModelMNDOState_Setup, QCModelMNDOState.c:477) and
 * QCAtomContainer assignment (pMolecule.QCAtomContainer.pyx:218-278).
 *   h_elements     n_elements * PDG_ELEMENT_STRIDE doubles
 *   h_atom_element n_atoms indices into h_elements
 *   charge         total QC charge (closed shell: nuclear charge - charge must be even) */
int pdg_system_create(const double *h_elements, int n_elements, int n_atoms, const int *h_atom_element,
                      int charge, pdg_system **out);
int pdg_system_destroy(pdg_system *sys);

/* Basis functions, occupied orbitals and atom-pair count of a system. */
int pdg_system_info(const pdg_system *sys, int *n_basis, int *n_occupied, int *n_pairs);

/* Workspace bytes needed for a batch of n_frames. */
size_t pdg_workspace_bytes(const pdg_system *sys, int n_frames);

/* Energy and gradient for a batch of frames.  One call does what one System.Energy(doGradients=True)
 * does for the QC part of each frame: QCModelMNDO_Integrals (QCModelMNDO.c:1032), the SCF loop of
 * QCModel.Energy with QCModelMNDO_Fock (:700), QCModelMNDO_QCMMFockLowdin (:1808) and the
 * DIISSCFConverger (DIISSCFConverger.c:147-770), then QCModelMNDO_Gradients (:732).
 *   d_xyz        n_frames * n_atoms * 3 (Bohr)
 *   d_phi        n_frames * n_atoms QC/MM potentials at the QC atoms, or NULL (no QC/MM)
 *   d_density    n_frames * N * N: in = start density when use_density != 0 (the reference keeps the
 *                previous density on the configuration, pMolecule.QCModel.pyx:153), else the diagonal
 *                guess (QCOnePDM.c:280); out = converged density.  use_density 1: a density the converger
 *                takes into its DIIS history at once (the previous converged one); 2: a start guess (a
 *                predicted density, not idempotent), from which the first Fock matrix is built and which the
 *                first density step replaces before DIIS starts, as the diagonal guess is
 *   d_energies   n_frames * PDG_NENERGY
 *   d_gradients  n_frames * n_atoms * 3 (Eh/Bohr) or NULL
 *   d_charges    n_frames * n_atoms Lowdin charges of the final density, or NULL
 *   d_status     n_frames pdg_status values (PDG_OK or PDG_NOT_CONVERGED / PDG_NAN)
 *   d_ncycles    n_frames SCF cycle counts, or NULL */
int pdg_energy_gradients(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_phi,
                         const pdg_scf_options *options, double *d_density, int use_density,
                         double *d_energies, double *d_gradients, double *d_charges, int *d_status,
                         int *d_ncycles, void *d_workspace, size_t workspace_bytes, void *stream);

/* The SCF alone, on the integrals a previous pdg_energy_gradients / pdg_one_electron / pdg_fock call left
 * in this workspace for the same frames and geometry (QCModel.Energy's loop, pMolecule.QCModel.pyx:160-170,
 * without QCModelMNDO_Integrals): e.g. to converge again with other options or other QC/MM potentials.
 * Arguments as pdg_energy_gradients; no gradients. */
int pdg_scf(pdg_system *sys, int n_frames, const double *d_phi, const pdg_scf_options *options, double *d_density,
            int use_density, double *d_energies, double *d_charges, int *d_status, int *d_ncycles,
            void *d_workspace, size_t workspace_bytes, void *stream);

/* Spin-unrestricted (UHF) energies and gradients, cardinal occupancies, the FP64 method (density_step 0):
 * QCModelMNDO with isSpinRestricted False (pMolecule.QCModelMNDO.pyx; QCModelMNDO_Fock over the alpha and beta
 * density sets, QCModelMNDO.c:700-730, MakeFockG with each spin's density for the exchange, MNDOIntegrals.c:51-143;
 * DIISSCFConverger.c:385-760 over both sets; QCModelMNDO_Gradients with the spin density's exchange terms,
 * QCModelMNDOState.c:178-260).  n_alpha + n_beta = the system's electrons, n_alpha >= n_beta.
 *   d_density     n_frames * 2 * N * N: alpha then beta of each frame (in: start densities when use_density != 0;
 *                 out: converged)
 *   d_total_spin  n_frames * N * N total densities, then n_frames * N * N spin densities (alpha - beta) of the
 *                 converged states (written when d_gradients is given)
 *   d_energies    as pdg_energy_gradients ([5] tr(P H) and [6] the two-electron energy summed over the spins)
 *   workspace     pdg_uhf_workspace_bytes(sys, n_frames, n_alpha, n_beta)
 * Other arguments as pdg_energy_gradients. */
size_t pdg_uhf_workspace_bytes(pdg_system *sys, int n_frames, int n_alpha, int n_beta);

/* Occupancies of the open-shell / fractional-occupancy SCF (QCModelMNDO's isSpinRestricted, occupancyType,
 * numberFractional*HOOs / LUOs and fermiBroadening options; the alpha and beta charges as
 * QCModel.CrossCheckModelAndState forms them, pMolecule.QCModel.pyx:91-140). */
enum { PDG_OCC_CARDINAL = 0, PDG_OCC_FIXED_FRACTIONAL = 1, PDG_OCC_VARIABLE_FRACTIONAL = 2 };
typedef struct {
    int spin_restricted;       /* 1: one density set (the total density, occupancy 2 per orbital); 0: alpha and beta */
    int occupancy_type;        /* PDG_OCC_* */
    double alpha_charge;       /* electrons of each spin; alpha + beta = the system's electrons */
    double beta_charge;
    int n_fractional[6];       /* fixed fractional: HOOs, LUOs (restricted), alpha HOOs, alpha LUOs, beta HOOs, beta LUOs */
    double fermi_broadening;   /* variable fractional: beta of the Fermi-Dirac occupancies (1 / Hartree) */
} pdg_occupancy;

/* Open-shell and fractional-occupancy energies and gradients (QCModelMNDO with isSpinRestricted and occupancyType;
 * QCOnePDM_MakeFromFock with the occupancies, QCOnePDM.c:403-460 and :505-599), the FP64 method: spin-restricted or
 * unrestricted, cardinal, fixed fractional or variable fractional occupancies.  The electronic energy includes the
 * occupancy energy of variable fractional occupancies, d_energies[1] - [5] - [6].
 *   d_density     n_frames * n_sets * N * N (n_sets 1 when spin_restricted: the total density; else alpha then beta)
 *   d_total_spin  unrestricted: as pdg_energy_gradients_uhf; restricted: unused
 *   workspace     pdg_open_workspace_bytes(sys, n_frames)
 * Invalid occupancies (a cardinal count that is not whole, fractional orbitals outside 1..occupied and 0..virtual,
 * charges that do not add up to the electrons or exceed the orbitals) return PDG_BAD_ARGUMENT.  Other arguments as
 * pdg_energy_gradients_uhf, which is this call with unrestricted cardinal occupancies. */
size_t pdg_open_workspace_bytes(pdg_system *sys, int n_frames);
int pdg_energy_gradients_open(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_phi, const pdg_scf_options *options,
                              const pdg_occupancy *occupancy, double *d_density, int use_density, double *d_energies,
                              double *d_gradients, double *d_charges, int *d_status, int *d_ncycles, double *d_total_spin,
                              void *d_workspace, size_t workspace_bytes, void *stream);
int pdg_energy_gradients_uhf(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_phi, const pdg_scf_options *options,
                             int n_alpha, int n_beta, double *d_density, int use_density, double *d_energies, double *d_gradients,
                             double *d_charges, int *d_status, int *d_ncycles, double *d_total_spin, void *d_workspace,
                             size_t workspace_bytes, void *stream);

/* Shared base of the mixed method's perturbative density steps (no counterpart in the reference; it stands where
 * the reference would call the FP64 eigensolver, QCOnePDM_MakeFromFock, QCOnePDM.c:403, for every frame).
 * Every FP64 density step of the mixed method leaves a base in its frame's workspace: the Fock matrix F0 and
 * density P0 it was made from, its wanted eigenvectors and their complement (FP32) and the reciprocal eigenvalue
 * gaps.  A perturbative step solves the block-diagonalisation (Riccati) equation for a nearby Fock matrix in the
 * basis of those vectors, in FP32 products whose factors are small, and falls back to an FP64 step when |K|
 * reaches 0.15 around a shared base (2e-3 around a frame's own).  pdg_base_capture copies frame `frame`'s base (pdg_base_bytes bytes, 16-byte aligned) out of the
 * workspace of the last mixed-method call; pdg_set_shared_base(sys, d_base) makes later mixed-method calls on
 * this system (pdg_energy_gradients, pdg_scf) start every frame from it: the start density is P0 (when
 * use_density is 0) and every density step is a perturbative step around it (no purification, no FP64 step)
 * until one fails, after which that frame takes FP64 steps and bases of its own.  The base must come from the
 * same QC region (basis, electron count) and stay valid until the calls that use it have run; NULL detaches it.
 * The converged results do not depend on the base: it changes the path, not the fixed point. */
/* A side stream for pdg_energy_gradients (NULL detaches it): work the caller queued on it before the call (the
 * QC/MM potentials) overlaps the integrals and the SCF waits for it; work queued on it after the call (the QC/MM
 * gradients) waits for the SCF and overlaps the pair gradients.  The caller makes its main stream wait for the
 * side stream before using those results.  System.Energy's order (QC/MM potentials, integrals, SCF, gradients,
 * QC/MM gradients; pMolecule/System.py:309-312) is kept for every data dependence. */
int pdg_set_side_stream(pdg_system *sys, void *side_stream);
size_t pdg_base_bytes(pdg_system *sys);
int pdg_base_capture(pdg_system *sys, int n_frames, int frame, const void *d_workspace, size_t workspace_bytes, void *d_base,
                     void *stream);
int pdg_set_shared_base(pdg_system *sys, const void *d_base);

/* One density step for given Fock matrices d_fock (n_frames * N * N): d_density (in: the previous density,
 * out: the density of the n_occ lowest eigenvectors) by the FP64 eigensolve (density_step 0) or by split-BF16
 * purification (3 or 6 partial products; N <= 144).  d_energies[PDG_EN_RMS_DENSITY] gets the RMS change. */
int pdg_density(pdg_system *sys, int n_frames, const double *d_fock, int density_step, double *d_density,
                double *d_energies, int *d_status, void *d_workspace, size_t workspace_bytes, void *stream);

/* Diagnostics for parity tests: the one-electron matrix H (n_frames * N * N) and the Fock matrix
 * F = H + G(P) - phi for given densities (QCModelMNDO_Fock + QCMMFockLowdin on one density), with
 * the energies of that density in d_energies. */
int pdg_one_electron(pdg_system *sys, int n_frames, const double *d_xyz, double *d_h,
                     void *d_workspace, size_t workspace_bytes, void *stream);
int pdg_fock(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_phi, const double *d_density,
             double *d_fock, double *d_energies, void *d_workspace, size_t workspace_bytes, void *stream);
/* Gradients (Eh/Bohr) for given densities, no SCF (QCModelMNDO_Gradients on a fixed density). */
int pdg_gradients(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_density,
                  double *d_gradients, void *d_workspace, size_t workspace_bytes, void *stream);

/* pdg_gradients without a workspace: the same gradients (Eh/Bohr) for given densities, with the
 * scratch held in the library itself, so the call allocates no device memory.  For callers that may
 * not allocate at call time: an MD or Monte Carlo inner step that must not synchronise the device
 * (cudaMalloc and cudaFree can), or a host application whose own allocator already owns the device
 * memory and gives the library none.  No counterpart in the reference (QCModelMNDO_Gradients,
 * QCModelMNDO.c:732, needs no scratch on the CPU).
 *   - Limit: n_frames * n_pairs * 3 <= 524288 doubles (4 MiB; e.g. 65 atoms = 2080 pairs: 84 frames);
 *     larger requests return PDG_TOO_LARGE with the sizes in pdg_last_error().
 *   - The scratch is one buffer per device: calls that overlap in time on the same device (two streams,
 *     or two host threads) race on it and give wrong gradients; serialise them.
 *   - The first call on each device looks the buffer's address up (cudaGetSymbolAddress, with that
 *     device current); make that first call before any stream capture.
 *   - Nothing in the scratch has to start at zero: every element read is written first in the call. */
int pdg_gradients_static_scratch(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_density,
                                 double *d_gradients, void *stream);

/* Device time of each phase of pdg_energy_gradients, for profiling.  pdg_phase_events(sys, 1) makes every later
 * pdg_energy_gradients call on sys record four CUDA events on its stream (before the integrals, after them, after
 * the SCF kernel, after the gradient kernels; 0 stops it).  pdg_phase_times waits for the last call's events and
 * writes h_ms[3]: the integral kernels, the SCF kernel and the gradient kernels, in milliseconds.  The device
 * counterpart of the reference's per-phase timings (pMolecule.QCModel.pyx:208-275, EnergyWithTimings: QC
 * Initialize, the converger, QC Gradients). */
int pdg_phase_events(pdg_system *sys, int enable);
int pdg_phase_times(const pdg_system *sys, float *h_ms);

/* Per-phase SCF timings of the last pdg_energy_gradients call that used this workspace: for every frame
 * PDG_NTIMERS GPU clock-cycle counts (clock64 of the frame's CTA), the device counterpart of the phase
 * timings of pMolecule.QCModel.pyx:208-275 (EnergyWithTimings: QC Fock, QC Converger Iterate,
 * QC Converger Densities), with the density step split into its parts.  d_out: n_frames * PDG_NTIMERS. */
#define PDG_RMS_HISTORY 40
#define PDG_NTIMERS (39 + PDG_RMS_HISTORY)
enum {
    PDG_T_FOCK = 0, PDG_T_DIIS_SAVE = 1, PDG_T_ITERATE = 2, PDG_T_TRIDIAGONAL = 3, PDG_T_EIGENVALUES = 4,
    PDG_T_EIGENVECTORS = 5, PDG_T_BACKTRANSFORM = 6, PDG_T_DENSITY = 7, PDG_T_TOTAL = 8, PDG_T_CYCLES = 9,
    PDG_T_ROUNDS = 10,         /* counts, not cycles: inverse-iteration rounds (largest eigenvalue cluster) summed over density steps */
    PDG_T_DENSITY_STEPS = 11,  /* FP64 density steps */
    PDG_T_PURIFICATION = 12,   /* cycles of the split-BF16 purification density steps */
    PDG_T_PURIFICATION_STEPS = 13, /* count: purification density steps */
    PDG_T_SP2_ITERATIONS = 14, /* count: SP2 iterations summed over them */
    PDG_T_SM_ID = 15,          /* the SM that ran the frame's CTA */
    PDG_T_START_NS = 16,       /* %globaltimer at the CTA's start and end (ns) */
    PDG_T_END_NS = 17,
    PDG_T_PUR_PRODUCTS = 18,   /* parts of PDG_T_PURIFICATION: tensor-core products from issue to completion, */
    PDG_T_PUR_READOUT = 19,    /* the readout that forms the next iterate and its BF16 parts, */
    PDG_T_PUR_CONTROL = 20,    /* traces and the SP2 step choice, */
    PDG_T_PUR_SETUP = 21,      /* spectral bounds and the parts of the first iterate, */
    PDG_T_PUR_FINISH = 22,     /* and the density from the last iterate */
    PDG_T_PERT = 23,           /* cycles of the perturbative density steps (mixed method), */
    PDG_T_PERT_STEPS = 24,     /* their count, */
    PDG_T_PERT_BASE = 25,      /* the cycles the FP64 steps spent keeping their base (the complement vectors), */
    PDG_T_PERT_FALLBACKS = 26, /* the count of perturbative steps that handed over to an FP64 step, */
    PDG_T_PERT_SWEEPS = 27,    /* the count of their fixed-point sweeps, and their cycles in: */
    PDG_T_PERT_COUPLING = 28,  /* the coupling blocks E, L', M' from dF, */
    PDG_T_PERT_SOLVE = 29,     /* the fixed-point sweeps, */
    PDG_T_PERT_DENSITY = 30,   /* the new density */
    PDG_T_DIIS_PACK = 31,      /* parts of PDG_T_DIIS_SAVE: P and F into the history, */
    PDG_T_DIIS_COMMUTATOR = 32,/* the error vector F P - P F, */
    PDG_T_DIIS_DOTS = 33,      /* its products with the stored error vectors (the B-matrix row); */
    PDG_T_ITER_EXTRAPOLATE = 34, /* parts of PDG_T_ITERATE: the DIIS solve and extrapolation of P and F, */
    PDG_T_ITER_RCA = 35,       /* the ODA (RCA) step and the copies of P and F it keeps */
    PDG_T_DIIS_COMMUTATOR_FULL = 36, /* the part of PDG_T_DIIS_COMMUTATOR spent on full products F P (after a
                                  purification step, or from a caller's start density) */
    PDG_T_RMS_HISTORY = 37,    /* PDG_RMS_HISTORY entries: RMS density change of each density step, in SCF cycle
                                  order, negative for purification steps, 0 beyond the last */
    PDG_T_PERT_KMAX = 37 + PDG_RMS_HISTORY,       /* largest max |K| of a perturbative step that was taken */
    PDG_T_PERT_FAIL_K = 38 + PDG_RMS_HISTORY      /* max |K| of the last perturbative step that handed over (negative
                                                     when its fixed-point sweeps had not settled), 0 if none */
};
int pdg_scf_timings(const pdg_system *sys, int n_frames, const void *d_workspace, size_t workspace_bytes,
                    double *d_out, void *stream);

/* QC/MM electrostatics with MM point charges.
 * model 0: NBModelFull, plain 1/r over all pairs (NBModelFull.c:604 potentials, :392 gradients).
 * model 1: NBModelABFS Delta/Gaussian spline in r^2 with outer cutoff (PairwiseInteraction.c:612, :542);
 *          the spline is given by n_knots knots d_knots = [x (A^2) | y (a.u.) | y'' (second derivatives)].
 * Coordinates here are in Angstrom, as the reference evaluates these pair terms in Angstrom.
 *   d_qc_xyz  n_frames * n_qc * 3,  d_mm_xyz n_frames * n_mm * 3,  d_mm_charges n_mm (shared by frames)
 *   d_phi     out n_frames * n_qc potentials (a.u.)
 *   d_workspace  at least pdg_qcmm_workspace_bytes(n_frames, n_mm) bytes, 256-byte aligned: each call first lists,
 *             per frame, the MM atoms within the cutoff of any QC atom (in MM index order; the pair-list step of the
 *             reference, whose cell-grid lists, PairListGenerator.c:414, serve the same purpose), and the pair
 *             kernels scan that list.  Nothing in it is read before it is written; it need not persist between calls. */
size_t pdg_qcmm_workspace_bytes(int n_frames, int n_mm);
int pdg_qcmm_potentials(int model, int n_frames, int n_qc, int n_mm, const double *d_qc_xyz,
                        const double *d_mm_xyz, const double *d_mm_charges, int n_knots, const double *d_knots,
                        double outer_cutoff, double *d_phi, void *d_workspace, size_t workspace_bytes, void *stream);
/* Gradients (Eh/Bohr) of q_A phi_A with respect to QC and MM coordinates for given QC charges.
 * d_qc_grad (n_frames*n_qc*3) and d_mm_grad (n_frames*n_mm*3) are overwritten; d_mm_grad may be NULL, and the
 * MM-side gradients are then not computed (dynamics with the MM atoms fixed never uses them).
 * model | PDG_QCMM_FP32_PAIRS evaluates the pair terms in FP32 (per-atom sums in FP64; errors ~1e-7 Hartree/Bohr,
 * used by the mixed method; the reference's arithmetic is FP64, which is the default here).  Workspace as above. */
#define PDG_QCMM_FP32_PAIRS 0x100
int pdg_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *d_qc_xyz,
                       const double *d_mm_xyz, const double *d_mm_charges, const double *d_qc_charges,
                       int n_knots, const double *d_knots, double outer_cutoff,
                       double *d_qc_grad, double *d_mm_grad, void *d_workspace, size_t workspace_bytes, void *stream);

/* Learned start density (no counterpart in the reference, whose SCF starts from the diagonal guess,
 * QCOnePDM.c:280, or from the previous density).  A per-atom-pair MLP (64 features -> 256 -> 256 -> 16, SiLU,
 * BF16 weights, FP32 accumulation) predicts, for every pair closer than 3.5 A, its density block and
 * one-centre contributions in the pair's local frame; pdg_guess_assemble rotates them into a start density.
 * Rows (pairs) of all frames are stored consecutively; *d_rows-style arguments point at the device count
 * (d_offsets[n_frames]), and max_rows = n_frames * n_pairs bounds every buffer.
 *   pdg_guess_features  d_xyz (Angstrom, n_frames * n_atoms * 3), d_phi (QC/MM potentials or NULL) ->
 *                       d_env (n_frames * n_atoms * 8), d_count (n_frames), d_offsets (n_frames + 1),
 *                       d_x (max_rows * 64), d_row_frame, d_row_pair (max_rows)
 *   pdg_mlp_forward     d_h = act(d_x W^T + b) (act 1: SiLU, 0: none), d_z = the pre-activation (or NULL);
 *                       W n x k BF16, rows x k in, rows x n out
 *   pdg_mlp_backward    d_dzin = (d_dz W) * SiLU'(d_zin) (if d_dzin), and per row segment the weight and bias
 *                       gradients d_part[segments][n][k + 1] from d_dz and the layer input d_hin
 *   pdg_mlp_adam        Adam step on the FP32 master weights d_wm (n x k) and biases d_bm (n) from the summed
 *                       segment gradients times scale; refreshes the BF16 weights d_w
 *   pdg_guess_assemble  start densities d_density (n_frames * N * N) from the outputs d_y (max_rows * 16)
 *   pdg_guess_loss      squared error of the assembled blocks against d_target; d_dy (max_rows * 16) its
 *                       gradient with respect to the outputs, d_loss (n_frames) */
int pdg_guess_features(pdg_system *sys, int n_frames, const double *d_xyz, const double *d_phi, float *d_env, int *d_count,
                       int *d_offsets, float *d_x, int *d_row_frame, int *d_row_pair, void *stream);
int pdg_mlp_forward(int max_rows, const int *d_rows, int k, int n, const float *d_x, const void *d_w, const float *d_b,
                    float *d_z, float *d_h, int act, void *stream);
int pdg_mlp_backward(int max_rows, const int *d_rows, int n, int k, const float *d_dz, const void *d_w, const float *d_zin,
                     const float *d_hin, float *d_dzin, int segments, float *d_part, void *stream);
int pdg_mlp_adam(int n, int k, int segments, const float *d_part, float scale, float *d_wm, float *d_bm, float *d_m1, float *d_m2,
                 void *d_w, float lr, float beta1, float beta2, int step, void *stream);
int pdg_guess_assemble(pdg_system *sys, int n_frames, const double *d_xyz, const int *d_offsets, const int *d_row_pair,
                       const float *d_y, double *d_density, void *stream);
int pdg_guess_loss(pdg_system *sys, int n_frames, const double *d_xyz, const int *d_offsets, const int *d_row_pair,
                   const double *d_density, const double *d_target, float *d_dy, double *d_loss, void *stream);

/* Check of the tensor-core (tcgen05) split-BF16 product used by the purification density step:
 * d_c = X X for a symmetric n x n FP32 matrix d_x (n <= 144), with kprod = 1, 3 or 6 BF16 partial
 * products accumulated in FP32.  d_status (one int) is 0, or 1 when the tensor-core completion wait ran out
 * after wait_limit polls of its mbarrier (wait_limit <= 0: the limit the SCF kernel uses, 2^22).
 * kprod = 0 checks that bounded wait alone: no tensor-core operation is issued (no allocation, no product), the
 * kernel waits wait_limit polls on a barrier nothing arrives on and writes status 1; d_x and d_c may be NULL.
 * No counterpart in the reference (its density step is an FP64 eigensolve). */
int pdg_tc_selftest(int n, int kprod, int wait_limit, const float *d_x, float *d_c, int *d_status, void *stream);

/* Launch configuration of the SCF kernel for this system on the current device: threads per CTA (one CTA
 * per frame), dynamic shared memory per CTA, and the CUDA runtime's occupancy estimate in CTAs per SM (the
 * SM id and start/end times each CTA records in pdg_scf_timings show what the hardware actually ran). */
int pdg_scf_occupancy(const pdg_system *sys, int *threads, int *smem_bytes, int *ctas_per_sm);

/* ---- Heterogeneous batches: independent molecules of different sizes, computed together ----
 * A batch is a list of items, each a system with one geometry (the same system may appear for several
 * items).  Per-item data are concatenated in item order: d_xyz, d_gradients (3 per atom, Bohr and
 * Hartree/Bohr), d_phi and d_charges (1 per atom), d_density (N_k^2 per item), d_energies
 * (PDG_NENERGY per item), d_status and d_ncycles (1 per item).  pdg_batch_energy_gradients queues one
 * launch per kernel over the whole batch: integrals, a persistent SCF kernel whose CTAs take items from a
 * queue (largest first), gradients.  The reference evaluates one molecule per QCModel.Energy call
 * (pMolecule.QCModel.pyx:146-185); its batched counterpart is a Python loop over systems. */
typedef struct pdg_batch pdg_batch;
typedef struct pdg_graph pdg_graph;

int pdg_batch_create(pdg_system *const *systems, int n_items, pdg_batch **out);
int pdg_batch_destroy(pdg_batch *batch);
/* n_items, total atoms, total density doubles, and the SCF launch the schedule gives: persistent CTAs, threads
 * per CTA, dynamic shared memory per CTA, items that can use the tensor-core purification step (256-thread
 * variant, N <= 144, matrix in shared memory). */
int pdg_batch_info(const pdg_batch *batch, int *n_items, int *n_atoms, long long *density_doubles, int *grid, int *threads,
                   int *smem_bytes, int *tensor_items);
size_t pdg_batch_workspace_bytes(const pdg_batch *batch);
/* Schedule of the persistent SCF kernel (the autotuner's knobs): threads 256 with ctas_per_sm 2 (112 KB of
 * shared memory each) or 1 (220 KB), or threads 512 with ctas_per_sm 1 (FP64 steps only; all of an SM's warps
 * on one molecule); order 0 = largest item first, 1 = item order. */
int pdg_batch_schedule(pdg_batch *batch, int threads, int ctas_per_sm, int order);
int pdg_batch_energy_gradients(pdg_batch *batch, const double *d_xyz, const double *d_phi, const pdg_scf_options *options,
                               double *d_density, int use_density, double *d_energies, double *d_gradients,
                               double *d_charges, int *d_status, int *d_ncycles, void *d_workspace, size_t workspace_bytes,
                               void *stream);
/* Per-item SCF phase timings of the last batch call, PDG_NTIMERS doubles per item (as pdg_scf_timings). */
int pdg_batch_timings(const pdg_batch *batch, const void *d_workspace, size_t workspace_bytes, double *d_out, void *stream);
/* The same work captured once into a CUDA graph on the given buffers (a queue reset and five kernel launches);
 * pdg_graph_launch replays it on a stream.  The buffers must outlive the graph.  No reference counterpart. */
int pdg_batch_graph_create(pdg_batch *batch, const double *d_xyz, const double *d_phi, const pdg_scf_options *options,
                           double *d_density, int use_density, double *d_energies, double *d_gradients,
                           double *d_charges, int *d_status, int *d_ncycles, void *d_workspace, size_t workspace_bytes,
                           pdg_graph **out);
int pdg_graph_launch(pdg_graph *graph, void *stream);
int pdg_graph_destroy(pdg_graph *graph);

/* ---- Langevin dynamics of independent replicas (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py) ----
 * The replicas are copies of one QC region in a fixed MM environment (System.DefineFixedAtoms on the MM atoms;
 * this library has no MM force field).  Coordinates d_xyz: n_replicas x n_atoms x 3 (Angstrom, the QC atoms in
 * the order the energy kernels take them); free atom f is atom d_free_atoms[f]; velocities and accelerations
 * n_replicas x n_free x 3 in A/ps and A/ps^2.  factors = {facR1, facR2, facV1, facV2, sdR, sdV1, sdV2}, the
 * integration constants of CalculateIntegrationConstants (:63-112; sdR, sdV1, sdV2 times
 * sqrt(T / _AMUA2PS2_TO_K)), in the reference's mass-weighted units.
 *   pdg_langevin_positions   the first half of Iteration (:126-137 and RandomForces :147-157): positions, half
 *                            velocities, random forces from Philox4x32-10 normal deviates for (seed, element,
 *                            step); d_deviates (NULL or n_replicas x n_free x 3 x 2) receives (w1, w2) per element.
 *                            random = 0 applies no random forces; random = 2 reads the deviates from d_deviates
 *                            instead (deviates with the linear constraints projected out, below).
 *   pdg_langevin_velocities  the second half (:139-144): accelerations a = -100 grad_scale (g_a + g_b) / m from the
 *                            gradients at the new point (rows d_grad_rows[f] of n_replicas x n_rows x 3 arrays;
 *                            d_grad_b may be NULL; grad_scale converts them to kJ/mol/A), v += facV3 a, and per
 *                            replica d_mv2 = sum m v^2 (amu A^2 ps^-2; NULL to skip), from which the host forms
 *                            the kinetic energy and temperature (SystemGeometryObjectiveFunction.py:255-260). */
int pdg_langevin_positions(int n_replicas, int n_atoms, int n_free, const int *d_free_atoms, const double *d_inv_sqrt_mass,
                           double *d_xyz, double *d_velocities, const double *d_accelerations, const double *h_factors, int random,
                           unsigned long long seed, unsigned int step, double *d_deviates, void *stream);
int pdg_langevin_velocities(int n_replicas, int n_free, int n_rows, const int *d_grad_rows, const double *d_mass,
                            const double *d_grad_a, const double *d_grad_b, double grad_scale, double facV3,
                            double *d_velocities, double *d_accelerations, double *d_mv2, void *stream);
/* Linear constraints of the dynamics (SystemGeometryObjectiveFunction.ApplyLinearConstraints / GradientsGet /
 * VelocitiesAssign, pMolecule-1.9.0/pMolecule/SystemGeometryObjectiveFunction.py:99-101, :177-183, :317-345, through
 * Real2DArray.ProjectOutOfArray): for each replica, x_w -= V (V^T x_w) where x_w = s x is the mass-weighted form of
 * the array and V the replica's n_vectors (1..6) orthonormal rotation and translation vectors
 * (Coordinates3_RotationTranslationVectors, pCore-1.9.0/extensions/csource/Coordinates3.c:1315; d_vectors
 * n_replicas x n_vectors x n_free x 3).  d_scale: s per free atom (sqrt(m) for velocities, 1/sqrt(m) for
 * gradients, NULL for 1: the deviates).  Element (fa, k, c) of replica r is d_array[((r n_rows + row) 3 + k) width
 * + c], row = d_rows[fa] (d_rows NULL: row fa, n_rows = n_free); width 1 or 2 (the two deviate vectors). */
int pdg_linear_constraints_project(int n_replicas, int n_free, int n_rows, const int *d_rows, int n_vectors, const double *d_vectors,
                                   const double *d_scale, int width, double *d_array, void *stream);
/* n_pairs pairs of standard normal deviates for counters (pair index, step, stream_id) under key seed, the
 * generator pdg_langevin_positions uses (stream_id 0); for tests and for velocity assignment. */
int pdg_normal_deviates(long long n_pairs, unsigned long long seed, unsigned int step, unsigned int stream_id, double *d_out,
                        void *stream);
/* Start density of an SCF as a linear combination d_out = sum_k h_coefficients[k] d_terms[k] of up to 8 device
 * arrays of n doubles (16-byte aligned): the previous step's density (the reference's warm start,
 * pMolecule.QCModel.pyx:153), extrapolations over earlier steps, learned corrections.  No counterpart in the
 * reference beyond the warm start. */
int pdg_density_combine(long long n, int count, const double *const *h_terms, const double *h_coefficients, double *d_out,
                        void *stream);

/* ---- MM/MM and QC/MM Lennard-Jones energies of NBModelABFS ----
 * Replace NBModelABFS_MMMMEnergy and NBModelABFS_QCMMEnergyLJ (pMolecule-1.9.0/extensions/csource/NBModelABFS.c:228,
 * :306) with PairwiseInteractionABFS_MMMMEnergy in its default analytic form (PairwiseInteraction.c:292) over the
 * pair lists of GenerateLists / GenerateLists14 (NBModelABFS.c:1050-1160), which the reference's cell-grid
 * generator makes (pCore-1.9.0/extensions/csource/PairListGenerator.c:414-530); here a cell grid is rebuilt on the
 * device for every call.  No symmetry images.
 *   pdg_mm_create  the MM side of a system (host arrays, copied): per atom the charge (e), LJ type and flags
 *                  (1 an active MM atom, 2 a QC atom with LJ interactions, 4 fixed: pairs of two fixed atoms are
 *                  left out, as the reference's free-atom selection does); LJ tables A and B (n_lj_types^2, full,
 *                  symmetric; kJ/mol A^12 and kJ/mol A^6: E = A / r^12 - B / r^6) and the 1-4 tables; exclusion
 *                  pairs and 1-4 pairs (i, j); the ABFS cutoffs (A), the dielectric and electrostaticScale14.
 *   pdg_mm_energy_gradients  for n_frames frames of d_xyz (n_frames x n_atoms x 3, A): d_energies n_frames x 6 in
 *                  kJ/mol (MM/MM Elect., MM/MM LJ, MM/MM 1-4 Elect., MM/MM 1-4 LJ, QC/MM LJ, QC/MM 1-4 LJ, the
 *                  labels of NBModelABFSState.GetEnergies, pMolecule.NBModelABFSState.pyx:41-52) and, unless NULL,
 *                  d_gradients n_frames x n_atoms x 3 in kJ/mol/A (overwritten; zero on atoms without terms). */
typedef struct pdg_mm_system pdg_mm_system;
int pdg_mm_create(int n_atoms, const double *h_charges, const int *h_lj_types, const unsigned char *h_flags, int n_lj_types,
                  const double *h_table_a, const double *h_table_b, const double *h_table_a14, const double *h_table_b14,
                  int n_exclusions, const int *h_exclusions, int n_pairs14, const int *h_pairs14, double inner_cutoff,
                  double outer_cutoff, double damping_cutoff, double dielectric, double electrostatic_scale14,
                  pdg_mm_system **out);
int pdg_mm_destroy(pdg_mm_system *m);
size_t pdg_mm_workspace_bytes(const pdg_mm_system *m, int n_frames);
int pdg_mm_energy_gradients(const pdg_mm_system *m, int n_frames, const double *d_xyz, double *d_energies, double *d_gradients,
                            void *d_workspace, size_t workspace_bytes, void *stream);

/* ---- Harmonic bond and angle terms of an MM model ----
 * Replace HarmonicBondContainer_Energy and HarmonicAngleContainer_Energy (pMolecule-1.9.0/extensions/csource/
 * HarmonicBondContainer.c:149, HarmonicAngleContainer.c:157): E = k (r - r0)^2 per bond and k (theta - theta0)^2 per angle
 * (theta at the middle atom, its cosine clamped to +-0.999999 as the reference does), for many frames.  kJ/mol, Angstrom,
 * radians.  For the flexible waters of MM models that move in dynamics.
 *   pdg_mm_bonded_create   n_atoms; bonds (i, j) with (r0, k); angles (i, j, k), j the apex, with (theta0, k)
 *   pdg_mm_bonded_energy_gradients  for n_frames frames of d_xyz (n_frames x n_atoms x 3): d_energies n_frames x 2 (bond,
 *                          angle), and unless NULL the gradients ADDED to d_gradients (n_frames x n_atoms x 3, kJ/mol/A) */
typedef struct pdg_mm_bonded pdg_mm_bonded;
int pdg_mm_bonded_create(int n_atoms, int n_bonds, const int *h_bonds, const double *h_bond_params, int n_angles,
                         const int *h_angles, const double *h_angle_params, pdg_mm_bonded **out);
int pdg_mm_bonded_destroy(pdg_mm_bonded *bonded);
int pdg_mm_bonded_energy_gradients(const pdg_mm_bonded *bonded, int n_frames, const double *d_xyz, double *d_energies,
                                   double *d_gradients, void *stream);

/* ---- One large QC region over the whole GPU ----
 * pdg_energy_gradients gives each frame one CTA (one SM): the throughput form for many frames of a small region.  A
 * single large region (hundreds of atoms, N up to PDG_MAX_BASIS) is computed here with every SCF phase spread over all
 * SMs: the Fock build and the DIIS/ODA vector work as grid-wide kernels, the FP64 density step as a Householder
 * tridiagonalisation of two grid-wide kernels per column (replayed from a CUDA graph), bisection and inverse iteration
 * for the wanted eigenpairs, and a blocked compact-WY back-transformation and density by DGEMM; the integrals and
 * gradients are the pair kernels of pdg_energy_gradients on this one frame.  The results are those of
 * pdg_energy_gradients for the same frame (QCModel.Energy + EnergyGradients, pMolecule.QCModel.pyx:146-185).
 * options->density_step 0 is the reference's FP64 method; 3 or 6 the mixed method of this path: every FP64 density step
 * keeps a base (its matrix, density and all eigenpairs), and the following steps are perturbative ones around it in FP32
 * products with small factors (scf.cu's perturbative step as SGEMMs), falling back to an FP64 step when the correction
 * is not small (|K| >= 3e-2); the DIIS error is formed in FP32 from the change of F; the sp-sp and sp-s pair gradient terms are FP32.
 * The base stays with the wide engine and its workspace between calls, so a warm-started call (the next MD step) can run
 * perturbative steps from its first cycle.
 *   pdg_wide_create       a wide engine for sys (which must outlive it); holds a cuBLAS handle and, after the first
 *                         call, the tridiagonalisation graph of the workspace it was given
 *   pdg_wide_workspace_bytes   the workspace one call needs (256-byte aligned)
 *   pdg_wide_energy_gradients  one frame, arguments as pdg_energy_gradients with n_frames = 1.  The call waits for the
 *                         stream at every SCF cycle (the host reads the converger's state to decide whether to go on),
 *                         so it returns after the work is done; do not capture it in a CUDA graph. */
typedef struct pdg_wide pdg_wide;
int pdg_wide_create(pdg_system *sys, pdg_wide **out);
int pdg_wide_destroy(pdg_wide *wide);
size_t pdg_wide_workspace_bytes(const pdg_system *sys);
int pdg_wide_energy_gradients(pdg_wide *wide, const double *d_xyz, const double *d_phi, const pdg_scf_options *options,
                              double *d_density, int use_density, double *d_energies, double *d_gradients, double *d_charges,
                              int *d_status, int *d_ncycles, void *d_workspace, size_t workspace_bytes, void *stream);
/* Device time per phase of the last pdg_wide_energy_gradients call (after pdg_wide_phase_events(wide, 1)), in
 * milliseconds: integrals, Fock builds (with the converger's energy test), DIIS/ODA, tridiagonalisation (with the
 * host's read of its bounds), eigenvalues, eigenvectors, back-transformation, density (and the perturbative steps),
 * gradients; then two counts: the call's FP64 density steps and its perturbative steps.  PDG_WIDE_NPHASES values in
 * all.  The counterpart of the reference's phase timings (pMolecule.QCModel.pyx:208-275). */
#define PDG_WIDE_NPHASES 11
int pdg_wide_phase_events(pdg_wide *wide, int enable);
int pdg_wide_phase_times(pdg_wide *wide, float *h_ms);

/* Text of the last error on this host thread (never NULL). */
const char *pdg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
