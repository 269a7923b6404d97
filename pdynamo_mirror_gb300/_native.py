"""ctypes binding of libpdg.so (include/pdg.h).

The CUDA library is the only compute path: importing the energy functions on a machine without the
built library or without a CUDA device raises, there is no CPU fallback.
"""

import ctypes, os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpdg.so")

PDG_OK, PDG_NOT_CONVERGED, PDG_NAN, PDG_DIIS_SINGULAR, PDG_BAD_ARGUMENT, PDG_CUDA_ERROR, PDG_TOO_LARGE, PDG_TENSOR_TIMEOUT = range(8)
NENERGY = 8
EN_TOTAL_ELECTRONIC, EN_ELECTRONIC, EN_NUCLEAR, EN_BASELINE, EN_QCMM, EN_ONE_ELECTRON, EN_TWO_ELECTRON, EN_RMS_DENSITY = range(8)
MAX_HISTORY = 16
QCMM_FP32_PAIRS = 0x100   # pdg_qcmm_gradients model flag: FP32 pair terms (the mixed method)
MM_FLAG_MM, MM_FLAG_QC_LJ, MM_FLAG_FIXED = 1, 2, 4   # pdg_mm_create atom flags
WIDE_PHASES = ("integrals", "fock", "diis", "tridiagonal", "eigenvalues", "eigenvectors", "backtransform", "density", "gradients",
               "fp64_steps", "perturbative_steps")
MM_TERMS = ("MM/MM Elect.", "MM/MM LJ", "MM/MM 1-4 Elect.", "MM/MM 1-4 LJ", "QC/MM LJ", "QC/MM 1-4 LJ", "Harmonic Bond", "Harmonic Angle")

EXPORTS = ("pdg_version", "pdg_system_create", "pdg_system_destroy", "pdg_system_info", "pdg_workspace_bytes",
           "pdg_energy_gradients", "pdg_scf", "pdg_density", "pdg_one_electron", "pdg_fock", "pdg_gradients", "pdg_qcmm_potentials",
           "pdg_qcmm_gradients", "pdg_scf_timings", "pdg_gradients_static_scratch", "pdg_tc_selftest", "pdg_scf_occupancy", "pdg_guess_features", "pdg_mlp_forward",
           "pdg_mlp_backward", "pdg_mlp_adam", "pdg_guess_assemble", "pdg_guess_loss", "pdg_batch_create", "pdg_batch_destroy",
           "pdg_batch_info", "pdg_batch_workspace_bytes", "pdg_batch_schedule", "pdg_batch_energy_gradients", "pdg_batch_timings",
           "pdg_batch_graph_create", "pdg_graph_launch", "pdg_graph_destroy", "pdg_langevin_positions", "pdg_langevin_velocities",
           "pdg_normal_deviates", "pdg_linear_constraints_project", "pdg_density_combine", "pdg_mm_create", "pdg_mm_destroy", "pdg_mm_workspace_bytes",
           "pdg_mm_energy_gradients", "pdg_phase_events", "pdg_phase_times", "pdg_qcmm_workspace_bytes", "pdg_wide_create", "pdg_wide_destroy",
           "pdg_wide_workspace_bytes", "pdg_wide_energy_gradients", "pdg_wide_phase_events", "pdg_wide_phase_times",
           "pdg_mm_bonded_create", "pdg_mm_bonded_destroy", "pdg_mm_bonded_energy_gradients", "pdg_base_bytes",
           "pdg_base_capture", "pdg_set_shared_base", "pdg_set_side_stream", "pdg_uhf_workspace_bytes",
           "pdg_energy_gradients_uhf", "pdg_open_workspace_bytes", "pdg_energy_gradients_open", "pdg_last_error")
TIMERS = ("QC Fock", "QC Converger DIIS Save", "QC Converger Iterate", "QC Densities Tridiagonal", "QC Densities Eigenvalues",
          "QC Densities Eigenvectors", "QC Densities Back-transform", "QC Densities Density", "QC SCF Total", "QC SCF Fock Builds",
          "QC Densities Cluster Rounds", "QC Densities Steps", "QC Densities Purification",
          "QC Densities Purification Steps", "QC Densities SP2 Iterations", "SM", "Start ns", "End ns", "QC Densities Purification Products",
          "QC Densities Purification Readout", "QC Densities Purification Control", "QC Densities Purification Setup",
          "QC Densities Purification Finish", "QC Densities Perturbative", "QC Densities Perturbative Steps",
          "QC Densities Perturbative Base", "QC Densities Perturbative Fallbacks", "QC Densities Perturbative Sweeps",
          "QC Densities Perturbative Coupling", "QC Densities Perturbative Solve", "QC Densities Perturbative Density",
          "QC Converger DIIS Pack", "QC Converger DIIS Commutator", "QC Converger DIIS Dots", "QC Converger Extrapolate",
          "QC Converger RCA", "QC Converger DIIS Commutator Full") + tuple("RMS %d" % k for k in range(40)) + \
         ("QC Densities Perturbative Kmax", "QC Densities Perturbative Failed K")


class SCFOptions(ctypes.Structure):
    _fields_ = [("density_tolerance", ctypes.c_double), ("energy_tolerance", ctypes.c_double),
                ("diis_onset", ctypes.c_double), ("maximum_scf_cycles", ctypes.c_int),
                ("history", ctypes.c_int), ("use_rca", ctypes.c_int), ("density_step", ctypes.c_int),
                ("mixed_switch", ctypes.c_double)]


OCC_TYPES = {"Cardinal": 0, "Fixed Fractional": 1, "Variable Fractional": 2}


class Occupancy(ctypes.Structure):
    """pdg_occupancy: density sets and occupancies of pdg_energy_gradients_open."""
    _fields_ = [("spin_restricted", ctypes.c_int), ("occupancy_type", ctypes.c_int), ("alpha_charge", ctypes.c_double),
                ("beta_charge", ctypes.c_double), ("n_fractional", ctypes.c_int * 6), ("fermi_broadening", ctypes.c_double)]


class NativeError(RuntimeError):
    pass


_lib = None


def load(path=LIB_PATH):
    """Load libpdg.so and declare its signatures (no GPU needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise NativeError("libpdg.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    P, I, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    PP = ctypes.POINTER(ctypes.c_void_p)
    L.pdg_version.restype = I
    L.pdg_last_error.restype = ctypes.c_char_p
    L.pdg_system_create.argtypes = [P, I, I, P, I, PP]
    L.pdg_system_destroy.argtypes = [P]
    L.pdg_system_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]
    L.pdg_workspace_bytes.argtypes = [P, I]
    L.pdg_workspace_bytes.restype = S
    L.pdg_energy_gradients.argtypes = [P, I, P, P, ctypes.POINTER(SCFOptions), P, I, P, P, P, P, P, P, S, P]
    L.pdg_scf.argtypes = [P, I, P, ctypes.POINTER(SCFOptions), P, I, P, P, P, P, P, S, P]
    L.pdg_density.argtypes = [P, I, P, I, P, P, P, P, S, P]
    L.pdg_one_electron.argtypes = [P, I, P, P, P, S, P]
    L.pdg_fock.argtypes = [P, I, P, P, P, P, P, P, S, P]
    L.pdg_gradients.argtypes = [P, I, P, P, P, P, S, P]
    L.pdg_scf_timings.argtypes = [P, I, P, S, P, P]
    L.pdg_phase_events.argtypes = [P, I]
    L.pdg_wide_create.argtypes = [P, PP]
    L.pdg_wide_destroy.argtypes = [P]
    L.pdg_wide_workspace_bytes.argtypes = [P]
    L.pdg_wide_phase_events.argtypes = [P, I]
    L.pdg_wide_phase_times.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
    L.pdg_wide_workspace_bytes.restype = S
    L.pdg_wide_energy_gradients.argtypes = [P, P, P, ctypes.POINTER(SCFOptions), P, I, P, P, P, P, P, P, S, P]
    L.pdg_phase_times.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
    L.pdg_gradients_static_scratch.argtypes = [P, I, P, P, P, P]
    L.pdg_tc_selftest.argtypes = [I, I, I, P, P, P, P]
    L.pdg_scf_occupancy.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]
    F = ctypes.c_float
    L.pdg_guess_features.argtypes = [P, I, P, P, P, P, P, P, P, P, P]
    L.pdg_mlp_forward.argtypes = [I, P, I, I, P, P, P, P, P, I, P]
    L.pdg_mlp_backward.argtypes = [I, P, I, I, P, P, P, P, P, I, P, P]
    L.pdg_mlp_adam.argtypes = [I, I, I, P, F, P, P, P, P, P, F, F, F, I, P]
    L.pdg_guess_assemble.argtypes = [P, I, P, P, P, P, P, P]
    L.pdg_guess_loss.argtypes = [P, I, P, P, P, P, P, P, P, P]
    L.pdg_qcmm_workspace_bytes.argtypes = [I, I]
    L.pdg_qcmm_workspace_bytes.restype = S
    L.pdg_qcmm_potentials.argtypes = [I, I, I, I, P, P, P, I, P, D, P, P, S, P]
    L.pdg_qcmm_gradients.argtypes = [I, I, I, I, P, P, P, P, I, P, D, P, P, P, S, P]
    LL = ctypes.c_longlong
    L.pdg_batch_create.argtypes = [P, I, PP]
    L.pdg_batch_destroy.argtypes = [P]
    L.pdg_batch_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(LL), ctypes.POINTER(I), ctypes.POINTER(I),
                                 ctypes.POINTER(I), ctypes.POINTER(I)]
    L.pdg_batch_workspace_bytes.argtypes = [P]
    L.pdg_batch_workspace_bytes.restype = S
    L.pdg_batch_schedule.argtypes = [P, I, I, I]
    L.pdg_batch_energy_gradients.argtypes = [P, P, P, ctypes.POINTER(SCFOptions), P, I, P, P, P, P, P, P, S, P]
    L.pdg_batch_graph_create.argtypes = [P, P, P, ctypes.POINTER(SCFOptions), P, I, P, P, P, P, P, P, S, PP]
    L.pdg_batch_timings.argtypes = [P, P, S, P, P]
    L.pdg_graph_launch.argtypes = [P, P]
    L.pdg_graph_destroy.argtypes = [P]
    U32, U64 = ctypes.c_uint, ctypes.c_ulonglong
    L.pdg_langevin_positions.argtypes = [I, I, I, P, P, P, P, P, P, I, U64, U32, P, P]
    L.pdg_langevin_velocities.argtypes = [I, I, I, P, P, P, P, D, D, P, P, P, P]
    L.pdg_normal_deviates.argtypes = [LL, U64, U32, U32, P, P]
    L.pdg_linear_constraints_project.argtypes = [I, I, I, P, I, P, P, I, P, P]
    L.pdg_density_combine.argtypes = [LL, I, P, P, P, P]
    L.pdg_mm_create.argtypes = [I, P, P, P, I, P, P, P, P, I, P, I, P, D, D, D, D, D, PP]
    L.pdg_mm_destroy.argtypes = [P]
    L.pdg_mm_bonded_create.argtypes = [I, I, P, P, I, P, P, PP]
    L.pdg_mm_bonded_destroy.argtypes = [P]
    L.pdg_mm_bonded_energy_gradients.argtypes = [P, I, P, P, P, P]
    L.pdg_base_bytes.argtypes = [P]; L.pdg_base_bytes.restype = S
    L.pdg_base_capture.argtypes = [P, I, I, P, S, P, P]
    L.pdg_set_shared_base.argtypes = [P, P]
    L.pdg_set_side_stream.argtypes = [P, P]
    L.pdg_uhf_workspace_bytes.argtypes = [P, I, I, I]; L.pdg_uhf_workspace_bytes.restype = S
    L.pdg_energy_gradients_uhf.argtypes = [P, I, P, P, ctypes.POINTER(SCFOptions), I, I, P, I, P, P, P, P, P, P, P, S, P]
    L.pdg_open_workspace_bytes.argtypes = [P, I]; L.pdg_open_workspace_bytes.restype = S
    L.pdg_energy_gradients_open.argtypes = [P, I, P, P, ctypes.POINTER(SCFOptions), ctypes.POINTER(Occupancy), P, I, P, P, P, P, P, P,
                                            P, S, P]
    L.pdg_mm_workspace_bytes.argtypes = [P, I]
    L.pdg_mm_workspace_bytes.restype = S
    L.pdg_mm_energy_gradients.argtypes = [P, I, P, P, P, P, S, P]
    for name in EXPORTS:
        getattr(L, name).restype = getattr(L, name).restype or I
    _lib = L
    return L


def check(rc, what):
    if rc != PDG_OK:
        msg = load().pdg_last_error().decode()
        raise NativeError("%s failed (status %d): %s" % (what, rc, msg))


def ptr(t):
    """Device (or host) address of a torch tensor or None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle(torch_stream):
    return ctypes.c_void_p(torch_stream.cuda_stream)

