// common.cuh - shared definitions of the GB300 NDDO QC/MM energy + gradient library.
//
// Layout in HBM (one batch of n_frames configurations of one QC region):
//   element table      n_elements * PDG_ELEMENT_STRIDE doubles (atomic units), read through L1
//   atom tables        element index, first basis function, orbital count per atom
//   pair tables        (i, j) for every atom pair i > j, in pDynamo's loop order (QCModelMNDO.c:1047-1063),
//                      and the offset of the pair's two-electron block in the compact per-frame TEI array
//   per-frame arrays   frame-major: everything one frame needs is contiguous, so that the CTA that runs
//                      a frame's SCF streams its own data and nothing else.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/pdg.h"

// SCF CTAs resident per SM (one frame each) and the threads of one SCF CTA.
#ifndef PDG_SCF_CTAS_PER_SM
#define PDG_SCF_CTAS_PER_SM 2
#endif
#define PDG_BLOCK (512 / PDG_SCF_CTAS_PER_SM)
#define PDG_WARPS (PDG_BLOCK / 32)
#define PDG_MAX_HISTORY 16
#define PDG_PAIR_E_STRIDE 24   // e1b[10] | e2a[10] | enuc | spare
#define PDG_TEI_UNDERFLOW 1.0e-12

struct DeviceSystem {
    int n_atoms, n_basis, n_occ, n_pairs, n_elements, n_electrons, tei_total;
    int n_vec, vec_occupied;       // eigenvectors computed per density step: min(n_occ, N - n_occ)
    const double *elements;        // n_elements * PDG_ELEMENT_STRIDE
    const int *atom_elem, *atom_start, *atom_norb;
    const int *pair_i, *pair_j, *pair_tei;   // n_pairs
    const double *terms;           // multipole (o, a) tables per ordered element pair (multipole.cuh)
    const double *ovl;             // overlap primitive records (overlap.cuh), all ordered element pairs
    const int *ovl_off, *ovl_n;    // per ordered element pair: first record, record count
    const int *cel, *xel;          // Fock outputs: diagonal-block elements (atom << 4 | mn), off-diagonal (pair << 4 | ac)
    int n_cel, n_xel;
    const int *pairs_ss, *pairs_gen;   // pairs of two one-orbital (s) atoms, and pairs of two sp atoms, in pair order
    int n_ss, n_gen;
    const int *pairs_sps;              // pairs of one sp and one s atom, in pair order
    int n_sps;
    const void *mp_map;                // MultipoleMap of sp-sp pairs (multipole.cuh)
    const int *atom_pk;                // n_atoms + 1: first entry of each atom's one-centre block in the cel order
    const float *ovl32;                // the overlap primitive records rounded to FP32 (the mixed method's gradients)
    const float *mp_w32;               // the multipole map's weights rounded to FP32 (same layout as MultipoleMap::w)
    // The overlap radial sums tabulated against R (overlap.cuh, overlap_table), for the mixed method only: null in
    // every call of the FP64 method, which sums the primitives
    const double *ovl_tab;
    const int *ovl_tab_off, *ovl_tab_n;   // per ordered element pair: first double, node count
    double ovl_tab_inv_h;
    // spin density (alpha - beta) per frame, at the same offsets as the total density, for the spin-unrestricted
    // gradients; null for closed shells
    const double *spin;
};

// Per-frame workspace plan (all offsets in doubles from the frame's base).
struct FramePlan {
    size_t tei, pair_e, pair_g, H, F, P0, A, G, Z, LU, LO, hP, hF, hE, rP, rF, misc, stride;
    size_t BF, BP, BZ, BL, BW;   // perturbative density steps: base F, P, wanted vectors, eigenvalues, FP32 work (incl. the complement)
    int hist_len;   // packed history vector length N(N+1)/2 (errors use N(N-1)/2 within the same slot)
};

__host__ __device__ inline size_t align32(size_t x) { return (x + 31) & ~size_t(31); }

// FP32 work of a perturbative density step (floats): dF (N x N), dF Z^T (N x kv), E (nc x kv), Lambda' (kv x kv),
// dF V^T (N x nc), M' (nc x nc), K and its next iterate (nc x kv each), E^T K and U (kv x kv each), Y and W
// (kv x N each), dQ (N x N), then (from pert_dq_offset + N^2) the DIIS save's F - F~ (N x N) and the base's
// wanted and complement vectors rounded to FP32 (kv rows of N, then nc rows of N), and the reciprocal eigenvalue
// gaps 1 / (lambda_a - mu_i) (nc x kv).
__host__ __device__ inline size_t pert_work_floats(int N, int kv)
{
    const size_t n = N, k = kv, c = N - kv;
    return 2 * n * n + n * k + n * c + 3 * c * k + 3 * k * k + c * c + 2 * k * n + 64
         + n * n + (k + c) * n    // + dF of the DIIS save (N x N), the base vectors in FP32 (kv + nc rows of N)
         + c * k;                 // + 1 / (lambda_a - mu_i) (nc x kv)
}

// Offset (floats) of dQ in that work.
__host__ __device__ inline size_t pert_dq_offset(int N, int kv)
{
    const size_t n = N, k = kv, c = N - kv;
    return n * n + n * k + c * k + k * k + n * c + c * c + 2 * c * k + 2 * k * k + 2 * k * n;
}

// Offset (floats) of Y (then W) in that work.
__host__ __device__ inline size_t pert_y_offset(int N, int kv) { return pert_dq_offset(N, kv) - 2 * (size_t)kv * N; }

__host__ inline FramePlan make_plan(const DeviceSystem &s, int history)
{
    FramePlan p;
    size_t N = s.n_basis, NN = N * N, o = 0;
    p.hist_len = (int)(N * (N + 1) / 2);
    p.tei = o;    o += align32(s.tei_total);
    p.pair_e = o; o += align32((size_t)s.n_pairs * PDG_PAIR_E_STRIDE);
    p.pair_g = o; o += align32((size_t)s.n_pairs * 3);
    p.H = o;      o += align32(NN);
    p.F = o;      o += align32(NN);
    p.P0 = o;     o += align32(NN);          // F in FP32 (N x round4(N)) for the commutator after a purification step
    p.A = o;      o += align32(2 * NN + 4 * N);  // work matrix: F P product, packed tridiagonal matrix, or the FP32
                                                 // purification iterates (two N x N) and P in FP32 (N x round4(N))
    const size_t kv = s.n_vec > 0 ? s.n_vec : 1, nc = N > kv ? N - kv : 1;
    const size_t kvp = ((nc > kv ? nc : kv) + 31) & ~size_t(31);   // inverse iteration of the wanted vectors or of their complement
    p.G = o;      o += align32(kv * N);      // DIIS: the vectors times F
    p.Z = o;      o += align32(kv * (N | 1)); // wanted eigenvectors when they do not fit in shared memory
    p.LU = o;     o += align32(5 * N * kvp + (N * kvp + 7) / 8);   // inverse iteration factors + iterates
    // BF16 lo parts of the purification iterate (canonical tensor-core layout, R x Kp, R = max(Kp, 128)), N <= 144
    const size_t Kp = (N + 15) & ~size_t(15), Rr = Kp > 128 ? Kp : 128;
    p.LO = o;     o += align32(N <= 144 ? (Rr * Kp * 2 + 7) / 8 : 0);
    p.hP = o;     o += align32((size_t)history * p.hist_len);
    p.hF = o;     o += align32((size_t)history * p.hist_len);
    p.hE = o;     o += align32((size_t)history * p.hist_len);
    p.rP = o;     o += align32(NN);
    p.rF = o;     o += align32(NN);
    p.misc = o;   o += align32(PDG_MAX_HISTORY * PDG_MAX_HISTORY + 96);   // DIIS B matrix, then PDG_NTIMERS phase timers
    // base of the perturbative density steps (mixed method): the Fock matrix and density of the last FP64
    // step, its wanted vectors (FP64, rows of N | 1), all eigenvalues, and FP32 work (which holds the complementary
    // vectors, computed in FP32)
    p.BF = o;     o += align32(NN);
    p.BP = o;     o += align32(NN);
    p.BZ = o;     o += align32(kv * (N | 1));
    p.BL = o;     o += align32(N);
    p.BW = o;     o += align32((pert_work_floats(N, (int)kv) + 1) / 2);
    p.stride = align32(o);
    return p;
}

// Heterogeneous batches: independent molecules of different sizes (each its own system, one geometry each)
// computed by the same launches.  Per-item data are concatenated in item order: coordinates, gradients,
// charges and potentials by atom, densities by N_k^2, workspaces by the item's plan stride.
enum { PDG_WORK_GEN = 0, PDG_WORK_SS = 1, PDG_WORK_ATOM = 2, PDG_WORK_SPS = 3, PDG_WORK_KINDS = 4 };

struct BatchItem {
    DeviceSystem s;
    FramePlan plan;
    long long ws, dens;   // first workspace double, first density double
    int atom;             // first atom
    int work[PDG_WORK_KINDS];   // first global work unit: batches of 32 sp-sp pairs, s-s pairs, atoms, sp-s pairs
};

struct Batch {
    const BatchItem *items;   // device table (null: homogeneous frames of one system)
    int n;
    int total[PDG_WORK_KINDS];   // work units of each kind over all items
};

// What a kernel thread (or warp) works on: the system, plan and data offsets of one frame or batch item
// (s and plan are filled for batch items only; homogeneous frames use the kernel's own arguments).
struct FrameView {
    DeviceSystem s;
    FramePlan plan;
    size_t ws, dens, atom;
    int f;   // frame (homogeneous) or item (batch): index of its energies, status and cycle count
};

__host__ __device__ inline int work_units(const DeviceSystem &s, int kind)
{
    return kind == PDG_WORK_GEN ? (s.n_gen + 31) / 32 : kind == PDG_WORK_SS ? s.n_ss : kind == PDG_WORK_SPS ? s.n_sps : s.n_atoms;
}

// Global work unit g of the given kind -> its frame or item and the unit's index within it; false past the end.
// Batch items are found by binary search on their first units (the last item starting at or before g owns it;
// items with no units of this kind share their start with the next item and are skipped that way).
template <bool BATCH, int KIND>
__device__ __forceinline__ bool locate(const DeviceSystem &s0, const FramePlan &p0, int n_frames, const Batch &b, long g,
                                       FrameView &v, int &local)
{
    if (!BATCH) {
        const int per = work_units(s0, KIND);
        if (per == 0 || g >= (long)n_frames * per) return false;
        v.f = (int)(g / per);
        local = (int)(g % per);
        v.ws = (size_t)v.f * p0.stride;
        v.dens = (size_t)v.f * s0.n_basis * s0.n_basis;
        v.atom = (size_t)v.f * s0.n_atoms;
        return true;
    }
    if (g >= b.total[KIND]) return false;
    int lo = 0, hi = b.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b.items[mid].work[KIND] <= g) lo = mid; else hi = mid - 1;
    }
    const BatchItem &it = b.items[lo];
    v.f = lo;
    local = (int)(g - it.work[KIND]);
    v.s = it.s; v.plan = it.plan;
    v.ws = (size_t)it.ws; v.dens = (size_t)it.dens; v.atom = (size_t)it.atom;
    return true;
}

__device__ __forceinline__ const double *elem(const DeviceSystem &s, int e) { return s.elements + e * PDG_ELEMENT_STRIDE; }
__device__ __forceinline__ int pk(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// Deterministic reductions: fixed thread-to-element assignment, fixed shuffle tree, fixed warp order.
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum; every thread gets the result.  red must hold blockDim.x / 32 doubles.
__device__ __forceinline__ double block_sum(double v, double *red)
{
    v = warp_sum(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < nw; i++) t += red[i];
    __syncthreads();
    return t;
}
// Two block-wide sums at once (the same per-value summation order as block_sum); red must hold 32 doubles.
__device__ __forceinline__ double2 block_sum2(double a, double b, double *red)
{
    a = warp_sum(a); b = warp_sum(b);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) { red[w] = a; red[16 + w] = b; }
    __syncthreads();
    double s = 0.0, t = 0.0;
    for (int i = 0; i < nw; i++) { s += red[i]; t += red[16 + i]; }
    __syncthreads();
    return make_double2(s, t);
}
__device__ __forceinline__ double block_max(double v, double *red)
{
    v = warp_max(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = red[0];
    for (int i = 1; i < nw; i++) t = fmax(t, red[i]);
    __syncthreads();
    return t;
}

// Units (pCore-1.9.0/extensions/cinclude/Units.h:21,55-58).
#define PDG_BOHRS_TO_ANGSTROMS (5.291772083e-11 / 1.0e-10)
#define PDG_ANGSTROMS_TO_BOHRS (1.0e-10 / 5.291772083e-11)

// Kernel launchers (defined in the .cu files, called by api.cu).
void launch_pair_integrals(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *xyz, double *ws, cudaStream_t st);
void launch_assemble_h(const DeviceSystem &s, const FramePlan &p, int n_frames, double *ws, cudaStream_t st);
void launch_pair_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *xyz,
                           const double *density, double *ws, cudaStream_t st, bool fp32_terms = false);
void launch_reduce_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *ws,
                             double *gradients, cudaStream_t st);
// Heterogeneous batches (the same kernels over a BatchItem table).
void launch_batch_integrals(const Batch &b, const double *xyz, double *ws, cudaStream_t st);
void launch_batch_gradients(const Batch &b, const double *xyz, const double *density, double *ws, double *gradients, cudaStream_t st,
                            bool fp32_terms = false);
#define PDG_SMEM_LIMIT_1 (220 * 1024)   // shared-memory budget of one SCF CTA alone on its SM
#define PDG_SMEM_LIMIT_2 (112 * 1024)   // ... of each of two
size_t qcmm_workspace_bytes(int n_frames, int n_mm);
// One large QC region's SCF over the whole GPU (wide.cu).
size_t wide_workspace_bytes(const DeviceSystem &s);
int wide_create(const DeviceSystem &s, pdg_wide **out);
size_t wide_workspace_size(const pdg_wide *W);
int wide_timing(pdg_wide *W, int enable);
int wide_phase_times(pdg_wide *W, float *ms);
void wide_destroy(pdg_wide *W);
int wide_energy_gradients(pdg_wide *W, const double *xyz, const double *phi, const pdg_scf_options &o, double *P, int use_density,
                          double *energies, double *gradients, double *charges, int *status, int *ncycles, double *ws, cudaStream_t st);
int launch_qcmm_potentials(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                           const double *q, int n_knots, const double *knots, double cutoff, double *phi, void *ws, cudaStream_t st);
int launch_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                          const double *q, const double *qcq, int n_knots, const double *knots, double cutoff,
                          double *gqc, double *gmm, void *ws, cudaStream_t st);
int launch_tc_selftest(int n, int kprod, int wait_limit, const float *x, float *c, int *status, cudaStream_t st);

// Density sets and occupancies of the open-shell / fractional-occupancy SCF (k_scf_open): from pdg_occupancy by
// occupancy_init's rules (QCOnePDM.c:290-330; host side, api.cu).
struct OpenOccupancy {
    int n_sets, type;        // 1 (restricted) or 2 sets; PDG_OCC_*
    double factor;           // 2 (restricted) or 1
    double charge[2];        // electrons of each set
    int ncard[2], nfrac[2];  // full and fractional orbitals (cardinal, fixed fractional)
    double frac[2];          // fraction of a full occupancy on each fractional orbital
    double beta;             // Fermi broadening (variable fractional)
};

// SCF kernels (scf.cu), in two compiled variants: scf_n (256 threads per CTA, tensor-core step) and scf_w
// (scf_wide.cu: 512 threads per CTA, FP64 only).  The single-system entry points use scf_n.
#define PDG_SCF_LAUNCHERS                                                                                                   \
    void launch_scf(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *phi, const pdg_scf_options &o, \
                    double *density, int use_density, double *energies, double *charges, int *status, int *ncycles,      \
                    double *ws, int fock_only, double *fock_out, cudaStream_t st, const double *base = nullptr);          \
    void launch_scf_open(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *phi, const pdg_scf_options &o, \
                         const OpenOccupancy &oc, double *density, int use_density, double *energies, double *charges,       \
                         int *status, int *ncycles, double *ws, cudaStream_t st);                                             \
    void launch_uhf_densities(int n_frames, int N, const double *P, double *out, cudaStream_t st);                       \
    int scf_occupancy(const DeviceSystem &s, int *threads, int *smem_bytes, int *ctas_per_sm);                           \
    void launch_batch_scf(const Batch &b, const int *order, int *queue, int grid, int smem_limit, size_t smem_bytes,     \
                          int tensor_items, const double *phi, const pdg_scf_options &o, double *density, int use_density, \
                          double *energies, double *charges, int *status, int *ncycles, double *ws, cudaStream_t st);    \
    size_t scf_smem_bytes_limit(int N, int kv, int limit_bytes);                                                         \
    int configure_batch_scf(size_t smem_bytes);
namespace scf_n { PDG_SCF_LAUNCHERS }
namespace scf_w { PDG_SCF_LAUNCHERS }
using scf_n::launch_scf;
using scf_n::launch_scf_open;
using scf_n::launch_uhf_densities;
using scf_n::scf_occupancy;
void launch_guess_features(const DeviceSystem &s, int n_frames, const double *xyz, const double *phi, float *env, int *count,
                           int *offsets, float *X, int *row_frame, int *row_pair, cudaStream_t st);
void launch_mlp_forward(int max_rows, const int *rows, int K, int N, const float *X, const void *W, const float *b, float *Z, float *H,
                        int act, cudaStream_t st);
void launch_mlp_backward(int max_rows, const int *rows, int N, int K, const float *dZ, const void *W, const float *Zin, const float *Hin,
                         float *dZin, int segments, float *part, cudaStream_t st);
void launch_mlp_adam(int N, int K, int segments, const float *part, float scale, float *Wm, float *bm, float *m1, float *m2, void *W,
                     float lr, float b1, float b2, float c1, float c2, cudaStream_t st);
void launch_guess_assemble(const DeviceSystem &s, int n_frames, const double *xyz, const int *offsets, const int *row_pair,
                           const float *Y, double *P, cudaStream_t st);
void launch_guess_loss(const DeviceSystem &s, int n_frames, const double *xyz, const int *offsets, const int *row_pair, const double *P,
                       const double *Ptarget, float *dY, double *loss, cudaStream_t st);

// Langevin dynamics (dynamics.cu).  Integration factors of LangevinVelocityVerletIntegrator
// (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py:63-112), computed on the host; sdR, sdV1, sdV2 already
// carry the temperature factor.
struct LangevinFactors {
    double facR1, facR2, facV1, facV2, sdR, sdV1, sdV2;
    int random;   // 0: no random forces (plain velocity Verlet with friction), 1: generated deviates, 2: given deviates
};
#define PDG_MAX_DENSITY_TERMS 8
struct DensityTerms {
    const double *d[PDG_MAX_DENSITY_TERMS];
    double c[PDG_MAX_DENSITY_TERMS];
    int count;
};
void launch_langevin_positions(int n_replicas, int n_atoms, int n_free, const int *free_atom, const double *inv_sqrt_mass, double *xyz,
                               double *vel, const double *acc, const LangevinFactors &f, uint64_t seed, uint32_t step,
                               double *deviates, cudaStream_t st);
void launch_langevin_velocities(int n_replicas, int n_free, int n_rows, const int *grad_row, const double *mass, const double *grad_a,
                                const double *grad_b, double grad_scale, double facV3, double *vel, double *acc, double *mv2,
                                cudaStream_t st);
void launch_density_combine(long long n, const DensityTerms &t, double *out, cudaStream_t st);
void launch_normal_deviates(long long n_pairs, uint64_t seed, uint32_t step, uint32_t stream, double *out, cudaStream_t st);
void launch_linear_project(int n_replicas, int n_free, int n_rows, const int *rows, int n_vectors, const double *vectors,
                           const double *scale, int width, double *arr, cudaStream_t st);

// ---- MM/MM and QC/MM Lennard-Jones energies (mmmm.cu) ----
// Per-atom flags: an active MM atom, a QC atom with LJ interactions (the reference's qcpSelection), a fixed atom.
constexpr int MM_FLAG_MM = 1, MM_FLAG_QC_LJ = 2, MM_FLAG_FIXED = 4;
constexpr int MM_NCH = 6;             // energies: MM/MM Elect., MM/MM LJ, MM/MM 1-4 Elect., MM/MM 1-4 LJ, QC/MM LJ, QC/MM 1-4 LJ
constexpr int MM_MAX_CELLS_1D = 32;   // cell-grid cells per dimension at most
// PairwiseInteractionABFSFactors (cinclude/PairwiseInteraction.h:39-66), made by the host (PairwiseInteraction.c:89-140)
struct MMFactors {
    double r2Damp, r2Off, r2On, a, b, c, d, qShift1, qShift2, qF0, qAlpha;
    double aF6, aK12, aShift12, aF0, aAlpha, bF3, bK6, bShift6, bF0, bAlpha;
};
struct MMDevice {
    int n_atoms, n_types;
    const double *charge;                 // n_atoms (e)
    const int *lj_type;                   // n_atoms
    const unsigned char *flags;           // n_atoms: MM_FLAG_*
    const double *A, *B, *A14, *B14;      // LJ tables, n_types x n_types (kJ/mol A^12, kJ/mol A^6)
    const int *excl_start, *excl;         // exclusions, both directions (n_atoms + 1 offsets)
    const int *p14_start, *p14;           // 1-4 partners, both directions
    MMFactors fac;
    double escale, escale14;              // e^2/A -> kJ/mol over the dielectric; times electrostaticScale14
    double outer;                         // outer cutoff (A)
};
// Per-frame workspace (byte offsets from the frame's base; stride bytes per frame)
struct MMLayout {
    size_t grid, count, start, cell_of, order, sxyzq, part, stride;
    int n_blocks;
};
MMLayout mm_layout(int n_atoms);
void launch_mm_energy(const MMDevice &m, int n_frames, const double *xyz, double *energies, double *grad, char *ws, cudaStream_t st);
