// scf.cu - the whole closed-shell RHF SCF of one frame in one CTA (FP64).
//
// One CTA per frame runs pDynamo's converger loop (pMolecule.QCModel.pyx:146-185 driving
// DIISSCFConverger.c:100-770) without returning to the host:
//   Fock build      F = H + G(P) by atom blocks (QCModelMNDO_Fock, QCModelMNDO.c:700, with the G(P) of
//                   MNDOIntegrals_MakeFockG, MNDOIntegrals.c:51, written as J/K block contractions),
//                   Lowdin-charge QC/MM term (QCModelMNDO_QCMMFockLowdin, :1808)
//   DIIS/ODA        DIIS_Fock_Save (:385), DIIS_Iterate (:530), RCA_Iterate (:661), mode switching (:147)
//   density step    QCOnePDM_MakeFromFock (QCOnePDM.c:403) without a full eigendecomposition: Householder
//                   tridiagonalisation, bisection for the min(n_occ, N - n_occ) eigenvalues needed, inverse
//                   iteration (with re-orthogonalisation inside clusters), back-transformation, and
//                   P = 2 C_occ C_occ^T or 2 (1 - C_virt C_virt^T).  The reference's dspevd computes all
//                   eigenpairs; the density depends only on the occupied subspace, which this reproduces.
// GB300's FP64 rate (~2 DFMA/clk/SM) makes this arithmetic-bound; the dense products run as register-tiled
// shared-memory GEMMs and everything sequential is confined to O(N) or O(N^2) work.
#include "common.cuh"
#include "multipole.cuh"
#include "tc.cuh"

// The SCF kernels are compiled twice: as scf_n (this file: 256 threads per CTA, two CTAs per SM, with the
// tensor-core purification step) and as scf_w (scf_wide.cu: 512 threads, one CTA per SM, FP64 steps only).
#ifndef PDG_SCF_NS
#define PDG_SCF_NS scf_n
#endif
namespace PDG_SCF_NS {


struct SCFArgs {
    DeviceSystem s; FramePlan plan; int n_frames;
    const double *phi; pdg_scf_options o;
    double *density; int use_density;
    double *energies, *charges; int *status, *ncycles;
    double *ws; int fock_only; double *fock_out;
    int smem_limit;   // bytes of shared memory one CTA may plan for (the launch provides the plan's bytes)
    const double *base;   // shared base of the perturbative density steps (the mixed method), or null
    // open-shell and fractional-occupancy SCF (k_scf_open): the density sets and their occupancies
    int n_sets;                      // 1: spin-restricted (the total density), 2: alpha and beta
    int occ_type;                    // PDG_OCC_CARDINAL, PDG_OCC_FIXED_FRACTIONAL or PDG_OCC_VARIABLE_FRACTIONAL
    double occ_factor;               // occupancy of a full orbital: 2 (restricted) or 1
    double occ_charge[2];            // electrons of each set
    int occ_ncard[2], occ_nfrac[2];  // fully and fractionally occupied orbitals (cardinal, fixed fractional)
    double occ_frac[2];              // the fraction of occ_factor on each of the occ_nfrac orbitals
    double fermi_beta;               // variable fractional: the Fermi broadening (1 / Hartree)
};

struct Smem {
    double *red, *small, *d, *e, *e2, *tau, *eig, *v, *v2, *p, *w, *part, *dot;
    double *ta, *tb;   // GEMM staging
    double *amat;      // packed lower triangle of the matrix being tridiagonalised (null: in the workspace)
    double *zs;        // the wanted eigenvectors, one row of ldz per vector (null: in the workspace)
    int ldz;
    int *iv;           // ints: [0..63] control, [64..64+N) per-vector cluster starts
};

// GEMM tile: GM x GN outputs per pass (GWR x 4 warps of 8 x 16), GK-deep staged chunks (padded rows
// against bank conflicts).
#define GWR (PDG_WARPS / 4)
#define GM (8 * GWR)
#define GN 64
#define GK 16
#define GA_LD (GM + 1)
#define GB_LD (GN + 1)

// Shared memory plan: red | small | d e e2 tau eig v v2 p w (9N) | part (4N) | dot | ints | GEMM staging | amat | zs.
// The packed matrix goes to shared memory when it fits, then the eigenvectors.
struct SmemPlan { size_t head, work, amat, zs, bytes; int ldz; };

// Doubles of the split-BF16 operand arrays (hi and mid or lo parts, R x Kp bf16 each) of the purification
// density step; 0 when N is beyond its one-tile limit.
__host__ __device__ inline size_t mix_doubles(int N)
{
    if (N > 144) return 0;
    const size_t Kp = (N + 15) & ~15, R = Kp > 128 ? Kp : 128;
    return 2 * R * Kp * 2 / 8;
}

__host__ __device__ inline size_t round16(size_t x) { return (x + 15) & ~size_t(15); }

// Default shared-memory budget of one SCF CTA: all of an SM's shared memory, or half of it for two CTAs.
#define PDG_SMEM_LIMIT (PDG_SCF_CTAS_PER_SM == 1 ? PDG_SMEM_LIMIT_1 : PDG_SMEM_LIMIT_2)

__host__ __device__ inline SmemPlan smem_plan(int N, int kv, int limit_bytes)
{
    SmemPlan p;
    p.head = round16(32 + 256 + 13 * (size_t)N + 64 + ((64 + (size_t)N + 2) * sizeof(int) + 7) / 8);
    p.work = round16((size_t)GK * GA_LD + (size_t)GK * GB_LD);
    p.ldz = N | 1;
    const size_t limit = (size_t)limit_bytes / 8, packed = (size_t)N * (N + 1) / 2;
    const size_t zsz = (size_t)(kv > 0 ? kv : 1) * p.ldz, mix = mix_doubles(N);
    const size_t slot = round16(packed > mix ? packed : mix);
    p.amat = (p.head + p.work + slot <= limit) ? slot : 0;
    p.zs = (p.amat && p.head + p.work + p.amat + zsz <= limit) ? zsz : 0;
    p.bytes = 8 * (p.head + p.work + p.amat + p.zs);
    return p;
}

__device__ __forceinline__ Smem carve(double *base, int N, int kv, int limit_bytes)
{
    Smem m;
    SmemPlan sp = smem_plan(N, kv, limit_bytes);
    m.red = base; m.small = base + 32;
    m.d = m.small + 256; m.e = m.d + N; m.e2 = m.e + N; m.tau = m.e2 + N; m.eig = m.tau + N;
    m.v = m.eig + N; m.v2 = m.v + N; m.p = m.v2 + N; m.w = m.p + N; m.part = m.w + N; m.dot = m.part + 4 * (size_t)N;
    m.iv = (int *)(m.dot + 64);
    double *work = base + sp.head;
    m.ta = work; m.tb = work + GK * GA_LD;
    m.amat = sp.amat ? work + sp.work : nullptr;
    m.zs = sp.zs ? work + sp.work + sp.amat : nullptr;
    m.ldz = sp.ldz;
    return m;
}

// C = A B over M x Nc outputs with inner dimension K; fa(i, k) and fb(k, j) fetch the operands (AK / BK: k is
// the contiguous index of that operand, which picks the coalesced staging order).  Each warp owns an
// 8 x 16 sub-tile of the GM x GN pass (2 x 2 outputs per lane) and skips the FMA loop when the sub-tile lies
// outside the output, or above the diagonal when lower_only; warp (wr, wc) sits on FP64 unit (wr + wc) % 4,
// so the partial warps of edge tiles stay spread over all four.  The epilogue receives every (i, j) < (M, Nc)
// of an active sub-tile; lower_only callers filter j > i there.
template <bool AK, bool BK, typename FA, typename FB, typename Epi, typename T = double>
__device__ void tgemm(int M, int Nc, int K, FA fa, FB fb, bool lower_only, Smem &sm, Epi epi, T = T())
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int wr = w >> 2, wc = ((w & 3) - wr) & 3;
    const int r0 = wr * 8 + (lane >> 3) * 2, c0 = wc * 16 + (lane & 7) * 2;
    T *ga = (T *)sm.ta, *gb = (T *)sm.tb;
    for (int i0 = 0; i0 < M; i0 += GM)
        for (int j0 = 0; j0 < Nc; j0 += GN) {
            if (lower_only && j0 > i0 + GM - 1) continue;
            const bool active = (i0 + wr * 8 < M) && (j0 + wc * 16 < Nc) && !(lower_only && j0 + wc * 16 > i0 + wr * 8 + 7);
            T a00 = 0, a01 = 0, a10 = 0, a11 = 0;
            for (int k0 = 0; k0 < K; k0 += GK) {
                const int kc = min(GK, K - k0);
                __syncthreads();
                for (int t = tid; t < GM * GK; t += PDG_BLOCK) {
                    const int r = AK ? t / GK : t % GM, kk = AK ? t % GK : t / GM, gi = i0 + r;
                    ga[kk * GA_LD + r] = (kk < kc && gi < M) ? (T)fa(gi, k0 + kk) : (T)0;
                }
                for (int t = tid; t < GK * GN; t += PDG_BLOCK) {
                    const int c = BK ? t / GK : t % GN, kk = BK ? t % GK : t / GN, gj = j0 + c;
                    gb[kk * GB_LD + c] = (kk < kc && gj < Nc) ? (T)fb(k0 + kk, gj) : (T)0;
                }
                __syncthreads();
                if (active) {
#pragma unroll 4
                    for (int kk = 0; kk < kc; kk++) {
                        const T x0 = ga[kk * GA_LD + r0], x1 = ga[kk * GA_LD + r0 + 1];
                        const T y0 = gb[kk * GB_LD + c0], y1 = gb[kk * GB_LD + c0 + 1];
                        a00 = fma(x0, y0, a00); a01 = fma(x0, y1, a01); a10 = fma(x1, y0, a10); a11 = fma(x1, y1, a11);
                    }
                }
            }
            if (active) {
                const int gi = i0 + r0, gj = j0 + c0;
                if (gi < M && gj < Nc) epi(gi, gj, (double)a00);
                if (gi < M && gj + 1 < Nc) epi(gi, gj + 1, (double)a01);
                if (gi + 1 < M && gj < Nc) epi(gi + 1, gj, (double)a10);
                if (gi + 1 < M && gj + 1 < Nc) epi(gi + 1, gj + 1, (double)a11);
            }
        }
    __syncthreads();
}

// FP32 C = A B for the perturbative density step and the mixed method's commutators.  Output tiles of
// (4 TY) x 64 (TY = threads / 16) with 4 x 4 outputs per thread, so every 16-deep staged chunk gives each thread
// 16 FMAs per pair of float4 shared-memory reads; the next chunk's operands are loaded into registers while the
// current one is multiplied, so the L2 latency of the staging loads overlaps the FMAs.  The staging fits in the
// FP64 GEMM's staging area.  The epilogue receives every (i, j) < (M, Nc) of a computed tile; lower_only skips
// tiles wholly above the diagonal (callers filter j > i).
template <bool AK, bool BK, typename FA, typename FB, typename Epi>
__device__ void tgemm32(int M, int Nc, int K, FA fa, FB fb, bool lower_only, Smem &sm, Epi epi)
{
    constexpr int TX = 16, TY = PDG_BLOCK / TX, TM = 4 * TY, TN = 64, KC = 16, LDA = TM + 4, LDB = TN;
    constexpr int NA = TM * KC / PDG_BLOCK, NB = KC * TN / PDG_BLOCK;
    static_assert(KC * (LDA + LDB) * sizeof(float) <= GK * (GA_LD + GB_LD) * sizeof(double), "staging area");
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    float *ga = (float *)sm.ta, *gb = ga + KC * LDA;
    for (int i0 = 0; i0 < M; i0 += TM)
        for (int j0 = 0; j0 < Nc; j0 += TN) {
            if (lower_only && j0 > i0 + TM - 1) continue;
            float acc[4][4];
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = 0.f;
            float ra[NA], rb[NB];
            auto fetch = [&](int k0) {
                const int kc = min(KC, K - k0);
#pragma unroll
                for (int u = 0; u < NA; u++) {
                    const int t = tid + u * PDG_BLOCK;
                    const int r = AK ? t / KC : t % TM, kk = AK ? t % KC : t / TM, gi = i0 + r;
                    ra[u] = (kk < kc && gi < M) ? (float)fa(gi, k0 + kk) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < NB; u++) {
                    const int t = tid + u * PDG_BLOCK;
                    const int c = BK ? t / KC : t % TN, kk = BK ? t % KC : t / TN, gj = j0 + c;
                    rb[u] = (kk < kc && gj < Nc) ? (float)fb(k0 + kk, gj) : 0.f;
                }
            };
            fetch(0);
            for (int k0 = 0; k0 < K; k0 += KC) {
                const int kc = min(KC, K - k0);
                __syncthreads();
#pragma unroll
                for (int u = 0; u < NA; u++) {
                    const int t = tid + u * PDG_BLOCK;
                    const int r = AK ? t / KC : t % TM, kk = AK ? t % KC : t / TM;
                    ga[kk * LDA + r] = ra[u];
                }
#pragma unroll
                for (int u = 0; u < NB; u++) {
                    const int t = tid + u * PDG_BLOCK;
                    const int c = BK ? t / KC : t % TN, kk = BK ? t % KC : t / TN;
                    gb[kk * LDB + c] = rb[u];
                }
                __syncthreads();
                if (k0 + KC < K) fetch(k0 + KC);
#pragma unroll 4
                for (int kk = 0; kk < kc; kk++) {
                    const float4 av = *(const float4 *)(ga + kk * LDA + 4 * ty), bv = *(const float4 *)(gb + kk * LDB + 4 * tx);
                    const float x4[4] = { av.x, av.y, av.z, av.w }, y4[4] = { bv.x, bv.y, bv.z, bv.w };
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) acc[x][y] = fmaf(x4[x], y4[y], acc[x][y]);
                }
            }
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) {
                    const int gi = i0 + 4 * ty + x, gj = j0 + 4 * tx + y;
                    if (gi < M && gj < Nc) epi(gi, gj, (double)acc[x][y]);
                }
        }
    __syncthreads();
}

// ----------------------------------------------------------------------------------------------------
// F = H + G(P) and the energies tr(PH), tr(PG)/2; then the QC/MM Lowdin term.  Returns eqcmm.
__device__ void fock_build(const SCFArgs &a, int f, const double *H, const double *P, double *F, const double *tei,
                           Smem &sm, double *e1, double *e2, double *eqcmm, double *scratch)
{
    const DeviceSystem &s = a.s;
    const int N = s.n_basis, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // One-centre densities of every atom with the off-diagonal factor 2 (the Coulomb contractions' right-hand
    // sides), in the order of the diagonal-block element list: in the GEMM staging area when they fit, else in
    // the workspace scratch.
    double *pk = s.n_cel <= GK * (GA_LD + GB_LD) ? sm.ta : scratch;
    for (int e = threadIdx.x; e < s.n_cel; e += PDG_BLOCK) {
        const int A = s.cel[e] >> 4, ab = s.cel[e] & 15, as = s.atom_start[A];
        const int m = MP_DA[ab], n = MP_DB[ab];
        pk[e] = (m == n ? 1.0 : 2.0) * P[(size_t)(as + m) * N + as + n];
    }
    __syncthreads();
    // One flat pass, one thread per output element (lists built by pdg_system_create):
    //  * diagonal-block element (A, m >= n): H + one-centre G + Coulomb sum_B sum_cd (mn|cd) P_B,cd over every
    //    partner atom B (QCModelMNDO_Fock's one-centre terms and MakeFockG's Coulomb part);
    //  * off-diagonal-block element (pair, a, c): F_ac = H_ac - 1/2 sum_bd (ab|cd) P_bd (exchange), the
    //    elements sorted by pair class so that the lanes of a warp run the same loop lengths.
    const int n_out = s.n_cel + s.n_xel;
    for (int e = threadIdx.x; e < n_out; e += PDG_BLOCK) {
        if (e < s.n_cel) {
            const int A = s.cel[e] >> 4, ab = s.cel[e] & 15;
            const int no = s.atom_norb[A], as = s.atom_start[A], na = no * (no + 1) / 2;
            const int m = MP_DA[ab], n = MP_DB[ab];   // m >= n
            double acc = 0.0;
            for (int B = 0; B < s.n_atoms; B++) {
                if (B == A) continue;
                const int hi = A > B ? A : B, lo = A > B ? B : A, pp = hi * (hi - 1) / 2 + lo;
                const int k0 = s.atom_pk[B], nb = s.atom_pk[B + 1] - k0;
                const double *blk = tei + s.pair_tei[pp], *pb = pk + k0;
                if (A > B) for (int cd = 0; cd < nb; cd++) acc = fma(blk[ab * nb + cd], pb[cd], acc);
                else       for (int cd = 0; cd < nb; cd++) acc = fma(blk[cd * na + ab], pb[cd], acc);
            }
            const double *E = elem(s, s.atom_elem[A]);
            const double gss = E[PDG_E_GSS], gsp = E[PDG_E_GSP], gpp = E[PDG_E_GPP], gp2 = E[PDG_E_GP2], hsp = E[PDG_E_HSP], hpp = E[PDG_E_HPP];
            const double *PA = P + (size_t)as * N + as;
            double g = 0.0;
            if (no == 1) g = 0.5 * PA[0] * gss;
            else if (m == 0 && n == 0) { g = 0.5 * PA[0] * gss; for (int q = 1; q < 4; q++) g += PA[q * N + q] * (gsp - 0.5 * hsp); }
            else if (m == n) {
                g = PA[0] * (gsp - 0.5 * hsp) + 0.5 * PA[m * N + m] * gpp;
                for (int q = 1; q < 4; q++) if (q != m) g += PA[q * N + q] * (gp2 - 0.5 * hpp);
            } else if (n == 0) g = PA[m * N + n] * (1.5 * hsp - 0.5 * gsp);
            else g = PA[m * N + n] * (1.5 * hpp - 0.5 * gp2);
            const double v = H[(size_t)(as + m) * N + as + n] + g + acc;
            F[(size_t)(as + m) * N + as + n] = v;
            F[(size_t)(as + n) * N + as + m] = v;
        } else {
            const int x = s.xel[e - s.n_cel], pp = x >> 4, lid = x & 15;
            const int i = s.pair_i[pp], j = s.pair_j[pp];
            const int noi = s.atom_norb[i], noj = s.atom_norb[j], is = s.atom_start[i], js = s.atom_start[j];
            const int nj = noj * (noj + 1) / 2, aa = lid / noj, c = lid % noj;
            const double *blk = tei + s.pair_tei[pp];
            double t = 0.0;
            for (int b = 0; b < noi; b++) {
                const int ab = aa >= b ? aa * (aa + 1) / 2 + b : b * (b + 1) / 2 + aa;
                for (int d = 0; d < noj; d++) {
                    const int cd = c >= d ? c * (c + 1) / 2 + d : d * (d + 1) / 2 + c;
                    t = fma(blk[ab * nj + cd], P[(size_t)(is + b) * N + js + d], t);
                }
            }
            const double v = fma(-0.5, t, H[(size_t)(is + aa) * N + js + c]);
            F[(size_t)(is + aa) * N + js + c] = v;
            F[(size_t)(js + c) * N + is + aa] = v;
        }
    }
    __syncthreads();
    // tr(P H) and tr(P G) = tr(P F) - tr(P H) over the lower triangle (all three matrices are symmetric), warp per row
    double th = 0.0, tf = 0.0, dh = 0.0, df = 0.0;
    for (int i = w; i < N; i += PDG_WARPS)
        for (int j = lane; j <= i; j += 32) {
            const size_t k = (size_t)i * N + j;
            const double pv = P[k];
            if (j < i) { th = fma(pv, H[k], th); tf = fma(pv, F[k], tf); }
            else { dh = fma(pv, H[k], dh); df = fma(pv, F[k], df); }
        }
    const double2 tr_h = block_sum2(th, dh, sm.red), tr_f = block_sum2(tf, df, sm.red);
    *e1 = 2.0 * tr_h.x + tr_h.y;
    *e2 = 0.5 * ((2.0 * tr_f.x + tr_f.y) - *e1);
    // QC/MM: q_A = Z_A - sum P_mm, E += q . phi, F_mm -= phi_A (QCModelMNDO.c:1459-1520, 1808-1860)
    double tq = 0.0;
    const double *phi = a.phi ? a.phi + (size_t)f * s.n_atoms : nullptr;
    for (int A = threadIdx.x; A < s.n_atoms; A += PDG_BLOCK) {
        int no = s.atom_norb[A], as = s.atom_start[A];
        double ps = 0.0;
        for (int m = 0; m < no; m++) ps += P[(size_t)(as + m) * N + as + m];
        double q = elem(s, s.atom_elem[A])[PDG_E_ZCORE] - ps;
        if (a.charges) a.charges[(size_t)f * s.n_atoms + A] = q;
        if (phi) {
            tq += q * phi[A];
            for (int m = 0; m < no; m++) F[(size_t)(as + m) * N + as + m] -= phi[A];
        }
    }
    *eqcmm = block_sum(tq, sm.red);
}

// ----------------------------------------------------------------------------------------------------
// Small dense solve A x = b (n <= 17) by one warp: Gauss-Jordan with partial pivoting on [A | I | b] in
// shared memory M (n x (2n+1)), lanes over columns; rejects a reciprocal 1-norm condition below 1e-15
// (SymmetricMatrix_SolveLinearEquations' test, SymmetricMatrix.c:1412-1450, computed exactly from the
// inverse).  A(i, j) and b(i) are accessors; the solution is returned in x (lanes < n hold x[lane]).
template <typename FA, typename FB>
__device__ bool warp_small_solve(int n, FA A, FB b, double *M, double *x)
{
    const int lane = threadIdx.x & 31, w2 = 2 * n + 1;
    for (int e = lane; e < n * w2; e += 32) {
        const int i = e / w2, j = e % w2;
        M[e] = j < n ? A(i, j) : (j < 2 * n ? (j - n == i ? 1.0 : 0.0) : b(i));
    }
    __syncwarp();
    double cs = 0.0;
    if (lane < n) for (int i = 0; i < n; i++) cs += fabs(M[i * w2 + lane]);
    const double anorm = warp_max(cs);
    bool ok = true;
    for (int k = 0; k < n; k++) {
        // pivot: the first row i >= k of largest |M[i][k]|
        double v = (lane >= k && lane < n) ? fabs(M[lane * w2 + k]) : -1.0;
        int iv = lane;
        for (int o = 16; o > 0; o >>= 1) {
            const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, iv, o);
            if (v2 > v || (v2 == v && i2 < iv)) { v = v2; iv = i2; }
        }
        if (v == 0.0) { ok = false; break; }
        if (iv != k)
            for (int j = lane; j < w2; j += 32) { const double t = M[k * w2 + j]; M[k * w2 + j] = M[iv * w2 + j]; M[iv * w2 + j] = t; }
        __syncwarp();
        const double r = 1.0 / M[k * w2 + k];
        const double fi = lane < n ? M[lane * w2 + k] * r : 0.0;
        const double pk0 = lane < w2 ? M[k * w2 + lane] : 0.0, pk1 = lane + 32 < w2 ? M[k * w2 + lane + 32] : 0.0;
        __syncwarp();
        for (int i = 0; i < n; i++) {
            const double f = __shfl_sync(0xffffffffu, fi, i);
            if (i == k) continue;
            if (lane < w2) M[i * w2 + lane] = fma(-f, pk0, M[i * w2 + lane]);
            if (lane + 32 < w2) M[i * w2 + lane + 32] = fma(-f, pk1, M[i * w2 + lane + 32]);
        }
        __syncwarp();
    }
    if (!ok) return false;
    double ci = 0.0;
    if (lane < n) for (int i = 0; i < n; i++) ci += fabs(M[i * w2 + n + lane] / M[i * w2 + i]);
    const double inorm = warp_max(ci);
    if (lane < n) x[lane] = M[lane * w2 + 2 * n] / M[lane * w2 + lane];
    __syncwarp();
    return anorm * inorm < 1.0e15;
}

// ----------------------------------------------------------------------------------------------------
// Density step: P <- density of the lowest n_occ eigenvectors of F.  Returns the RMS change
// ||P_new - P||_F / N (QCOnePDM_Make, QCOnePDM.c:369-400).
__device__ unsigned int hash2(unsigned int a, unsigned int b)
{
    unsigned int h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    return h;
}

// Sturm count in FP32: number of eigenvalues of T below x (LDL^T pivots, pivmin guard).  The counts only
// locate shifts for inverse iteration, which then converges in FP64 on the FP64 matrix.
__device__ int sturm_count32(int N, const float *d, const float *e2, float x, float pivmin)
{
    int c = 0;
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    c += (q < 0.0f);
    for (int i = 1; i < N; i++) {
        q = (d[i] - x) - __fdividef(e2[i - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        c += (q < 0.0f);
    }
    return c;
}

// Phase timers: thread 0 accumulates clock64() deltas between block-wide barriers into the frame's
// timer slots (workspace misc area, after the DIIS B matrix).
static_assert(PDG_NTIMERS <= 96, "timer slots live in the 96 doubles after the DIIS B matrix");
struct Timer {
    double *slot; long long t;
    __device__ void start() { if (threadIdx.x == 0) t = clock64(); }
    __device__ void lap(int k) { if (threadIdx.x == 0) { long long n = clock64(); slot[k] += (double)(n - t); t = n; } }
    // a sub-phase inside a lapped phase: adds the cycles since t0 to slot k without moving the lap origin
    __device__ long long now() const { return clock64(); }
    __device__ void add(int k, long long t0) { if (threadIdx.x == 0) slot[k] += (double)(clock64() - t0); }
};

// Packed lower-triangle element (i >= j) of the matrix being tridiagonalised.
__device__ __forceinline__ int plo(int i, int j) { return i * (i + 1) / 2 + j; }

// Householder reflector for column c (rows c+1 .. N-1) of the packed matrix, by one warp (dlarfg): writes
// v (v[0] = 1) to vout and into the column below the subdiagonal, tau and the subdiagonal beta.
__device__ void make_reflector(double *A, int N, int c, double *vout, Smem &sm)
{
    const int lane = threadIdx.x & 31, m = N - c - 1, r0 = c + 1;
    const double alpha = A[plo(r0, c)];
    double part = 0.0;
    for (int i = 1 + lane; i < m; i += 32) { const double x = A[plo(r0 + i, c)]; part = fma(x, x, part); }
    const double xn2 = warp_sum(part);
    double tau = 0.0, e = alpha, scal = 0.0;
    if (xn2 != 0.0) {
        const double beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
        tau = (beta - alpha) / beta; e = beta; scal = 1.0 / (alpha - beta);
    }
    for (int i = lane; i < m; i += 32) {
        const double vi = (i == 0) ? 1.0 : A[plo(r0 + i, c)] * scal;
        vout[i] = vi;
        if (i > 0 && tau != 0.0) A[plo(r0 + i, c)] = vi;
    }
    if (lane == 0) { sm.e[c] = e; sm.tau[c] = tau; }
}

__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }

// Inverse iteration for one eigenvector of the tridiagonal T (d, e) at shift sigma, by ONE thread: the LU
// factors of T - sigma I with row interchanges (dgttrf form: multiplier l_k, pivot flag, U row
// 1/u_kk, u_k,k+1, u_k,k+2), four solves, re-orthogonalisation against the earlier vectors q0 .. t-1 of the
// same cluster (dstein), normalisation.  The factor arrays and the iterate are interleaved by vector (stride
// ld) so the threads of a warp access them coalesced.  Pivoting is branch-free (selects), so the lanes of a
// warp never diverge; loads are issued in blocks of eight ahead of the dependent recurrence.  R = float (the
// perturbative base's complementary vectors): T - sigma I is formed in FP64 and rounded, everything after it is
// FP32, and the iterate is rescaled by its largest element between solves (folded into the next forward pass).
template <typename R>
__device__ void inverse_iteration(int N, int t, double sigma, double tiny, const double *__restrict__ d, const double *__restrict__ e,
                                  R *__restrict__ u0, R *__restrict__ u1, R *__restrict__ u2, R *__restrict__ lm,
                                  unsigned char *__restrict__ pv, R *y, int ldy, int ld, const R *zq0, int nq, int ldz, R *zout)
{
    constexpr bool F32 = sizeof(R) == 4;
    const R rtiny = (R)tiny;
    R ak = (R)(d[0] - sigma), bk = (R)e[0];
    for (int k = 0; k < N - 1; k++) {
        const R ck = (R)e[k], an = (R)(d[k + 1] - sigma), bn = (R)e[k + 1];
        const bool sw = fabs(ak) < fabs(ck);
        R piv = sw ? ck : ak;
        if (fabs(piv) < rtiny) piv = copysign(rtiny, piv);
        const R r = rcp_rn(piv), l = (sw ? ak : ck) * r;
        const R uu1 = sw ? an : bk, uu2 = sw ? bn : (R)0;
        u0[(size_t)k * ld] = r; u1[(size_t)k * ld] = uu1; u2[(size_t)k * ld] = uu2; lm[(size_t)k * ld] = l; pv[(size_t)k * ld] = sw;
        ak = fma(-l, uu1, sw ? bk : an);
        bk = fma(-l, uu2, sw ? (R)0 : bn);
    }
    if (fabs(ak) < rtiny) ak = copysign(rtiny, ak);
    u0[(size_t)(N - 1) * ld] = rcp_rn(ak);
    for (int i = 0; i < N; i++) y[(size_t)i * ldy] = (R)(((hash2(t * 2654435761u + 17u, i) >> 8) * (1.0 / 16777216.0)) * 2.0 - 1.0);
    R sc = (R)1;   // FP32: scale of the stored iterate (1 / its largest element after the last solve)
    for (int it = 0; it < 4; it++) {
        // forward: interchanges and L
        R c = F32 ? y[0] * sc : y[0];
        int k = 0;
        for (; k + 8 <= N - 1; k += 8) {
            R xn[8], l[8]; bool sw[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                xn[q] = y[(size_t)(k + 1 + q) * ldy]; l[q] = lm[(size_t)(k + q) * ld]; sw[q] = pv[(size_t)(k + q) * ld];
                if (F32) xn[q] *= sc;
            }
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const R yk = sw[q] ? xn[q] : c, cn = sw[q] ? c : xn[q];
                y[(size_t)(k + q) * ldy] = yk;
                c = fma(-l[q], yk, cn);
            }
        }
        for (; k < N - 1; k++) {
            const R xn = F32 ? y[(size_t)(k + 1) * ldy] * sc : y[(size_t)(k + 1) * ldy], l = lm[(size_t)k * ld];
            const bool sw = pv[(size_t)k * ld];
            const R yk = sw ? xn : c, cn = sw ? c : xn;
            y[(size_t)k * ldy] = yk;
            c = fma(-l, yk, cn);
        }
        // back substitution with U
        R x1 = c * u0[(size_t)(N - 1) * ld], x2 = (R)0, mx = fabs(x1);
        y[(size_t)(N - 1) * ldy] = x1;
        k = N - 2;
        for (; k - 7 >= 0; k -= 8) {
            R yy[8], a0[8], a1[8], a2[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const size_t o = (size_t)(k - q) * ld;
                yy[q] = y[(size_t)(k - q) * ldy]; a0[q] = u0[o]; a1[q] = u1[o]; a2[q] = u2[o];
            }
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const R x0 = fma(-a2[q], x2, fma(-a1[q], x1, yy[q])) * a0[q];
                y[(size_t)(k - q) * ldy] = x0;
                x2 = x1; x1 = x0;
                if (F32) mx = fmax(mx, fabs(x0));
            }
        }
        for (; k >= 0; k--) {
            const size_t o = (size_t)k * ld;
            const R x0 = fma(-u2[o], x2, fma(-u1[o], x1, y[(size_t)k * ldy])) * u0[o];
            y[(size_t)k * ldy] = x0;
            x2 = x1; x1 = x0;
            if (F32) mx = fmax(mx, fabs(x0));
        }
        // FP64: the iterate is never rescaled between solves: four solves grow it by at most (1/tiny)^4, far
        // inside the double range, and the projections below do not depend on its scale.  FP32: one solve grows
        // it by at most 1/tiny (~1e7), and the next pass reads it times 1/max.
        if (F32) sc = mx > (R)0 ? (R)1 / mx : (R)1;
        for (int q = 0; q < nq; q++) {
            const R *zq = zq0 + (size_t)q * ldz;
            R dt = (R)0;
            for (int i = 0; i < N; i++) dt = fma(y[(size_t)i * ldy], zq[i], dt);
            for (int i = 0; i < N; i++) y[(size_t)i * ldy] = fma(-dt, zq[i], y[(size_t)i * ldy]);
        }
    }
    R nr = (R)0;
    for (int i = 0; i < N; i++) { const R v = F32 ? y[(size_t)i * ldy] * sc : y[(size_t)i * ldy]; nr = fma(v, v, nr); }
    const R nsc = F32 ? sc * rsqrt(nr) : rsqrt(nr);
    for (int i = 0; i < N; i++) zout[i] = y[(size_t)i * ldy] * nsc;
}

// Back-transformation of nv vectors of T in FP32 (rows of Zt, N floats each): the blocked compact-WY scheme of
// tridiag_vectors with V^T V, T and both products in FP32.  For the complementary vectors of the perturbative base:
// they enter the perturbative steps only in products with a small factor (dF, K), so their FP32 errors (~1e-7,
// their orthogonality to the FP64 wanted vectors included) stay ~1e-7 of a small quantity, while the wanted vectors,
// whose projector is the base density, keep the FP64 transformation.  work: 32 nv + 512 floats.  N >= 32.
__device__ void back_transform32(int N, float *work, const double *A, Smem &sm, int nv, float *Zt)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nref = N - 2;
    float *Wm = work, *W2 = Wm + (size_t)16 * nv, *Sg = W2 + (size_t)16 * nv, *Tt = Sg + 256;
    for (int k0 = ((nref - 1) / 16) * 16; k0 >= 0; k0 -= 16) {
        const int nbk = min(16, nref - k0), m0 = N - k0 - 1;
        auto V = [&](int i, int c) -> float { return i < c ? 0.f : (i == c ? 1.f : (float)A[plo(k0 + 1 + i, k0 + c)]); };
        tgemm32<false, true>(nbk, 16 + nv, m0, [&](int c, int i) { return V(i, c); },
                             [&](int i, int j) { return j < 16 ? (j < nbk ? V(i, j) : 0.f) : Zt[(size_t)(j - 16) * N + k0 + 1 + i]; },
                             false, sm, [&](int c, int j, double v) {
                                 if (j < 16) Sg[c * 16 + j] = (float)v;
                                 else Wm[(size_t)c * nv + (j - 16)] = (float)v;
                             });
        if (w == 0) {   // T(c, c) = tau_c;  T(0:c, c) = -tau_c T(0:c, 0:c) S(0:c, c)
            for (int c = 0; c < nbk; c++) {
                const float tau = (float)sm.tau[k0 + c];
                float t = 0.f;
                if (lane < c) {
                    for (int j = lane; j < c; j++) t = fmaf(Tt[lane * 16 + j], Sg[j * 16 + c], t);
                    t *= -tau;
                }
                __syncwarp();
                if (lane < 16) Tt[lane * 16 + c] = lane < c ? t : (lane == c ? tau : 0.f);
                __syncwarp();
            }
        }
        __syncthreads();
        for (int e = tid; e < nbk * nv; e += PDG_BLOCK) {
            const int c = e / nv, t = e % nv;
            float acc = 0.f;
            for (int j = c; j < nbk; j++) acc = fmaf(Tt[c * 16 + j], Wm[(size_t)j * nv + t], acc);
            W2[(size_t)c * nv + t] = acc;
        }
        __syncthreads();
        tgemm32<false, true>(nv, m0, nbk, [&](int t, int c) { return W2[(size_t)c * nv + t]; }, [&](int c, int i) { return V(i, c); },
                             false, sm, [&](int t, int i, double v) { Zt[(size_t)t * N + k0 + 1 + i] -= (float)v; });
    }
}

// Eigenvalues first .. first + kv - 1 of the tridiagonal T (sm.d, sm.e) left by the Householder reduction of the
// matrix whose reflectors are in A, their eigenvectors by inverse iteration, back-transformed to the rows of Z
// (kv rows of ldz; z_in_smem when Z is the shared-memory slot).  The eigenvalues are left in sm.eig[0 .. kv).
template <typename R>
__device__ void tridiag_vectors(const SCFArgs &a, double *wsf, const double *A, Smem &sm, Timer &tm, int first, int kv, R *Z, int ldz,
                                bool z_in_smem, bool count_step = true, bool refine = false)
{
    constexpr bool F32 = sizeof(R) == 4;
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int N = s.n_basis, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // --- shifts: eigenvalues first .. first + kv - 1 of T by FP32 Sturm multisection, eight threads per eigenvalue,
    //     each round narrowing the bracket ninefold
    float *d32 = (float *)sm.e2, *e232 = d32 + N;
    double gl = 1e300, gu = -1e300, emax2 = 0.0, onen = 0.0;
    for (int i = tid; i < N; i += PDG_BLOCK) {
        const double r = (i > 0 ? fabs(sm.e[i - 1]) : 0.0) + (i < N - 1 ? fabs(sm.e[i]) : 0.0);
        gl = fmin(gl, sm.d[i] - r); gu = fmax(gu, sm.d[i] + r); onen = fmax(onen, fabs(sm.d[i]) + r);
        d32[i] = (float)sm.d[i];
        const double e2 = (i < N - 1) ? sm.e[i] * sm.e[i] : 0.0;
        e232[i] = (float)e2; emax2 = fmax(emax2, e2);
    }
    gl = -block_max(-gl, sm.red); gu = block_max(gu, sm.red); emax2 = block_max(emax2, sm.red); onen = block_max(onen, sm.red);
    const double tnorm = fmax(fabs(gl), fabs(gu));
    const float pivmin = (float)(1.0e-30 * fmax(1.0, emax2));
    const float glo = (float)(gl - 1.0e-6 * tnorm - 1.0e-30), ghi = (float)(gu + 1.0e-6 * tnorm + 1.0e-30);
    for (int g0 = 0; g0 < kv; g0 += PDG_BLOCK / 8) {
        const int t = g0 + tid / 8, sl = tid % 8;
        const unsigned gmask = 0xFFu << (lane & ~7);
        const bool live = t < kv;
        const int mi = first + t;
        float lo = glo, hi = ghi;
        for (int round = 0; round < 16; round++) {
            const float x = lo + (hi - lo) * (float)(sl + 1) * (1.0f / 9.0f);
            const bool below = live && sturm_count32(N, d32, e232, x, pivmin) <= mi;   // x <= lambda_mi
            const unsigned bal = (__ballot_sync(0xffffffffu, below) & gmask) >> (lane & ~7);
            const int nb = __popc(bal);   // Sturm counts grow with x: the first nb points lie below
            const float xl = __shfl_sync(0xffffffffu, x, (lane & ~7) + (nb > 0 ? nb - 1 : 0));
            const float xh = __shfl_sync(0xffffffffu, x, (lane & ~7) + (nb < 8 ? nb : 7));
            const float nlo = nb > 0 ? xl : lo, nhi = nb < 8 ? xh : hi;
            const bool progress = live && (nlo > lo || nhi < hi);
            lo = nlo; hi = nhi;
            if (!__any_sync(0xffffffffu, progress)) break;   // every group of the warp is at FP32 resolution
        }
        if (live && sl == 0) sm.eig[t] = 0.5 * ((double)lo + (double)hi);
    }
    __syncthreads();
    tm.lap(PDG_T_EIGENVALUES);
    // --- clusters: neighbours closer than ortol are re-orthogonalised against each other (dstein-style);
    //     shifts within the FP32 resolution are separated.  iv[64 + t] = first vector of t's cluster,
    //     iv[0] = largest cluster.
    if (tid == 0) {
        const double ortol = 1.0e-4 * fmax(onen, 1.0);
        int start = 0, big = kv > 0 ? 1 : 0;
        sm.iv[64] = 0;
        for (int t = 1; t < kv; t++) {
            const double pert = 1.0e-7 * fmax(fabs(sm.eig[t]), 1.0);
            if (sm.eig[t] - sm.eig[t - 1] < pert) sm.eig[t] = sm.eig[t - 1] + pert;
            if (sm.eig[t] - sm.eig[t - 1] > ortol) start = t;
            sm.iv[64 + t] = start;
            big = max(big, t - start + 1);
        }
        sm.iv[0] = big;
        sm.small[0] = onen;
    }
    __syncthreads();
    // --- eigenvectors: one thread per vector; cluster members in rounds so that each one is projected
    //     against the finished earlier members
    {
        const int rounds = sm.iv[0], kvp = (kv + 31) & ~31;
        if (tid == 0 && count_step) { tm.slot[PDG_T_ROUNDS] += rounds; tm.slot[PDG_T_DENSITY_STEPS] += 1.0; }
        const double tiny = (F32 ? 1.2e-7 : 2.2e-16) * fmax(sm.small[0], 1.0);
        R *U0 = (R *)(wsf + pl.LU), *U1 = U0 + (size_t)N * kvp, *U2 = U1 + (size_t)N * kvp, *LM = U2 + (size_t)N * kvp;
        R *Y = LM + (size_t)N * kvp;
        unsigned char *PV = (unsigned char *)(Y + (size_t)N * kvp);
        for (int r = 0; r < rounds; r++) {
            for (int t = tid; t < kv; t += PDG_BLOCK) {
                const int cs = sm.iv[64 + t];
                if (t - cs != r) continue;
                R *y = z_in_smem ? Z + (size_t)t * ldz : Y + t;   // in place in the output row when Z is in shared memory
                inverse_iteration<R>(N, t, sm.eig[t], tiny, sm.d, sm.e, U0 + t, U1 + t, U2 + t, LM + t, PV + t, y, z_in_smem ? 1 : kvp, kvp,
                                  Z + (size_t)cs * ldz, t - cs, ldz, Z + (size_t)t * ldz);
            }
            __syncthreads();
        }
    }
    if (refine) {
        // eigenvalues to FP64 accuracy: the Rayleigh quotients z^T T z / z^T z of the inverse-iteration vectors (the
        // multisection's shifts carry FP32 resolution, enough for the vectors but not for Fermi occupancies)
        for (int t = tid; t < kv; t += PDG_BLOCK) {
            const R *z = Z + (size_t)t * ldz;
            double num = 0.0, den = 0.0;
            for (int i = 0; i < N; i++) {
                const double zi = (double)z[i];
                den = fma(zi, zi, den);
                num = fma(sm.d[i] * zi, zi, num);
                if (i + 1 < N) num = fma(2.0 * sm.e[i] * zi, (double)z[i + 1], num);
            }
            sm.eig[t] = num / den;
        }
        __syncthreads();
    }
    tm.lap(PDG_T_EIGENVECTORS);
    // --- back-transformation Z <- Q Z, Q = H_0 H_1 ... H_{N-3} with the reflectors stored in A
    if constexpr (F32) {
        if (N >= 32) { back_transform32(N, (float *)(wsf + pl.LU), A, sm, kv, Z); return; }   // rows of N floats
    }
    if (!F32 && N >= 32) {
        // blocked (compact WY, as LAPACK's dlarft / dlarfb): blocks of up to 16 consecutive reflectors, last
        // block first; block b is I - V T V^T with V the reflectors' unit lower-trapezoidal columns over rows
        // k0 + 1 .. N - 1 (row i of V is contiguous in the packed A) and T upper triangular.  Per block one GEMM
        // gives S = V^T V and W = V^T Z together, one warp builds T from S, W2 = T W, and a second GEMM applies
        // Z^T -= W2^T V^T (stores along Z's rows).  Same 2 N^2 kv flops as reflector-by-reflector, but Z and the
        // reflectors pass through the GEMM staging once per block instead of once per reflector and vector.
        const int nref = N - 2;
        double *Wm = wsf + pl.LU, *W2 = Wm + (size_t)16 * kv, *Sg = W2 + (size_t)16 * kv, *Tt = Sg + 256;
        for (int k0 = ((nref - 1) / 16) * 16; k0 >= 0; k0 -= 16) {
            const int nbk = min(16, nref - k0), m0 = N - k0 - 1;
            auto V = [&](int i, int c) -> double { return i < c ? 0.0 : (i == c ? 1.0 : A[plo(k0 + 1 + i, k0 + c)]); };
            tgemm<false, true>(nbk, 16 + kv, m0, [&](int c, int i) { return V(i, c); },
                               [&](int i, int j) { return j < 16 ? (j < nbk ? V(i, j) : 0.0) : (double)Z[(size_t)(j - 16) * ldz + k0 + 1 + i]; },
                               false, sm, [&](int c, int j, double v) {
                                   if (j < 16) Sg[c * 16 + j] = v;
                                   else Wm[(size_t)c * kv + (j - 16)] = v;
                               });
            if (w == 0) {   // T(c, c) = tau_c;  T(0:c, c) = -tau_c T(0:c, 0:c) S(0:c, c)
                for (int c = 0; c < nbk; c++) {
                    const double tau = sm.tau[k0 + c];
                    double t = 0.0;
                    if (lane < c) {
                        for (int j = lane; j < c; j++) t = fma(Tt[lane * 16 + j], Sg[j * 16 + c], t);
                        t *= -tau;
                    }
                    __syncwarp();
                    if (lane < 16) Tt[lane * 16 + c] = lane < c ? t : (lane == c ? tau : 0.0);
                    __syncwarp();
                }
            }
            __syncthreads();
            for (int e = tid; e < nbk * kv; e += PDG_BLOCK) {
                const int c = e / kv, t = e % kv;
                double acc = 0.0;
                for (int j = c; j < nbk; j++) acc = fma(Tt[c * 16 + j], Wm[(size_t)j * kv + t], acc);
                W2[(size_t)c * kv + t] = acc;
            }
            __syncthreads();
            tgemm<false, true>(kv, m0, nbk, [&](int t, int c) { return W2[(size_t)c * kv + t]; }, [&](int c, int i) { return V(i, c); },
                               false, sm, [&](int t, int i, double v) { Z[(size_t)t * ldz + k0 + 1 + i] -= v; });
        }
    } else {
        // reflector by reflector, one warp per vector
        for (int t = w; t < kv; t += PDG_WARPS) {
            R *zt = Z + (size_t)t * ldz;
            for (int k = N - 3; k >= 0; k--) {
                const double tau = sm.tau[k];
                if (tau == 0.0) continue;
                const int m = N - k - 1;
                double dt = 0.0;
                for (int i = lane; i < m; i += 32) dt = fma(i == 0 ? 1.0 : A[plo(k + 1 + i, k)], (double)zt[k + 1 + i], dt);
                dt = warp_sum(dt) * tau;
                for (int i = lane; i < m; i += 32) zt[k + 1 + i] = (R)fma(-dt, i == 0 ? 1.0 : A[plo(k + 1 + i, k)], (double)zt[k + 1 + i]);
                __syncwarp();
            }
        }
        __syncthreads();
    }
}

__device__ int occupancy_weights(const SCFArgs &a, int q, Smem &sm, double *wt);

// One density step.  W false: P = 2 Z^T Z over the wanted vectors (closed shell).  W true (every eigenpair computed,
// vec_occupied): P = sum_k w_k z_k z_k^T with the weights of density set occ_set's occupancies (occupancy_weights),
// whose occupancy energy is left in sm.small[128].
template <bool W = false>
__device__ double density_step(const SCFArgs &a, double *wsf, const double *F, double *P, Smem &sm, Timer &tm, bool make_base = false,
                               int occ_set = 0)
{
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int N = s.n_basis, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int kv = s.n_vec, ldz = sm.ldz;
    double *A = sm.amat ? sm.amat : wsf + pl.A;   // packed lower triangle
    double *Z = sm.zs ? sm.zs : wsf + pl.Z;       // wanted eigenvectors, kv rows of ldz
    for (int i = w; i < N; i += PDG_WARPS)
        for (int j = lane; j <= i; j += 32) A[plo(i, j)] = F[(size_t)i * N + j];
    __syncthreads();
    // --- Householder tridiagonalisation A = Q T Q^T (dsytd2 'L'), (2/3) N^3 FMA.  Per step: the product
    //     p = tau A22 v one thread per row (no reductions); K = tau (p.v)/2 and w = p - K v; the rank-2
    //     update of the lower triangle over all warps by flat element index, while warp 0 updates the
    //     first column of A22 and builds the next reflector from it (look-ahead).
    double *vc = sm.v, *vn = sm.v2;
    if (tid == 0) sm.d[0] = A[0];
    if (N >= 3 && w == 0) make_reflector(A, N, 0, vc, sm);
    __syncthreads();
    for (int k = 0; k + 2 < N; k++) {
        const int m = N - k - 1, c0 = k + 1, R = (m + 31) >> 5;
        const double tau = sm.tau[k];
        // items (row block rb, column segment q): Q segments per row so that short steps still spread over
        // the four FP64 units; each item leaves its partial products and its partial p.v
        const int Q = max(1, min(4, PDG_WARPS / R)), seg = (m + Q - 1) / Q;
        for (int item = w; item < R * Q; item += PDG_WARPS) {
            const int rb = item % R, qs = item / R, i = rb * 32 + lane;
            const int j0 = qs * seg, j1 = min(m, j0 + seg);
            double t = 0.0;
            if (i < m) {
                const int bi = plo(c0 + i, c0);
                int tj = plo(c0 + j0, c0);
                for (int j = j0; j < j1; j++) {
                    const int ad = (j <= i) ? bi + j : tj + i;
                    t = fma(A[ad], vc[j], t);
                    tj += c0 + j + 1;
                }
                sm.part[qs * N + i] = t;
            }
            const double pv = warp_sum(i < m ? t * vc[i] : 0.0);
            if (lane == 0) sm.dot[item] = pv;
        }
        __syncthreads();
        for (int rb = w; rb < R; rb += PDG_WARPS) {
            double sdot = 0.0;
            for (int q = lane; q < R * Q; q += 32) sdot += sm.dot[q];
            const double K = 0.5 * tau * tau * warp_sum(sdot);   // K = tau (p.v) / 2 with p = tau A v
            const int i = rb * 32 + lane;
            if (i < m) {
                double t = 0.0;
                for (int q = 0; q < Q; q++) t += sm.part[q * N + i];
                const double p = tau * t;
                sm.p[i] = p;
                sm.w[i] = fma(-K, vc[i], p);
            }
        }
        __syncthreads();
        if (w == 0) {
            const double v0 = vc[0], w0 = sm.w[0];
            for (int i = lane; i < m; i += 32) { const int ad = plo(c0 + i, c0); A[ad] = fma(-vc[i], w0, fma(-sm.w[i], v0, A[ad])); }
            __syncwarp();
            if (lane == 0) sm.d[c0] = A[plo(c0, c0)];
            if (m >= 3) make_reflector(A, N, c0, vn, sm);
            else if (lane == 0) { sm.e[c0] = A[plo(c0 + 1, c0)]; sm.tau[c0] = 0.0; }
        } else {
            const int nt = (m - 1) * m / 2;   // elements (i, j) of A22 with 1 <= j <= i < m
            for (int el = tid - 32; el < nt; el += PDG_BLOCK - 32) {   // warps 1 .. PDG_WARPS-1
                int ii = (int)((sqrtf(8.0f * (float)el + 1.0f) - 1.0f) * 0.5f);
                while ((ii + 1) * (ii + 2) / 2 <= el) ii++;
                while (ii * (ii + 1) / 2 > el) ii--;
                const int i = ii + 1, j = el - ii * (ii + 1) / 2 + 1;
                const int ad = plo(c0 + i, c0 + j);
                A[ad] = fma(-vc[i], sm.w[j], fma(-sm.w[i], vc[j], A[ad]));
            }
        }
        __syncthreads();
        double *tmp = vc; vc = vn; vn = tmp;
    }
    if (tid == 0) {
        if (N == 2) { sm.e[0] = A[plo(1, 0)]; sm.tau[0] = 0.0; }
        if (N >= 2) sm.d[N - 1] = A[plo(N - 1, N - 1)];
        sm.e[N - 1] = 0.0;
    }
    __syncthreads();
    tm.lap(PDG_T_TRIDIAGONAL);
    tridiag_vectors<double>(a, wsf, A, sm, tm, s.vec_occupied ? 0 : N - kv, kv, Z, ldz, sm.zs != nullptr, true,
                            W && a.occ_type == PDG_OCC_VARIABLE_FRACTIONAL);
    tm.lap(PDG_T_BACKTRANSFORM);
    // --- P = 2 Z^T Z (occupied) or 2 (1 - Z^T Z) (virtual), or sum_k w_k z_k z_k^T; lower triangle then mirrored
    const bool occ = s.vec_occupied;
    double *wt = sm.part;   // per-vector weights (the tridiagonalisation's partial sums are dead here)
    int kuse = kv;
    if constexpr (W) kuse = occupancy_weights(a, occ_set, sm, wt);
    double rms = 0.0;
    tgemm<false, false>(N, N, kuse, [&](int i, int k) { if constexpr (W) return wt[k] * Z[(size_t)k * ldz + i]; else return Z[(size_t)k * ldz + i]; },
                        [&](int k, int j) { return Z[(size_t)k * ldz + j]; }, true, sm, [&](int i, int j, double v) {
        if (j > i) return;
        double pn;
        if constexpr (W) pn = v;
        else pn = occ ? 2.0 * v : ((i == j ? 2.0 : 0.0) - 2.0 * v);
        const double dlt = pn - P[(size_t)i * N + j];
        rms += (i == j) ? dlt * dlt : 2.0 * dlt * dlt;
        P[(size_t)i * N + j] = pn;
        if (i != j) P[(size_t)j * N + i] = pn;
    });
    const double out = sqrt(block_sum(rms, sm.red)) / (double)N;
    tm.lap(PDG_T_DENSITY);
    if (make_base) {
        // base of the following perturbative steps: this step's matrix, density, wanted vectors and, from a second
        // pass over the same tridiagonal form in FP32, the complementary eigenvectors; all eigenvalues (wanted first)
        const int nc = N - kv;
        double *BF = wsf + pl.BF, *BP = wsf + pl.BP, *BZ = wsf + pl.BZ, *BL = wsf + pl.BL;
        for (size_t k = tid; k < (size_t)N * N; k += PDG_BLOCK) { BF[k] = F[k]; BP[k] = P[k]; }
        for (int e = tid; e < kv * N; e += PDG_BLOCK) BZ[(size_t)(e / N) * ldz + e % N] = Z[(size_t)(e / N) * ldz + e % N];
        for (int t = tid; t < kv; t += PDG_BLOCK) BL[t] = sm.eig[t];
        __syncthreads();
        // The vectors in FP32 are the operands of the products with small factors: the wanted ones rounded, the
        // complementary ones computed in FP32 (inverse iteration and back-transformation), since they enter the
        // perturbative steps only in products with dF or K.
        float *Zf = (float *)(wsf + pl.BW) + pert_dq_offset(N, kv) + 2 * (size_t)N * N, *Vf = Zf + (size_t)kv * N;
        for (int e = tid; e < kv * N; e += PDG_BLOCK) Zf[e] = (float)BZ[(size_t)(e / N) * ldz + e % N];
        __syncthreads();
        if (nc > 0) {
            tridiag_vectors<float>(a, wsf, A, sm, tm, s.vec_occupied ? kv : 0, nc, Vf, N, false, false);
            for (int t = tid; t < nc; t += PDG_BLOCK) BL[kv + t] = sm.eig[t];
        }
        __syncthreads();
        float *Gi = Vf + (size_t)nc * N;   // reciprocal gaps, the fixed-point sweeps' divisors
        for (int e = tid; e < nc * kv; e += PDG_BLOCK) Gi[e] = (float)(1.0 / (BL[e % kv] - BL[kv + e / kv]));
        __syncthreads();
        tm.lap(PDG_T_PERT_BASE);
    }
    return out;
}

// ----------------------------------------------------------------------------------------------------
// Base of the perturbative density steps: the block from FramePlan::BF to the end of a frame's workspace, either the
// frame's own (left by its last FP64 step) or a shared copy of another frame's (pdg_base_capture), read-only here.
struct PertBase { const double *BF, *BP; const float *Z32, *V32, *Gi; };

// Tensor memory (columns from tmem), the completion mbarrier and its phase of a CTA that may use tcgen05.
struct TCState { uint32_t tmem, bar, phase; };

// C[0:128, 0:Kp] = A[0:128, 0:K] B[0:Kp, 0:K]^T on the tensor cores (accumulator in tensor memory at tc.tmem, Kp
// columns), FP32 operands given by accessors (zero outside rows < ma / nb and K), each split into BF16 hi + mid + lo
// and multiplied as hi.hi + hi.mid + mid.hi + hi.lo + lo.hi + mid.mid (the FP32 value to ~2^-24; the three dropped
// products are below that).  K is staged in chunks of 32 columns through `stage` (shared memory, 16-byte aligned,
// 3 * (128 + Kp) * 64 bytes), one commit and bounded wait per chunk.  False when a wait ran out.
// AT / BT: the operand is stored with K as its slow index (a transposed accessor), so a chunk is read with
// consecutive threads on consecutive rows (coalesced) instead of consecutive K.
template <bool AT = false, bool BT = false, typename FA, typename FB>
__device__ bool tc_product_f32(TCState &tc, unsigned char *stage, int ma, int nb, int K, int Kp, FA fa, FB fb)
{
    const int tid = threadIdx.x;
    constexpr int KC = 32;
    const size_t pa = (size_t)TC_M * KC * 2, pbs = (size_t)Kp * KC * 2;   // bytes of one part of A and of B
    unsigned char *A0 = stage, *B0 = stage + 3 * pa;
    // each thread's elements of a chunk: all loads first (independent, in flight together), then the splits and
    // the shared-memory stores
    constexpr int UA = TC_M * KC / PDG_BLOCK, UB = 144 * KC / PDG_BLOCK;
    static_assert(TC_M * KC % PDG_BLOCK == 0 && 144 * KC % PDG_BLOCK == 0, "chunk elements per thread");
    for (int k0 = 0; k0 < K; k0 += KC) {
        float va[UA], vb[UB];
        // element e of a chunk: row e / KC, column e % KC (K fastest), or row e % rows, column e / rows (transposed)
        auto arow = [&](int e) { return AT ? e % TC_M : e / KC; };
        auto acol = [&](int e) { return AT ? e / TC_M : e % KC; };
        auto brow = [&](int e) { return BT ? e % Kp : e / KC; };
        auto bcol = [&](int e) { return BT ? e / Kp : e % KC; };
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int e = tid + u * PDG_BLOCK, r = arow(e), k = k0 + acol(e);
            va[u] = (r < ma && k < K) ? fa(r, k) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < UB; u++) {
            const int e = tid + u * PDG_BLOCK, r = brow(e), k = k0 + bcol(e);
            vb[u] = (e < Kp * KC && r < nb && k < K) ? fb(r, k) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int e = tid + u * PDG_BLOCK;
            __nv_bfloat16 h, m, l;
            bf16_split3(va[u], h, m, l);
            const uint32_t o = tc_offset(arow(e), acol(e), KC);
            *(__nv_bfloat16 *)(A0 + o) = h; *(__nv_bfloat16 *)(A0 + pa + o) = m; *(__nv_bfloat16 *)(A0 + 2 * pa + o) = l;
        }
#pragma unroll
        for (int u = 0; u < UB; u++) {
            const int e = tid + u * PDG_BLOCK;
            if (e >= Kp * KC) break;
            __nv_bfloat16 h, m, l;
            bf16_split3(vb[u], h, m, l);
            const uint32_t o = tc_offset(brow(e), bcol(e), KC);
            *(__nv_bfloat16 *)(B0 + o) = h; *(__nv_bfloat16 *)(B0 + pbs + o) = m; *(__nv_bfloat16 *)(B0 + 2 * pbs + o) = l;
        }
        tc_fence_proxy();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a = tc_smem_addr(A0), b = tc_smem_addr(B0);
            const uint32_t ah = a, am = a + (uint32_t)pa, al = a + 2 * (uint32_t)pa;
            const uint32_t bh = b, bm = b + (uint32_t)pbs, bl = b + 2 * (uint32_t)pbs;
            tc_product(tc.tmem, ah, 0, bh, Kp, KC, k0 > 0);
            tc_product(tc.tmem, ah, 0, bm, Kp, KC, true);
            tc_product(tc.tmem, am, 0, bh, Kp, KC, true);
            tc_product(tc.tmem, ah, 0, bl, Kp, KC, true);
            tc_product(tc.tmem, al, 0, bh, Kp, KC, true);
            tc_product(tc.tmem, am, 0, bm, Kp, KC, true);
            tc_commit(tc.bar);
        }
        const bool ok = mbar_wait(tc.bar, tc.phase, 1 << 22);
        tc.phase ^= 1u;
        if (__syncthreads_or(!ok)) return false;
    }
    tc_fence_after();
    return true;
}

// Thread (row r = 32 (warp % 4) + lane of the accumulator) reads its columns of C: warps 0-3 the first half of the
// 16-column chunks, warps 4-7 the rest; put(r, c, v) for r < 128, c < n.
template <typename Put>
__device__ void tc_readout(const TCState &tc, int Kp, int n, Put put)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int rr = 32 * (w & 3) + lane, nch = Kp / 16, half = (nch + 1) / 2, c0 = w < 4 ? 0 : half, c1 = w < 4 ? half : nch;
    for (int ch = c0; ch < c1; ch++) {
        float v[16];
        tc_ld16(tc.tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(ch * 16), v);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int c = ch * 16 + j;
            if (c < n) put(rr, c, v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
}

__device__ __forceinline__ PertBase pert_base(const double *blk, const FramePlan &pl, int N, int kv)
{
    PertBase b;
    b.BF = blk;
    b.BP = blk + (pl.BP - pl.BF);
    const float *bw = (const float *)(blk + (pl.BW - pl.BF));
    b.Z32 = bw + pert_dq_offset(N, kv) + 2 * (size_t)N * N;
    b.V32 = b.Z32 + (size_t)kv * N;
    b.Gi = b.V32 + (size_t)(N - kv) * N;
    return b;
}

// Largest |K| the perturbative step takes around a shared base.  It bounds the FP32 rounding carried into P (~1e-7
// |K| per product, 1.5e-8 at 0.15) and the truncation of U = -A + A^2 - A^3 + A^4 - A^5 (|K|^12, 1.3e-10); frames
// 0.03 A from the base geometry (RMS per coordinate) reach |K| ~ 0.1 with energies within 1e-7 Hartree of the FP64
// method's.
#ifndef PDG_PERT_KMAX_SHARED
#define PDG_PERT_KMAX_SHARED 0.15f
#endif
// Around a frame's own base (made by its FP64 step from a Fock matrix of the same geometry) the steps stay small:
// the limit keeps their rounding at ~2e-10, so that the mixed method reproduces the FP64 energies to 1e-8.
#ifndef PDG_PERT_KMAX
#define PDG_PERT_KMAX 2.0e-3f
#endif

// ----------------------------------------------------------------------------------------------------
// Perturbative density step (mixed method; no counterpart in the reference).  The last FP64 step left a base:
// its matrix F0, density P0, wanted eigenvectors Z0 (kv rows) with eigenvalues lambda, and the complementary
// eigenvectors V (nc = N - kv rows) with eigenvalues mu, all exact to FP64 round-off.  For the new matrix
// F = F0 + dF, the wanted invariant subspace is spanned by the rows of Z0 + K^T V, where K (nc x kv) solves the
// Riccati equation of block diagonalisation in the basis [Z0; V]:
//     E + M' K - K L' - K (E^T K) = (lambda_a - mu_i) K_ia,   E = V dF Z0^T,  M' = V dF V^T,  L' = Z0 dF Z0^T,
// solved by fixed-point iteration from K = E / (lambda_a - mu_i) (first-order perturbation theory).  The new
// projector differs from Z0^T Z0 by dQ = Z0^T W + Y^T (Z0 + W), with Y = K^T V, U = (1 + A)^-1 - 1 = -A + A^2 - A^3
// (A = K^T K) and W = Y + U (Z0 + Y); P = P0 + 2 dQ (occupied vectors) or P0 - 2 dQ (virtual).  Every FP32
// product here has a small factor (dF, K, Y, W), so its rounding error is ~1e-7 of a small quantity; only P0
// (FP64) carries the full magnitude.  Returns the RMS change of P, or -1 without touching P when the base no
// longer carries the step (the iteration does not settle, or K is not small): the caller then runs an FP64 step,
// which makes a new base.
__device__ double density_step_pert(const SCFArgs &a, double *wsf, const double *F, double *P, Smem &sm, Timer &tm, const PertBase &pb,
                                   bool warm_k, float kmax_limit, TCState *tc = nullptr)
{
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int N = s.n_basis, kv = s.n_vec, nc = N - kv, tid = threadIdx.x;
    const double *BF = pb.BF, *BP = pb.BP;
    float *D = (float *)(wsf + pl.BW), *T1 = D + (size_t)N * N, *E = T1 + (size_t)N * kv, *Lp = E + (size_t)nc * kv;
    float *T2 = Lp + (size_t)kv * kv, *Mp = T2 + (size_t)N * nc, *K = Mp + (size_t)nc * nc, *K2 = K + (size_t)nc * kv;
    float *EK = K2 + (size_t)nc * kv, *U = EK + (size_t)kv * kv, *Y = U + (size_t)kv * kv, *Wz = Y + (size_t)kv * N;
    float *DQ = Wz + (size_t)kv * N;   // Y, W (and dQ) stay for the DIIS save's commutator: pert_y_offset, pert_dq_offset
    if (nc <= 0) return -1.0;
    const long long t_coupling = tm.now();
    for (size_t k = tid; k < (size_t)N * N; k += PDG_BLOCK) D[k] = (float)(F[k] - BF[k]);
    __syncthreads();
    const float *Z32 = pb.Z32, *V32 = pb.V32, *Gi = pb.Gi;
    auto Zf = [&](int t, int i) { return Z32[(size_t)t * N + i]; };
    auto Vf = [&](int j, int i) { return V32[(size_t)j * N + i]; };
#ifndef PDG_SCF_NO_TENSOR
    const int Kp = (N + 15) & ~15;
    if (tc && N <= 144 && N > kv && sm.amat && smem_plan(N, kv, a.smem_limit).amat * 8 >= (size_t)3 * (TC_M + Kp) * 64) {
        // On the tensor cores: with Q = [Z0; V] (the base's orthonormal basis, Z32 and V32 contiguous: N rows of N),
        // C = Q dF Q^T holds L' (rows, columns < kv), E (rows >= kv, columns < kv) and M' (both >= kv).  R = Q dF and
        // C's first 128 rows come from two tensor-core products; C is symmetric, so its columns >= 128 give rows
        // >= 128 (the mirror); the corner of rows and columns >= 128 (N - 128 <= 16) is summed on the FP32 cores
        // from R's rows >= 128.  R lives where the DIIS save later puts dF (free here).  The staging chunks use the
        // shared-memory slot of the packed matrix (free between FP64 steps; large enough from N = 65 on).
        float *R32 = (float *)(wsf + pl.BW) + pert_dq_offset(N, kv) + (size_t)N * N;
        unsigned char *stage = (unsigned char *)sm.amat;
        auto Qf = [&](int t, int k) { return Z32[(size_t)t * N + k]; };
        auto put_c = [&](int r, int c, float v) {
            if (r >= N) return;
            if (r < kv) { if (c < kv) Lp[(size_t)r * kv + c] = v; }
            else if (c < kv) E[(size_t)(r - kv) * kv + c] = v;
            else Mp[(size_t)(r - kv) * nc + (c - kv)] = v;
        };
        if (!tc_product_f32(*tc, stage, min(N, TC_M), N, N, Kp, Qf, [&](int n, int k) { return D[(size_t)n * N + k]; })) return -2.0;
        tc_readout(*tc, Kp, N, [&](int r, int c, float v) { if (r < N) R32[(size_t)r * N + c] = v; });
        for (int e = tid; e < (N - TC_M) * N; e += PDG_BLOCK) {   // R's rows >= 128 (dF symmetric: column c of dF
            const int r = TC_M + e / N, c = e % N;                // read along its rows, coalesced over c)
            float acc = 0.0f;
#pragma unroll 4
            for (int k = 0; k < N; k++) acc = fmaf(Qf(r, k), D[(size_t)k * N + c], acc);
            R32[(size_t)r * N + c] = acc;
        }
        __syncthreads();
        if (!tc_product_f32(*tc, stage, min(N, TC_M), N, N, Kp, [&](int r, int k) { return R32[(size_t)r * N + k]; }, Qf)) return -2.0;
        tc_readout(*tc, Kp, N, [&](int r, int c, float v) {
            if (r >= N) return;
            put_c(r, c, v);
            if (c >= TC_M) put_c(c, r, v);
        });
        for (int e = tid; e < (N - TC_M) * (N - TC_M); e += PDG_BLOCK) {   // the corner
            const int r = TC_M + e / (N - TC_M), c = TC_M + e % (N - TC_M);
            float acc = 0.0f;
            for (int k = 0; k < N; k++) acc = fmaf(R32[(size_t)r * N + k], Qf(c, k), acc);
            put_c(r, c, acc);
        }
        __syncthreads();
    } else
#endif
    {
    // T1 = dF Z0^T (N x kv);  E = V T1 (nc x kv);  L' = Z0 T1 (kv x kv)
    tgemm32<true, true>(N, kv, N, [&](int i, int k) { return D[(size_t)i * N + k]; }, [&](int k, int t) { return Zf(t, k); }, false, sm,
                       [&](int i, int t, double v) { T1[(size_t)i * kv + t] = (float)v; });
    tgemm32<true, false>(nc, kv, N, [&](int j, int k) { return Vf(j, k); }, [&](int k, int t) { return T1[(size_t)k * kv + t]; }, false, sm,
                        [&](int j, int t, double v) { E[(size_t)j * kv + t] = (float)v; });
    tgemm32<true, false>(kv, kv, N, [&](int b, int k) { return Zf(b, k); }, [&](int k, int t) { return T1[(size_t)k * kv + t]; }, false, sm,
                        [&](int b, int t, double v) { Lp[(size_t)b * kv + t] = (float)v; });
    // T2 = dF V^T (N x nc);  M' = V T2 (nc x nc)
    tgemm32<true, true>(N, nc, N, [&](int i, int k) { return D[(size_t)i * N + k]; }, [&](int k, int j) { return Vf(j, k); }, false, sm,
                       [&](int i, int j, double v) { T2[(size_t)i * nc + j] = (float)v; });
    tgemm32<true, false>(nc, nc, N, [&](int j, int k) { return Vf(j, k); }, [&](int k, int l) { return T2[(size_t)k * nc + l]; }, false, sm,
                        [&](int j, int l, double v) { Mp[(size_t)j * nc + l] = (float)v; });
    }
    tm.add(PDG_T_PERT_COUPLING, t_coupling);
    const long long t_solve = tm.now();
    // K from first-order theory, or the previous step's K around the same base (warm_k), then the fixed-point
    // iteration (each sweep one GEMM over [M' | -K] [K ; L' + E^T K]); the last iterate goes back to the first buffer
    float *const K0 = K;
    if (!warm_k) {
        for (int e = tid; e < nc * kv; e += PDG_BLOCK) K[e] = E[e] * Gi[e];
        __syncthreads();
    }
    bool settled = false;
    float kmax = 0.f;
    for (int it = 0; it < 12 && !settled; it++) {
        tgemm32<false, false>(kv, kv, nc, [&](int b, int j) { return E[(size_t)j * kv + b]; }, [&](int j, int t) { return K[(size_t)j * kv + t]; },
                      false, sm, [&](int b, int t, double v) { EK[(size_t)b * kv + t] = (float)v; });
        float dmax = 0.f, km = 0.f;
        tgemm32<true, false>(nc, kv, nc + kv,
            [&](int j, int k) { return k < nc ? Mp[(size_t)j * nc + k] : -K[(size_t)j * kv + (k - nc)]; },
            [&](int k, int t) { return k < nc ? K[(size_t)k * kv + t] : Lp[(size_t)(k - nc) * kv + t] + EK[(size_t)(k - nc) * kv + t]; },
     false, sm, [&](int j, int t, double v) {
                const size_t e = (size_t)j * kv + t;
                const float kn = (E[e] + (float)v) * Gi[e];
                K2[e] = kn;
                dmax = fmaxf(dmax, fabsf(kn - K[e]));
                km = fmaxf(km, fabsf(kn));
            });
        dmax = (float)block_max((double)dmax, sm.red); km = (float)block_max((double)km, sm.red);
        float *tmp = K; K = K2; K2 = tmp;
        kmax = km;
        settled = dmax <= 1.0e-5f * km + 1.0e-30f;   // remaining error ~ (contraction) x this change
        if (tid == 0) tm.slot[PDG_T_PERT_SWEEPS] += 1.0;
    }
    if (K != K0) {
        for (int e = tid; e < nc * kv; e += PDG_BLOCK) K0[e] = K[e];
        __syncthreads();
        K2 = K;
        K = K0;
    }
    tm.add(PDG_T_PERT_SOLVE, t_solve);
    const long long t_density = tm.now();
    if (!settled || !(kmax < kmax_limit)) {
        if (tid == 0) { tm.slot[PDG_T_PERT_FALLBACKS] += 1.0; tm.slot[PDG_T_PERT_FAIL_K] = settled ? (double)kmax : -(double)kmax; }
        tm.lap(PDG_T_PERT);
        return -1.0;
    }
    // Y = K^T V (kv x N);  U = -K^T K (kv x kv)
    tgemm32<false, false>(N, kv, nc, [&](int i, int j) { return Vf(j, i); }, [&](int j, int t) { return K[(size_t)j * kv + t]; }, false, sm,
                         [&](int i, int t, double v) { Y[(size_t)t * N + i] = (float)v; });   // Y^T = V^T K
    if (tid == 0) tm.slot[PDG_T_PERT_KMAX] = fmax(tm.slot[PDG_T_PERT_KMAX], (double)kmax);
    // U = (1 + K^T K)^-1 - 1 = -A S4 + O(|K|^12), A = K^T K, by Horner: S1 = 1 - A, S(r+1) = 1 - A S(r) (kv x kv;
    // EK holds A, Lp and U (free after the sweeps) take the S in turn, and Lp the result)
    tgemm32<false, false>(kv, kv, nc, [&](int t, int j) { return K[(size_t)j * kv + t]; }, [&](int j, int c) { return K[(size_t)j * kv + c]; },
                  false, sm, [&](int t, int c, double v) { EK[(size_t)t * kv + c] = (float)v; });
    for (int e = tid; e < kv * kv; e += PDG_BLOCK) Lp[e] = (e / kv == e % kv ? 1.f : 0.f) - EK[e];
    __syncthreads();
    {
        float *Sa = Lp, *Sb = U;
        for (int r = 0; r < 3; r++) {
            tgemm32<true, false>(kv, kv, kv, [&](int t, int j) { return EK[(size_t)t * kv + j]; }, [&](int j, int c) { return Sa[(size_t)j * kv + c]; },
                           false, sm, [&](int t, int c, double v) { Sb[(size_t)t * kv + c] = (float)((t == c ? 1.0 : 0.0) - v); });
            float *tmp = Sa; Sa = Sb; Sb = tmp;
        }
        // Sa = S4 (in U); the result into Lp
        tgemm32<true, false>(kv, kv, kv, [&](int t, int j) { return EK[(size_t)t * kv + j]; }, [&](int j, int c) { return Sa[(size_t)j * kv + c]; },
                       false, sm, [&](int t, int c, double v) { Sb[(size_t)t * kv + c] = (float)(-v); });
        U = Sb;
    }
    // W = Y + U (Z0 + Y)
    tgemm32<false, true>(N, kv, 2 * kv, [&](int i, int k) { return k < kv ? Zf(k, i) : Y[(size_t)(k - kv) * N + i]; },
                        [&](int k, int t) { return U[(size_t)t * kv + (k < kv ? k : k - kv)]; }, false, sm,
                        [&](int i, int t, double v) { Wz[(size_t)t * N + i] = (float)((double)Y[(size_t)t * N + i] + v); });   // W^T
    // dQ = Z0^T W + Y^T (Z0 + W) (symmetric; lower triangle) and P = P0 +- 2 dQ
    const double c = s.vec_occupied ? 2.0 : -2.0;
    double rms = 0.0;
    auto dqa = [&](int i, int k) { return k < kv ? Zf(k, i) : Y[(size_t)(k - kv) * N + i]; };
    auto dqb = [&](int j, int k) { return k < kv ? Wz[(size_t)k * N + j] : Zf(k - kv, j) + Wz[(size_t)(k - kv) * N + j]; };
    auto dq_put = [&](int i, int j, double v) {   // i >= j
        const double pn = BP[(size_t)i * N + j] + c * v;
        const double dlt = pn - P[(size_t)i * N + j];
        rms += (i == j) ? dlt * dlt : 2.0 * dlt * dlt;
        P[(size_t)i * N + j] = pn;
        P[(size_t)j * N + i] = pn;
        DQ[(size_t)i * N + j] = (float)v;
        DQ[(size_t)j * N + i] = (float)v;
    };
    // (on the FP32 cores: P takes dQ at full weight, and around a frame's own base the steps need its rounding at
    // ~1e-10, which the tensor-core products' FP32 accumulation does not keep)
    tgemm32<false, false>(N, N, 2 * kv, dqa, [&](int k, int j) { return dqb(j, k); }, true, sm, [&](int i, int j, double v) {
        if (j > i) return;
        dq_put(i, j, v);
    });
    const double out = sqrt(block_sum(rms, sm.red)) / (double)N;
    tm.add(PDG_T_PERT_DENSITY, t_density);
    if (tid == 0) tm.slot[PDG_T_PERT_STEPS] += 1.0;
    tm.lap(PDG_T_PERT);
    return out;
}

// ----------------------------------------------------------------------------------------------------
// Mixed density step: SP2 purification (Niklasson's second-order spectral projection) with every product
// X X on the tensor cores as kprod split-BF16 partial products accumulated in FP32 (N <= 144: one M = 128
// tcgen05 tile, rows >= 128 by symmetry, the trailing corner on FP32 cores).  X0 = (e_max - F) / (e_max -
// e_min) from Gershgorin bounds maps the occupied spectrum to [~1, 1]; each step takes X^2 or 2X - X^2,
// whichever trace is closer to n_occ, until the idempotency defect tr X - tr X^2 stops falling.  P = X + X^T
// (closed shell, symmetrised).  The FP32 iterate lives in the workspace matrix A; the BF16 parts in the
// shared-memory slot of the packed matrix.  Returns the RMS change of P, or -1 when a tensor-core wait ran
// out (P is then left unchanged).

// Sum of the BF16 parts of eight consecutive iterate elements (16 bytes of each part array).
__device__ __forceinline__ void bf16_sum8(const uint4 &a, const uint4 &b, const uint4 &c, float *x)
{
    const __nv_bfloat16 *pa = (const __nv_bfloat16 *)&a, *pb = (const __nv_bfloat16 *)&b, *pc = (const __nv_bfloat16 *)&c;
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = __bfloat162float(pa[j]) + __bfloat162float(pb[j]) + __bfloat162float(pc[j]);
}

__device__ double density_step_mixed(const SCFArgs &a, double *wsf, const double *F, double *P, Smem &sm, Timer &tm,
                                     TCState &tc, int kprod)
{
    const DeviceSystem &s = a.s;
    const int N = s.n_basis, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int Kp = (N + 15) & ~15, R = Kp > TC_M ? Kp : TC_M, m2 = Kp - TC_M;   // second tile: rows m2 .. m2+127
    const size_t NN4 = ((size_t)N * N + 3) & ~size_t(3);
    // The iterate X lives only as its BF16 parts hi + mid + lo (24 significant bits, the FP32 value): hi and mid in
    // shared memory as the tensor-core operands, lo in the workspace region LO.  With 6 partial products the second
    // product phase copies lo over mid in shared memory, so mid is also kept in the workspace (region A).
    float *P32 = (float *)(wsf + a.plan.A) + 2 * NN4;
    unsigned char *ph = (unsigned char *)sm.amat, *pm = ph + (size_t)R * Kp * 2;
    unsigned char *plo_g = (unsigned char *)(wsf + a.plan.LO), *pmid_g = (unsigned char *)(wsf + a.plan.A);
    // the part of the current iterate outside shared memory at readout time (shared memory then holds hi and
    // either mid (3 products) or lo (6 products))
    const unsigned char *third = kprod == 6 ? pmid_g : plo_g;
    const double nocc = (double)s.n_occ;
    const long long t_setup = tm.now();
    // Gershgorin bounds and X0 = (e_max - F) / (e_max - e_min)
    double lo = 1e300, hi = -1e300;
    for (int i = w; i < N; i += PDG_WARPS) {
        double off = 0.0;
        for (int j = lane; j < N; j += 32) if (j != i) off += fabs(F[(size_t)i * N + j]);
        off = warp_sum(off);
        const double d = F[(size_t)i * N + i];
        lo = fmin(lo, d - off); hi = fmax(hi, d + off);
    }
    lo = -block_max(-lo, sm.red); hi = block_max(hi, sm.red);
    const float scale = (float)(1.0 / fmax(hi - lo, 1e-12)), fhi = (float)hi;
    // BF16 parts of X0 (rows beyond N and the padding zero), its trace and squared norm; later iterates get their
    // parts from the readout
    float trl = 0.0f, sql = 0.0f;
    for (int e = tid; e < R * Kp; e += PDG_BLOCK) {
        const int r = e / Kp, c = e % Kp;
        const float x = (r < N && c < N) ? ((r == c ? fhi : 0.0f) - (float)F[(size_t)r * N + c]) * scale : 0.0f;
        trl += (r == c) ? x : 0.0f; sql = fmaf(x, x, sql);
        __nv_bfloat16 h, m, l;
        bf16_split3(x, h, m, l);
        const uint32_t o = tc_offset(r, c, Kp);
        *(__nv_bfloat16 *)(ph + o) = h;
        *(__nv_bfloat16 *)(pm + o) = m;
        *(__nv_bfloat16 *)(plo_g + o) = l;
        if (kprod == 6) *(__nv_bfloat16 *)(pmid_g + o) = m;
    }
    const double2 ts = block_sum2((double)trl, (double)sql, sm.red);
    double tr = ts.x, sq = ts.y;
    tm.add(PDG_T_PUR_SETUP, t_setup);
    double defect_1 = 1e300, defect_2 = 1e300;   // defects of the last two iterations
    const int rr = 32 * (w & 3) + lane, nch = Kp / 16, half = (nch + 1) / 2, c0 = w < 4 ? 0 : half, c1 = w < 4 ? half : nch;
    for (int it = 0; it < 100; it++) {
        const bool square = fabs(sq - nocc) < fabs(2.0 * tr - sq - nocc);   // X <- X^2, else 2X - X^2
        const long long t_products = tm.now();
        tc_fence_proxy();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // tile 1: rows 0..127 x all Kp columns (tensor-memory columns 0..Kp-1); tile 2, when N > 128: rows
        // m2..m2+127 x columns 128..Kp-1 (tensor-memory columns Kp..Kp+m2-1), whose last m2 lanes are the corner
        const uint32_t t2 = tc.tmem + (uint32_t)Kp;
        if (tid == 0) {
            const uint32_t H = tc_smem_addr(ph), M = tc_smem_addr(pm);
            tc_product(tc.tmem, H, 0, H, Kp, Kp, false);
            tc_product(tc.tmem, H, 0, M, Kp, Kp, true);
            tc_product(tc.tmem, M, 0, H, Kp, Kp, true);
            if (kprod == 6) tc_product(tc.tmem, M, 0, M, Kp, Kp, true);
            if (m2 > 0) {
                tc_product(t2, H, m2, H, m2, Kp, false, TC_M);
                tc_product(t2, H, m2, M, m2, Kp, true, TC_M);
                tc_product(t2, M, m2, H, m2, Kp, true, TC_M);
                if (kprod == 6) tc_product(t2, M, m2, M, m2, Kp, true, TC_M);
            }
            tc_commit(tc.bar);
        }
        bool ok = mbar_wait(tc.bar, tc.phase, 1 << 22);
        tc.phase ^= 1u;
        if (kprod == 6 && __syncthreads_and(ok)) {
            // second phase: the lo parts into the mid array (hi.lo + lo.hi)
            tc_fence_after();
            const uint4 *src = (const uint4 *)plo_g;
            uint4 *dst = (uint4 *)pm;
            for (int e = tid; e < R * Kp / 8; e += PDG_BLOCK) dst[e] = src[e];
            tc_fence_proxy();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const uint32_t H = tc_smem_addr(ph), L = tc_smem_addr(pm);
                tc_product(tc.tmem, H, 0, L, Kp, Kp, true);
                tc_product(tc.tmem, L, 0, H, Kp, Kp, true);
                if (m2 > 0) { tc_product(t2, H, m2, L, m2, Kp, true, TC_M); tc_product(t2, L, m2, H, m2, Kp, true, TC_M); }
                tc_commit(tc.bar);
            }
            ok = mbar_wait(tc.bar, tc.phase, 1 << 22);
            tc.phase ^= 1u;
        }
        if (__syncthreads_or(!ok)) return -1.0;
        tc_fence_after();
        tm.add(PDG_T_PUR_PRODUCTS, t_products);
        const long long t_readout = tm.now();
        // X <- X X or 2X - X X.  Thread (row r) reads its 16 product columns from tensor memory and, for 2X - X X,
        // the old X of the same elements as the sum of its parts (16-byte loads per 8 columns); then writes the
        // new parts in place (the products are complete, so the operand arrays are free; each element is read
        // and written by the same thread).  X X is symmetric: tile 1's columns >= 128 also give rows >= 128 (the
        // mirror, one element at a time) and tile 2's last lanes the corner; padding columns stay zero.
        float trn = 0.0f, sqn = 0.0f;
        for (int ch = c0; ch < c1; ch++) {
            float v[16];
            tc_ld16(tc.tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(ch * 16), v);
            if (rr < N) {
                float xv[16];
                if (!square) {
#pragma unroll
                    for (int g = 0; g < 2; g++) {
                        const uint32_t o = tc_offset(rr, ch * 16 + 8 * g, Kp);
                        const uint4 pc = *(const uint4 *)(third + o), pa = *(const uint4 *)(ph + o), pb = *(const uint4 *)(pm + o);
                        bf16_sum8(pa, pb, pc, xv + 8 * g);
                    }
                }
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = ch * 16 + j;
                    const float xn = c >= N ? 0.0f : (square ? v[j] : 2.0f * xv[j] - v[j]);
                    xv[j] = xn;
                    sqn = fmaf((c >= TC_M) ? 2.0f * xn : xn, xn, sqn);
                    if (c == rr) trn += xn;
                }
#pragma unroll
                for (int g = 0; g < 2; g++) {
                    __align__(16) __nv_bfloat16 hv[8], mv[8], lv[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) bf16_split3(xv[8 * g + j], hv[j], mv[j], lv[j]);
                    const uint32_t o = tc_offset(rr, ch * 16 + 8 * g, Kp);
                    *(uint4 *)(ph + o) = *(const uint4 *)hv;
                    *(uint4 *)(pm + o) = *(const uint4 *)mv;
                    *(uint4 *)(plo_g + o) = *(const uint4 *)lv;
                    if (kprod == 6) *(uint4 *)(pmid_g + o) = *(const uint4 *)mv;
                }
#pragma unroll
                for (int j = 0; j < 16; j++) {   // rows >= 128 of the operands: the mirror (c, r)
                    const int c = ch * 16 + j;
                    if (c < TC_M || c >= N) continue;
                    __nv_bfloat16 h, m, l;
                    bf16_split3(xv[j], h, m, l);
                    const uint32_t o = tc_offset(c, rr, Kp);
                    *(__nv_bfloat16 *)(ph + o) = h;
                    *(__nv_bfloat16 *)(pm + o) = m;
                    *(__nv_bfloat16 *)(plo_g + o) = l;
                    if (kprod == 6) *(__nv_bfloat16 *)(pmid_g + o) = m;
                }
            }
        }
        if (m2 > 0 && w == 3) {   // lanes 128-m2 .. 127 of tile 2 hold corner rows 128 .. Kp-1
            float v[16];
            tc_ld16(t2 + ((uint32_t)96 << 16), v);
            const int r = m2 + 96 + lane;   // matrix row of this lane in tile 2
            if (r >= TC_M && r < N) {
                for (int j = 0; j < m2 && j < 16; j++) {
                    const int c = TC_M + j;
                    if (c >= N) continue;
                    const uint32_t o = tc_offset(r, c, Kp);
                    float xn = v[j];
                    if (!square) {
                        const float xo = __bfloat162float(*(const __nv_bfloat16 *)(ph + o)) + __bfloat162float(*(const __nv_bfloat16 *)(pm + o))
                                       + __bfloat162float(*(const __nv_bfloat16 *)(third + o));
                        xn = 2.0f * xo - v[j];
                    }
                    sqn = fmaf(xn, xn, sqn);
                    if (c == r) trn += xn;
                    __nv_bfloat16 h, m, l;
                    bf16_split3(xn, h, m, l);
                    *(__nv_bfloat16 *)(ph + o) = h;
                    *(__nv_bfloat16 *)(pm + o) = m;
                    *(__nv_bfloat16 *)(plo_g + o) = l;
                    if (kprod == 6) *(__nv_bfloat16 *)(pmid_g + o) = m;
                }
            }
        }
        tc_fence_before();
        tm.add(PDG_T_PUR_READOUT, t_readout);
        const long long t_control = tm.now();
        const double2 tsn = block_sum2((double)trn, (double)sqn, sm.red);
        tr = tsn.x; sq = tsn.y;
        const double defect = tr - sq;   // sum of lambda (1 - lambda) over the spectrum
        if (tid == 0) tm.slot[PDG_T_SP2_ITERATIONS] += 1.0;
        // converged (after Kruchinina, Rudberg and Rubensson's criterion for SP2): in the asymptotic regime the
        // defect falls quadratically every two steps until rounding dominates; stop at the first step where it
        // no longer falls below the value two steps back.  The regime is entered only once every eigenvalue is
        // within the products' precision of 0 or 1 (defect below 1e-3 for 3 partial products, 1e-5 for 6):
        // before that, a nearly degenerate HOMO/LUMO pair separating slowly around 1/2 also stalls the defect.
        const double floor_defect = kprod == 6 ? 1e-5 : 1e-3;
        tm.add(PDG_T_PUR_CONTROL, t_control);
        if ((defect < floor_defect && defect >= defect_2) || defect < 1e-9 * nocc || it >= 80) break;
        defect_2 = defect_1; defect_1 = defect;
    }
    // P = X + X^T from the parts of the last iterate (hi and mid in shared memory, lo in the workspace), in FP64
    // for the SCF and in FP32 (N x round4(N)) for the commutator of the next DIIS save
    const long long t_finish = tm.now();
    double rms = 0.0;
    const int N4 = (N + 3) & ~3;
    auto xval = [&](int i, int j) {
        const uint32_t o = tc_offset(i, j, Kp);
        return __bfloat162float(*(const __nv_bfloat16 *)(ph + o)) + __bfloat162float(*(const __nv_bfloat16 *)(pm + o))
             + __bfloat162float(*(const __nv_bfloat16 *)(plo_g + o));
    };
    const int npk = N * (N + 1) / 2;
    for (int q0 = tid; q0 < npk; q0 += 2 * PDG_BLOCK) {
        int ii[2], jj[2];
        float xij[2], xji[2];
        double po[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {   // element (i >= j) of packed index q; its loads issued before any store
            const int q = q0 + u * PDG_BLOCK;
            int i = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
            while ((i + 1) * (i + 2) / 2 <= q) i++;
            while (i * (i + 1) / 2 > q) i--;
            ii[u] = i; jj[u] = q - i * (i + 1) / 2;
            if (q < npk) { xij[u] = xval(i, jj[u]); xji[u] = xval(jj[u], i); po[u] = P[(size_t)i * N + jj[u]]; }
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (q0 + u * PDG_BLOCK >= npk) continue;
            const int i = ii[u], j = jj[u];
            const float p32 = xij[u] + xji[u];
            const double pn = (double)xij[u] + (double)xji[u], dlt = pn - po[u];
            rms += (i == j) ? dlt * dlt : 2.0 * dlt * dlt;
            P[(size_t)i * N + j] = pn;
            P[(size_t)j * N + i] = pn;
            P32[(size_t)i * N4 + j] = p32;
            P32[(size_t)j * N4 + i] = p32;
        }
    }
    for (int e = tid; e < N * (N4 - N); e += PDG_BLOCK) P32[(size_t)(e / (N4 - N)) * N4 + N + e % (N4 - N)] = 0.0f;
    const double out = sqrt(block_sum(rms, sm.red)) / (double)N;
    tm.add(PDG_T_PUR_FINISH, t_finish);
    if (tid == 0) tm.slot[PDG_T_PURIFICATION_STEPS] += 1.0;
    tm.lap(PDG_T_PURIFICATION);
    return out;
}

// ----------------------------------------------------------------------------------------------------
// The SCF of frame f of a (the whole of a batch item's SCF with f = 0), on shm; tc is the CTA's tensor memory
// and completion barrier when tc_ok (allocated by the kernel).
__device__ __forceinline__ void scf_frame(const SCFArgs &a, const int f, double *shm, TCState &tc, const bool tc_ok)
{
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, N = s.n_basis;
    const size_t NN = (size_t)N * N;
    Smem sm = carve(shm, N, s.n_vec, a.smem_limit);
    double *wsf = a.ws + (size_t)f * pl.stride;
    double *H = wsf + pl.H, *F = wsf + pl.F, *P = a.density + (size_t)f * NN;
    const double *tei = wsf + pl.tei;
    double *Bm = wsf + pl.misc;   // DIIS B matrix, PDG_MAX_HISTORY^2
    Timer tm;
    tm.slot = wsf + pl.misc + PDG_MAX_HISTORY * PDG_MAX_HISTORY;
    long long t_begin = clock64();
    if (tid < PDG_NTIMERS) tm.slot[tid] = 0.0;
    if (tid == 0) {
        unsigned int smid; unsigned long long gt;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
        tm.slot[PDG_T_SM_ID] = (double)smid; tm.slot[PDG_T_START_NS] = (double)gt;
    }
    __syncthreads();
    tm.start();
    // nuclear energy: sum of the pair terms in pair order
    double en = 0.0;
    for (int p = tid; p < s.n_pairs; p += PDG_BLOCK) en += wsf[pl.pair_e + (size_t)p * PDG_PAIR_E_STRIDE + 20];
    en = block_sum(en, sm.red);
    double base = 0.0;
    for (int A = tid; A < s.n_atoms; A += PDG_BLOCK) { const double *E = elem(s, s.atom_elem[A]); base += E[PDG_E_EHEAT] - E[PDG_E_EISOL]; }
    base = block_sum(base, sm.red);
#ifdef PDG_SCF_NO_TENSOR
    const bool want_mixed = false, tc_pert = false;
#else
    const bool want_mixed = tc_ok && a.fock_only != 1 && a.o.density_step != 0 && N <= 144 && sm.amat != nullptr;
    const bool tc_pert = tc_ok && N <= 144 && sm.amat != nullptr;   // the perturbative steps' coupling products
#endif
    bool mixed = want_mixed, last_mixed = false;
    int n_mixed = 0;
    bool valid = a.use_density == 1;   // 2: a start guess, which the first density step replaces before DIIS sees it
    if (!valid) {   // uniform diagonal guess (QCOnePDM.c:326-331)
        double g = (double)s.n_electrons / (double)N;
        for (size_t k = tid; k < NN; k += PDG_BLOCK) P[k] = ((k / N) == (k % N)) ? g : 0.0;
    }
    __syncthreads();
    double e1, e2, eq;
    if (a.fock_only == 2) {   // one density step for the given Fock matrices (pdg_density)
        for (size_t k = tid; k < NN; k += PDG_BLOCK) F[k] = a.fock_out[(size_t)f * NN + k];
        __syncthreads();
        const double r = want_mixed ? density_step_mixed(a, wsf, F, P, sm, tm, tc, a.o.density_step) : density_step(a, wsf, F, P, sm, tm);
        if (tid == 0) {
            double *E = a.energies + (size_t)f * PDG_NENERGY;
            for (int k = 0; k < PDG_NENERGY; k++) E[k] = 0.0;
            E[PDG_EN_RMS_DENSITY] = r;
            a.status[f] = r < 0.0 ? PDG_TENSOR_TIMEOUT : PDG_OK;
        }
        return;
    }
    if (a.fock_only) {
        fock_build(a, f, H, P, F, tei, sm, &e1, &e2, &eq, wsf + pl.P0);
        for (size_t k = tid; k < NN; k += PDG_BLOCK) a.fock_out[(size_t)f * NN + k] = F[k];
        if (tid == 0) {
            double *E = a.energies + (size_t)f * PDG_NENERGY;
            E[0] = e1 + e2 + eq; E[1] = e1 + e2; E[2] = en; E[3] = base; E[4] = eq; E[5] = e1; E[6] = e2; E[7] = 0.0;
        }
        return;
    }
    const pdg_scf_options &o = a.o;
    const int hist = o.history, hl = pl.hist_len;
    int *ctl = sm.iv;   // ctl[1] matnum, ctl[2..17] matind
    double *cf = sm.small + 32;   // DIIS coefficients
    if (tid == 0) { ctl[1] = 0; for (int i = 0; i < hist; i++) ctl[2 + i] = i; }
    int iteration = 0, converged = 0, qdiis = 0, qrca = o.use_rca ? 1 : 0, st = PDG_NOT_CONVERGED;
    bool rca_prev = false;   // rP, rF hold the last cycle's P, F (RCA_Save)
    double eold = 0.0, deltaeold = 0.0, rms = 0.0, eel = 0.0;
    __syncthreads();
    int ncyc = 0;
    bool have_z = false;   // P is the density of the vectors in Z
    bool have_pert = false, base_ok = false;   // P is a perturbative step's density; the base of those steps is valid
    // Mixed method: the Fock matrix of the last FP64 density step (the extrapolated one, still in F when the loop
    // comes round), kept so that the next DIIS save can form its commutator from the small difference F - F~
    double *Ft = wsf + pl.A;
    const bool delta_commutator = o.density_step != 0;
    // A shared base (mixed method): every density step is a perturbative step around it, with no purification, until
    // one fails (K not small); that frame then takes an FP64 step, which makes its own base.  Without a start
    // density the SCF starts from the base's density P0 = 2 Z0^T Z0, which commutes with F0: F = F0 stands for the
    // matrix it was made from, so the first DIIS save already takes the difference commutator.
    bool use_shared = delta_commutator && a.base != nullptr;
    // The mixed method forms the first DIIS error of a caller's start density (a learned guess, a previous step's
    // density) in FP32 as well, from an FP32 copy of P: no FP64 N^3 product for a vector that only steers DIIS
    bool fp32_start = delta_commutator && a.use_density == 1;
    if (fp32_start) {
        const int N4 = (N + 3) & ~3;
        float *P32 = (float *)(wsf + pl.A) + 2 * ((NN + 3) & ~size_t(3));
        for (int e = tid; e < N * N4; e += PDG_BLOCK) {
            const int i = e / N4, j = e % N4;
            P32[e] = j < N ? (float)P[(size_t)i * N + j] : 0.0f;
        }
        __syncthreads();
    }
    bool warm_k = false;   // the perturbative step's K buffer holds the last solution around the current base
    auto cur_base = [&]() { return pert_base(use_shared ? a.base : wsf + pl.BF, pl, N, s.n_vec); };
    if (use_shared) {
        mixed = false;
        base_ok = true;
        if (a.use_density == 0) {
            const PertBase b0 = cur_base();
            for (size_t k = tid; k < NN; k += PDG_BLOCK) { P[k] = b0.BP[k]; F[k] = b0.BF[k]; }
            valid = true;
            have_z = true;
        }
        __syncthreads();
    }
    while (iteration < o.maximum_scf_cycles && !converged) {
        if (delta_commutator && (have_z || have_pert)) {
            for (size_t k = tid; k < NN; k += PDG_BLOCK) Ft[k] = F[k];
            __syncthreads();
        }
        fock_build(a, f, H, P, F, tei, sm, &e1, &e2, &eq, wsf + pl.P0);
        tm.lap(PDG_T_FOCK);
        ncyc++;
        eel = e1 + e2 + eq;
        if (!isfinite(eel)) { st = PDG_NAN; break; }
        converged = (iteration > 0) && !last_mixed && (rms <= o.density_tolerance) && (deltaeold <= o.energy_tolerance);
        if (converged) break;
        double deltae = eel - eold, etemp = eel;
        if (valid) {
            // DIIS_Fock_Save: store P, F; e = F P - P F; B row
            if (tid == 0) {
                int mn = ctl[1], newest;
                if (mn < hist) { mn++; newest = ctl[2 + mn - 1]; }
                else { mn = hist; newest = ctl[2]; for (int i = 0; i < hist - 1; i++) ctl[2 + i] = ctl[3 + i]; ctl[2 + hist - 1] = newest; }
                ctl[1] = mn; ctl[20] = newest;
            }
            __syncthreads();
            const int newest = ctl[20], matnum = ctl[1];
            double *hp = wsf + pl.hP + (size_t)newest * hl, *hf = wsf + pl.hF + (size_t)newest * hl, *he = wsf + pl.hE + (size_t)newest * hl;
            // the mixed method keeps its DIIS error vectors in FP32 (in the same slots) and forms the B matrix from
            // FP32 products: the error vectors only steer the extrapolation
            float *hef = (float *)he;
            auto put_error = [&](int idx, double ev) { if (delta_commutator) hef[idx] = (float)ev; else he[idx] = ev; };
            long long t_sub = tm.now();
            for (int i = tid / 32; i < N; i += PDG_WARPS)
                for (int j = tid % 32; j <= i; j += 32) { hp[i * (i + 1) / 2 + j] = P[(size_t)i * N + j]; hf[i * (i + 1) / 2 + j] = F[(size_t)i * N + j]; }
            __syncthreads();
            tm.add(PDG_T_DIIS_PACK, t_sub);
            t_sub = tm.now();
            double emx = 0.0;
            if (have_z || have_pert) {
                // P = 2 Z^T Z (occupied) or 2 (1 - Z^T Z) (virtual) with the vectors Z of the last density step,
                // so with G = Z F:  F P - P F = sg (G^T Z - Z^T G), sg = +2 / -2.  2 N^2 kv FMA instead of N^3.
                // After a perturbative step the new projector is Q = S^T (1 + U) S with S = Z0 + Y (the step's K^T V
                // and U = (1 + K^T K)^-1 - 1), and (1 + U) S = Z0 + W, so with G = S dF and T = Z0 + W:
                // F P - P F = sg (G^T T - T^T G), dF = F - F~: the same two products as after an FP64 step.
                const double *Zc = have_pert ? wsf + pl.BZ : (sm.zs ? sm.zs : wsf + pl.Z);
                const int ldz = sm.ldz, kv = s.n_vec;
                const double sg = s.vec_occupied ? 2.0 : -2.0;
                auto store = [&](int i, int j, double v) {
                    if (j >= i) return;
                    const double ev = sg * v;
                    put_error(i * (i - 1) / 2 + j, ev);
                    emx = fmax(emx, fabs(ev));
                };
                if (delta_commutator) {
                    // mixed method: P commutes with F~ (the matrix it was made from), so F P - P F = dF P - P dF with
                    // dF = F - F~, small once the SCF settles; its products in FP32 carry errors ~1e-7 |dF|.  Every
                    // FP64 step of the mixed method keeps a base, so Z is the base's vectors, also held in FP32.
                    float *G32 = (float *)(wsf + pl.G);
                    float *DF = (float *)(wsf + pl.BW) + pert_dq_offset(N, kv) + (size_t)N * N;
                    const float *Z32 = cur_base().Z32;
                    for (size_t k = tid; k < NN; k += PDG_BLOCK) DF[k] = (float)(F[k] - Ft[k]);
                    __syncthreads();
                    // S = Z0 (+ Y after a perturbative step), T = Z0 (+ W); both kv x N in FP32
                    const float *Yp = (const float *)(wsf + pl.BW) + pert_y_offset(N, kv), *Wp = Yp + (size_t)kv * N;
                    auto Sv = [&](int t, int k) { return have_pert ? Z32[(size_t)t * N + k] + Yp[(size_t)t * N + k] : Z32[(size_t)t * N + k]; };
                    auto Tv = [&](int t, int k) { return have_pert ? Z32[(size_t)t * N + k] + Wp[(size_t)t * N + k] : Z32[(size_t)t * N + k]; };
                    auto fa2 = [&](int i, int k) { return k < kv ? G32[(size_t)k * N + i] : Tv(k - kv, i); };
                    auto fb2 = [&](int j, int k) { return k < kv ? Tv(k, j) : -G32[(size_t)(k - kv) * N + j]; };
                    bool on_tc = false;
#ifndef PDG_SCF_NO_TENSOR
                    const int Kp = (N + 15) & ~15;
                    if (tc_pert && kv <= TC_M && smem_plan(N, kv, a.smem_limit).amat * 8 >= (size_t)3 * (TC_M + Kp) * 64) {
                        // on the tensor cores (the perturbative step's split-BF16 products): G = S dF (kv x N, dF
                        // symmetric), then C = G^T T - T^T G, antisymmetric: its first 128 rows from the tensor cores,
                        // the lower elements of rows >= 128 from their columns there (C(c, r) = -C(r, c)), the corner
                        // of rows and columns >= 128 (N - 128 <= 16) on the FP32 cores
                        on_tc = true;
                        unsigned char *stage = (unsigned char *)sm.amat;
                        if (!tc_product_f32(tc, stage, kv, N, N, Kp, Sv, [&](int i, int k) { return DF[(size_t)i * N + k]; })) {
                            st = PDG_TENSOR_TIMEOUT;
                            break;
                        }
                        tc_readout(tc, Kp, N, [&](int r, int c, float v) { if (r < kv) G32[(size_t)r * N + c] = v; });
                        if (!tc_product_f32(tc, stage, min(N, TC_M), N, 2 * kv, Kp, fa2, fb2)) {
                            st = PDG_TENSOR_TIMEOUT;
                            break;
                        }
                        tc_readout(tc, Kp, N, [&](int r, int c, float v) {
                            if (r >= N) return;
                            if (c < r) store(r, c, (double)v);
                            else if (c >= TC_M && c > r) store(c, r, -(double)v);
                        });
                        for (int e = tid; e < (N - TC_M) * (N - TC_M); e += PDG_BLOCK) {
                            const int i = TC_M + e / (N - TC_M), j = TC_M + e % (N - TC_M);
                            if (j >= i) continue;
                            float acc = 0.0f;
                            for (int k = 0; k < 2 * kv; k++) acc = fmaf(fa2(i, k), fb2(j, k), acc);
                            store(i, j, (double)acc);
                        }
                        __syncthreads();
                    }
#endif
                    if (!on_tc) {
                        tgemm32<false, true>(N, kv, N, [&](int i, int k) { return DF[(size_t)k * N + i]; }, [&](int k, int t) { return Sv(t, k); },
                                     false, sm, [&](int i, int t, double v) { G32[(size_t)t * N + i] = (float)v; });   // G^T = DF S^T
                        tgemm32<false, false>(N, N, 2 * kv, fa2, [&](int k, int j) { return fb2(j, k); }, true, sm, store);
                    }
                } else {
                    double *G = wsf + pl.G;
                    tgemm<true, false>(kv, N, N, [&](int t, int k) { return Zc[(size_t)t * ldz + k]; }, [&](int k, int i) { return F[(size_t)k * N + i]; },
                                       false, sm, [&](int t, int i, double v) { G[(size_t)t * N + i] = v; });
                    tgemm<false, false>(N, N, 2 * kv,
                        [&](int i, int k) { return k < kv ? G[(size_t)k * N + i] : Zc[(size_t)(k - kv) * ldz + i]; },
                        [&](int k, int j) { return k < kv ? Zc[(size_t)k * ldz + j] : -G[(size_t)(k - kv) * N + j]; },
                        true, sm, store);
                }
            } else {
                // full commutator: FP64, or FP32 after a purification step (whose density carries BF16-level
                // errors anyway)
                double *FP = wsf + pl.A;
                const long long t_pur = tm.now();
                if (last_mixed || fp32_start) {
                    // FP32 outer products over k: thread block (i0..i0+3, j0..j0+3) += F[k][i0..] (x) P[k][j0..]
                    // (F symmetric), operands read as float4 rows with no shared-memory staging or barriers
                    const int N4 = (N + 3) & ~3;
                    float *F32 = (float *)(wsf + pl.P0);
                    const float *P32 = (const float *)(wsf + pl.A) + 2 * (((size_t)N * N + 3) & ~size_t(3));
                    for (int e = tid; e < N * N4; e += PDG_BLOCK) {
                        const int i = e / N4, j = e % N4;
                        F32[e] = j < N ? (float)F[(size_t)i * N + j] : 0.0f;
                    }
                    __syncthreads();
                    const int nb4 = N4 / 4;
                    for (int t = tid; t < nb4 * nb4; t += PDG_BLOCK) {
                        const int i0 = (t / nb4) * 4, j0 = (t % nb4) * 4;
                        float acc[4][4] = {};
#pragma unroll 4
                        for (int k = 0; k < N; k++) {
                            const float4 fa = *(const float4 *)(F32 + (size_t)k * N4 + i0);
                            const float4 pb = *(const float4 *)(P32 + (size_t)k * N4 + j0);
                            const float av[4] = { fa.x, fa.y, fa.z, fa.w }, bv[4] = { pb.x, pb.y, pb.z, pb.w };
#pragma unroll
                            for (int x = 0; x < 4; x++)
#pragma unroll
                                for (int y = 0; y < 4; y++) acc[x][y] = fmaf(av[x], bv[y], acc[x][y]);
                        }
                        for (int x = 0; x < 4; x++)
                            for (int y = 0; y < 4; y++)
                                if (i0 + x < N && j0 + y < N) FP[(size_t)(i0 + x) * N + j0 + y] = (double)acc[x][y];
                    }
                    __syncthreads();
                } else
                    tgemm<true, false>(N, N, N, [&](int i, int k) { return F[(size_t)i * N + k]; }, [&](int k, int j) { return P[(size_t)k * N + j]; },
                                       false, sm, [&](int i, int j, double v) { FP[(size_t)i * N + j] = v; });
                for (int i = tid / 32; i < N; i += PDG_WARPS)
                    for (int j = tid % 32; j < i; j += 32) {
                        const double ev = FP[(size_t)i * N + j] - FP[(size_t)j * N + i];
                        put_error(i * (i - 1) / 2 + j, ev);
                        emx = fmax(emx, fabs(ev));
                    }
                __syncthreads();
                tm.add(PDG_T_DIIS_COMMUTATOR_FULL, t_pur);
            }
            double maxerr = block_max(emx, sm.red);
            tm.add(PDG_T_DIIS_COMMUTATOR, t_sub);
            t_sub = tm.now();
            double dots[PDG_MAX_HISTORY];
            for (int m = 0; m < PDG_MAX_HISTORY; m++) dots[m] = 0.0;
            const int ne = N * (N - 1) / 2;
            if (delta_commutator) {
                float d32[PDG_MAX_HISTORY];
                for (int m = 0; m < PDG_MAX_HISTORY; m++) d32[m] = 0.f;
                for (int k = tid; k < ne; k += PDG_BLOCK) {
                    const float en_ = hef[k];
                    for (int m = 0; m < matnum; m++) d32[m] = fmaf(((const float *)(wsf + pl.hE + (size_t)ctl[2 + m] * hl))[k], en_, d32[m]);
                }
                for (int m = 0; m < matnum; m++) dots[m] = (double)d32[m];
            } else {
                for (int k = tid; k < ne; k += PDG_BLOCK) {
                    double en_ = he[k];
                    for (int m = 0; m < matnum; m++) dots[m] += wsf[pl.hE + (size_t)ctl[2 + m] * hl + k] * en_;
                }
            }
            {   // all B-matrix entries in one block reduction (per entry the order of block_sum: lanes, then warps)
                double *rs = sm.ta;
                for (int m = 0; m < matnum; m++) {
                    const double v = warp_sum(dots[m]);
                    if (lane == 0) rs[w * PDG_MAX_HISTORY + m] = v;
                }
                __syncthreads();
                if (tid < matnum) {
                    double t = 0.0;
                    for (int q = 0; q < PDG_WARPS; q++) t += rs[q * PDG_MAX_HISTORY + tid];
                    const double b = 2.0 * t;
                    const int n = ctl[2 + tid];
                    Bm[n * PDG_MAX_HISTORY + newest] = b; Bm[newest * PDG_MAX_HISTORY + n] = b;
                }
            }
            __syncthreads();
            tm.add(PDG_T_DIIS_DOTS, t_sub);
            tm.lap(PDG_T_DIIS_SAVE);
            t_sub = tm.now();
            if (iteration > 0) {
                if (o.use_rca) {
                    if (qdiis && maxerr > 0.8) { qdiis = 0; qrca = 1; }
                    else if (iteration > 1 && qrca && maxerr < o.diis_onset) { qdiis = 1; qrca = 0; }
                }
                if (qdiis) {
                    if (w == 0) {   // DIIS_Iterate: bordered solve, drop the oldest until well conditioned (warp 0)
                        int mn = ctl[1], good = 0;
                        while (mn > 1) {
                            const int n1 = mn + 1;
                            double *x = sm.small + 64;
                            const bool okk = warp_small_solve(n1,
                                [&](int i, int j) { return (i < mn && j < mn) ? Bm[ctl[2 + i] * PDG_MAX_HISTORY + ctl[2 + j]] : ((i == mn && j == mn) ? 0.0 : -1.0); },
                                [&](int i) { return i == mn ? -1.0 : 0.0; }, sm.ta, x);
                            double dev = 0.0;
                            for (int i = 0; i < mn; i++) dev += x[i];
                            dev += -1.0;
                            if (okk && fabs(dev) < 1.0e-6) {
                                if (lane < mn) cf[lane] = x[lane];
                                good = 1;
                                break;
                            }
                            mn--;
                            __syncwarp();
                            if (lane == 0) {
                                for (int i = 0; i < mn; i++) ctl[2 + i] = ctl[3 + i];
                                for (int i = mn; i < hist; i++) { ctl[2 + i] = ctl[2 + i - 1] + 1; if (ctl[2 + i] >= hist) ctl[2 + i] -= hist; }
                            }
                            __syncwarp();
                        }
                        if (lane == 0) { ctl[1] = mn; ctl[21] = good; }
                    }
                    __syncthreads();
                    if (ctl[21]) {
                        const int mn = ctl[1];
                        for (int q = tid; q < hl; q += PDG_BLOCK) {   // packed lower triangle, then mirrored
                            int i = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
                            while ((i + 1) * (i + 2) / 2 <= q) i++;
                            while (i * (i + 1) / 2 > q) i--;
                            const int j = q - i * (i + 1) / 2;
                            double pp = 0.0, ff = 0.0;
                            for (int m = 0; m < mn; m++) {
                                const size_t off = (size_t)ctl[2 + m] * hl + q;
                                pp = fma(cf[m], wsf[pl.hP + off], pp); ff = fma(cf[m], wsf[pl.hF + off], ff);
                            }
                            P[(size_t)i * N + j] = pp; F[(size_t)i * N + j] = ff;
                            P[(size_t)j * N + i] = pp; F[(size_t)j * N + i] = ff;
                        }
                        __syncthreads();
                    }
                    tm.add(PDG_T_ITER_EXTRAPOLATE, t_sub);
                    t_sub = tm.now();
                } else if (o.use_rca && qrca && rca_prev) {
                    // RCA_Iterate: cubic in mu from four traces (DIISSCFConverger.c:661-760)
                    const double *rP = wsf + pl.rP, *rF = wsf + pl.rF;
                    double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
                    for (size_t k = tid; k < NN; k += PDG_BLOCK) { t1 += F[k] * P[k]; t2 += F[k] * rP[k]; t3 += rF[k] * P[k]; t4 += rF[k] * rP[k]; }
                    t1 = block_sum(t1, sm.red); t2 = block_sum(t2, sm.red); t3 = block_sum(t3, sm.red); t4 = block_sum(t4, sm.red);
                    double ca = t1 - t2, cc = t3 - t4, dd = eold;
                    ca += cc + 2.0 * (dd - etemp);
                    double cb = etemp - ca - cc - dd, fmin_ = etemp, mub = 1.0, mu;
                    if (eold < etemp) { fmin_ = eold; mub = 0.0; }
                    if (ca == 0.0) {
                        if (cb == 0.0) mu = mub;
                        else { double mt = -cc / (2.0 * cb); mu = (cb > 0.0 && mt > 0.0 && mt < 1.0) ? mt : mub; }
                    } else {
                        double fac = cb * cb - 3.0 * ca * cc;
                        if (fac >= 0.0) {
                            double m1 = (-cb + sqrt(fac)) / (3.0 * ca), m2 = (-cb - sqrt(fac)) / (3.0 * ca);
                            if (m1 > 0.0 && m1 < 1.0) { double fv = ((ca * m1 + cb) * m1 + cc) * m1 + dd; if (fv < fmin_) { fmin_ = fv; mub = m1; } }
                            if (m2 > 0.0 && m2 < 1.0) { double fv = ((ca * m2 + cb) * m2 + cc) * m2 + dd; if (fv < fmin_) { fmin_ = fv; mub = m2; } }
                        }
                        mu = mub;
                    }
                    mu = fmax(mu, 0.01);
                    double nu = 1.0 - mu;
                    for (size_t k = tid; k < NN; k += PDG_BLOCK) { P[k] = mu * P[k] + nu * rP[k]; F[k] = mu * F[k] + nu * rF[k]; }
                    etemp = ((ca * mu + cb) * mu + cc) * mu + dd;
                    __syncthreads();
                }
            }
            // RCA_Save (DIISSCFConverger.c:231-235) every cycle in ODA mode; in DIIS mode the copies would only serve a
            // switch back to ODA (an error above 0.8 while extrapolating), which then skips one ODA interpolation
            // instead and saves from there
            rca_prev = false;
            if (o.use_rca && !qdiis) {
                double *rP = wsf + pl.rP, *rF = wsf + pl.rF;
                for (size_t k = tid; k < NN; k += PDG_BLOCK) { rP[k] = P[k]; rF[k] = F[k]; }
                __syncthreads();
                rca_prev = true;
            }
            tm.add(PDG_T_ITER_RCA, t_sub);
            iteration++;
            fp32_start = false;
        }
        deltaeold = deltae; eold = etemp;
        __syncthreads();
        tm.lap(PDG_T_ITERATE);
        if (mixed) {
            rms = density_step_mixed(a, wsf, F, P, sm, tm, tc, o.density_step);
            if (rms < 0.0) { st = PDG_TENSOR_TIMEOUT; break; }
            last_mixed = true;
            have_z = false; have_pert = false;
            // leave purification once the density has settled to its accuracy, or when it stalls
            n_mixed++;
            if (rms < o.mixed_switch || n_mixed >= 20) mixed = false;
        } else {
            double r = -1.0;
            if (base_ok) r = density_step_pert(a, wsf, F, P, sm, tm, cur_base(), warm_k, use_shared ? PDG_PERT_KMAX_SHARED : PDG_PERT_KMAX,
                                               tc_pert ? &tc : nullptr);
            if (r == -2.0) { st = PDG_TENSOR_TIMEOUT; break; }   // a tensor-core wait ran out
            warm_k = r >= 0.0;
            if (r >= 0.0) {
                rms = r;
                have_z = false; have_pert = true;
            } else if (use_shared && ncyc == 1 && a.use_density != 1) {
                // the shared base does not carry this frame from its first step: its density is no start either, so
                // the frame starts again as a cold one (the diagonal guess, then the per-frame mixed path)
                const double g = (double)s.n_electrons / (double)N;
                for (size_t k = tid; k < NN; k += PDG_BLOCK) P[k] = ((k / N) == (k % N)) ? g : 0.0;
                if (tid == 0) ctl[1] = 0;
                valid = false; have_z = false; have_pert = false; base_ok = false; use_shared = false;
                mixed = want_mixed; n_mixed = 0; last_mixed = false;
                iteration = 0; qdiis = 0; qrca = o.use_rca ? 1 : 0;
                eold = 0.0; deltaeold = 0.0; rms = 0.0;
                __syncthreads();
                continue;
            } else {
                // FP64 step; in the mixed method it also keeps the base of the following perturbative steps
                rms = density_step(a, wsf, F, P, sm, tm, delta_commutator);
                have_z = true; have_pert = false;
                base_ok = delta_commutator;
                use_shared = false;
            }
            last_mixed = false;
        }
        if (tid == 0 && ncyc <= PDG_RMS_HISTORY) tm.slot[PDG_T_RMS_HISTORY + ncyc - 1] = last_mixed ? -rms : rms;
        valid = true;
    }
    if (converged) st = PDG_OK;
    if (tid == 0) {
        double *E = a.energies + (size_t)f * PDG_NENERGY;
        E[0] = eel; E[1] = e1 + e2; E[2] = en; E[3] = base; E[4] = eq; E[5] = e1; E[6] = e2; E[7] = rms;
        a.status[f] = st;
        if (a.ncycles) a.ncycles[f] = iteration;
        tm.slot[PDG_T_TOTAL] = (double)(clock64() - t_begin);
        unsigned long long gt;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
        tm.slot[PDG_T_END_NS] = (double)gt;
        tm.slot[PDG_T_CYCLES] = (double)ncyc;
    }
}

// ----------------------------------------------------------------------------------------------------
// Spin-unrestricted SCF (UHF, cardinal occupancies; the FP64 method).  Restates the reference's open-shell path:
// QCModelMNDO_Fock with two density sets (QCModelMNDO.c:700-730; MakeFockG with the density of the spin for the
// exchange, MNDOIntegrals.c:51-143), the converger over both sets (DIISSCFConverger.c:385-521: one B matrix summed
// over the sets, the largest error doubled; :530-650 the same coefficients for both; :661-760 ODA traces summed) and
// one density step per spin (QCOnePDM_MakeFromFock, QCOnePDM.c:403, occupancy 1).  A frame's alpha data use the
// workspace slot of the frame (integrals included), its beta data slot n_frames + f; densities alpha then beta.

// F = H + J(Pt) - K(Ps) without the QC/MM term: Coulomb from the total density, exchange from the spin's, the
// one-centre terms split by spin as MakeFockG does (gss, gsp, gpp, gp2, hsp, hpp).
__device__ void fock_build_spin(const SCFArgs &a, const double *H, const double *Pt, const double *Ps, double *F, const double *tei,
                                Smem &sm, double *scratch)
{
    const DeviceSystem &s = a.s;
    const int N = s.n_basis;
    double *pk = s.n_cel <= GK * (GA_LD + GB_LD) ? sm.ta : scratch;
    for (int e = threadIdx.x; e < s.n_cel; e += PDG_BLOCK) {
        const int A = s.cel[e] >> 4, ab = s.cel[e] & 15, as = s.atom_start[A];
        const int m = MP_DA[ab], n = MP_DB[ab];
        pk[e] = (m == n ? 1.0 : 2.0) * Pt[(size_t)(as + m) * N + as + n];
    }
    __syncthreads();
    const int n_out = s.n_cel + s.n_xel;
    for (int e = threadIdx.x; e < n_out; e += PDG_BLOCK) {
        if (e < s.n_cel) {
            const int A = s.cel[e] >> 4, ab = s.cel[e] & 15;
            const int no = s.atom_norb[A], as = s.atom_start[A], na = no * (no + 1) / 2;
            const int m = MP_DA[ab], n = MP_DB[ab];
            double acc = 0.0;
            for (int B = 0; B < s.n_atoms; B++) {
                if (B == A) continue;
                const int hi = A > B ? A : B, lo = A > B ? B : A, pp = hi * (hi - 1) / 2 + lo;
                const int k0 = s.atom_pk[B], nb = s.atom_pk[B + 1] - k0;
                const double *blk = tei + s.pair_tei[pp], *pb = pk + k0;
                if (A > B) for (int cd = 0; cd < nb; cd++) acc = fma(blk[ab * nb + cd], pb[cd], acc);
                else       for (int cd = 0; cd < nb; cd++) acc = fma(blk[cd * na + ab], pb[cd], acc);
            }
            const double *E = elem(s, s.atom_elem[A]);
            const double gss = E[PDG_E_GSS], gsp = E[PDG_E_GSP], gpp = E[PDG_E_GPP], gp2 = E[PDG_E_GP2], hsp = E[PDG_E_HSP], hpp = E[PDG_E_HPP];
            const double *T = Pt + (size_t)as * N + as, *S = Ps + (size_t)as * N + as;
            double g = 0.0;
            if (m == 0 && n == 0) {
                g = (T[0] - S[0]) * gss;
                for (int q = 1; q < no; q++) g += T[q * N + q] * gsp - S[q * N + q] * hsp;
            } else if (m == n) {
                g = T[0] * gsp - S[0] * hsp + (T[m * N + m] - S[m * N + m]) * gpp;
                for (int q = 1; q < no; q++) if (q != m) g += T[q * N + q] * gp2 - S[q * N + q] * hpp;
            } else if (n == 0) g = 2.0 * T[m * N] * hsp - S[m * N] * (hsp + gsp);
            else g = 2.0 * T[m * N + n] * hpp - S[m * N + n] * (hpp + gp2);
            const double v = H[(size_t)(as + m) * N + as + n] + g + acc;
            F[(size_t)(as + m) * N + as + n] = v;
            F[(size_t)(as + n) * N + as + m] = v;
        } else {
            const int x = s.xel[e - s.n_cel], pp = x >> 4, lid = x & 15;
            const int i = s.pair_i[pp], j = s.pair_j[pp];
            const int noi = s.atom_norb[i], noj = s.atom_norb[j], is = s.atom_start[i], js = s.atom_start[j];
            const int nj = noj * (noj + 1) / 2, aa = lid / noj, c = lid % noj;
            const double *blk = tei + s.pair_tei[pp];
            double t = 0.0;
            for (int b = 0; b < noi; b++) {
                const int ab = aa >= b ? aa * (aa + 1) / 2 + b : b * (b + 1) / 2 + aa;
                for (int d = 0; d < noj; d++) {
                    const int cd = c >= d ? c * (c + 1) / 2 + d : d * (d + 1) / 2 + c;
                    t = fma(blk[ab * nj + cd], Ps[(size_t)(is + b) * N + js + d], t);
                }
            }
            const double v = H[(size_t)(is + aa) * N + js + c] - t;
            F[(size_t)(is + aa) * N + js + c] = v;
            F[(size_t)(js + c) * N + is + aa] = v;
        }
    }
    __syncthreads();
}

// tr(X Y) of two symmetric N x N matrices (lower triangle, warp per row).
__device__ double sym_trace(int N, const double *X, const double *Y, Smem &sm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double off = 0.0, dg = 0.0;
    for (int i = w; i < N; i += PDG_WARPS)
        for (int j = lane; j <= i; j += 32) {
            const size_t k = (size_t)i * N + j;
            if (j < i) off = fma(X[k], Y[k], off); else dg = fma(X[k], Y[k], dg);
        }
    const double2 t = block_sum2(off, dg, sm.red);
    return 2.0 * t.x + t.y;
}

// Occupancy weights of density set q from the eigenvalues in sm.eig (every eigenpair, ascending), as
// QCOnePDM_MakeFromFock forms the density (QCOnePDM.c:403-460, occupancies :505-599): cardinal and fixed-fractional
// weights are fixed (occ_ncard full orbitals, then occ_nfrac at occ_frac); variable-fractional ones are Fermi-Dirac
// occupancies at the Fermi energy of the reference's bisection (from [-1000, 1000] Hartree, only the lower bound
// moves, until the electron count is within 1e-12), the orbitals above 1e-10 kept, with the occupancy energy
// sum(p ln p + (1 - p) ln(1 - p)) / beta.  Weights (times occ_factor) go to wt; returns the number of weighted vectors
// (the leading ones); the occupancy energy goes to sm.small[128].
__device__ int occupancy_weights(const SCFArgs &a, int q, Smem &sm, double *wt)
{
    const int N = a.s.n_basis, tid = threadIdx.x, lane = tid & 31;
    const double fac = a.occ_factor;
    if (a.occ_type != PDG_OCC_VARIABLE_FRACTIONAL) {
        const int nc = a.occ_ncard[q], nf = a.occ_nfrac[q];
        const double fr = a.occ_frac[q] * fac;
        for (int k = tid; k < N; k += PDG_BLOCK) wt[k] = k < nc ? fac : (k < nc + nf ? fr : 0.0);
        if (tid == 0) sm.small[128] = 0.0;
        __syncthreads();
        return nc + nf;
    }
    if (tid < 32) {
        const double target = a.occ_charge[q] / fac, beta = a.fermi_beta;
        const double *ev = sm.eig;
        auto fermi = [&](double ef, int k) {
            const double e = -beta * (ef - ev[k]);
            return e > 500.0 ? 0.0 : (e < -500.0 ? 1.0 : 1.0 / (1.0 + exp(e)));
        };
        double ef = 0.0;
        if (target > 0.0) {
            double lo = -1000.0, dx = 2000.0;
            for (int it = 0; it < 500; it++) {
                dx *= 0.5;
                ef = lo + dx;
                double t = 0.0;
                for (int k = lane; k < N; k += 32) t += fermi(ef, k);
                const double fm = warp_sum(t) - target;
                if (fm <= 0.0) lo = ef;
                if (fabs(fm) <= 1.0e-12) break;
            }
        }
        int cnt = 0;
        double e = 0.0;
        for (int k = lane; k < N; k += 32) {
            const double p = target > 0.0 ? fermi(ef, k) : 0.0, r = 1.0 - p;
            wt[k] = p;
            if (p > 1.0e-10) { cnt++; e += p * log(p); if (r > 1.0e-10) e += r * log(r); }
        }
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        e = warp_sum(e);
        for (int k = lane; k < N; k += 32) wt[k] = k < cnt ? wt[k] * fac : 0.0;
        if (lane == 0) { sm.small[128] = e / beta * fac; sm.iv[40] = cnt; }
    }
    __syncthreads();
    return sm.iv[40];
}

// The open-shell and fractional-occupancy SCF of frame f (QCModelMNDO_Fock over the density sets, QCOnePDM_MakeFromFock
// with the sets' occupancies, DIISSCFConverger over the sets): one set (spin-restricted, the total density, occupancy
// factor 2) or two (alpha and beta, factor 1).  The sets' Fock matrices are J(P_total) - K(P_spin) + H (the restricted
// set's with P_spin = P / 2); the electronic energy adds the occupancy energy of the densities in use (zero but for
// variable fractional occupancies).  DIIS B entries and ODA traces are summed over the sets, the largest DIIS error is
// doubled for two sets, both sets are extrapolated or mixed with the same coefficients (DIISSCFConverger.c:385-528,
// 661-760).  The workspace holds two frame slots per frame: slot f has the integrals and set 0's matrices, slot
// n_frames + f set 1's (or the restricted set's P / 2).  Densities: n_sets per frame, N x N each.
__device__ void scf_frame_open(const SCFArgs &a, const int f, double *shm)
{
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, N = s.n_basis;
    const size_t NN = (size_t)N * N;
    const int ns = a.n_sets;
    Smem sm = carve(shm, N, N, a.smem_limit);
    double *wsp[2] = { a.ws + (size_t)f * pl.stride, a.ws + (size_t)(a.n_frames + f) * pl.stride };
    double *H = wsp[0] + pl.H;
    const double *tei = wsp[0] + pl.tei;
    double *Fs[2] = { wsp[0] + pl.F, wsp[1] + pl.F };
    double *Ps[2] = { a.density + (size_t)(ns * f) * NN, a.density + (size_t)(ns * f + ns - 1) * NN };
    double *Pt = wsp[1] + pl.P0;   // the total density (two sets) or half the density (one set)
    const double *Ptot = ns == 2 ? Pt : Ps[0];
    double *Bm = wsp[0] + pl.misc;
    Timer tm;
    tm.slot = wsp[0] + pl.misc + PDG_MAX_HISTORY * PDG_MAX_HISTORY;
    const long long t_begin = clock64();
    if (tid < PDG_NTIMERS) tm.slot[tid] = 0.0;
    __syncthreads();
    tm.start();
    double en = 0.0;
    for (int p = tid; p < s.n_pairs; p += PDG_BLOCK) en += wsp[0][pl.pair_e + (size_t)p * PDG_PAIR_E_STRIDE + 20];
    en = block_sum(en, sm.red);
    double base = 0.0;
    for (int A = tid; A < s.n_atoms; A += PDG_BLOCK) { const double *E = elem(s, s.atom_elem[A]); base += E[PDG_E_EHEAT] - E[PDG_E_EISOL]; }
    base = block_sum(base, sm.red);
    // the density steps compute every eigenpair of each set's matrix (the occupied/virtual boundary then lies
    // inside the vectors the inverse iteration orthogonalises, so a near-degenerate pair across it cannot mix, and
    // fractional occupancies need the orbitals on both sides of it) and weight them with the set's occupancies
    SCFArgs as = a;
    as.s.vec_occupied = 1;
    as.s.n_vec = N;
    bool valid = a.use_density == 1;
    if (a.use_density != 1)
        for (int q = 0; q < ns; q++) {   // uniform diagonal guess per set (QCOnePDM.c:326-331)
            const double g = a.occ_charge[q] / (double)N;
            for (size_t k = tid; k < NN; k += PDG_BLOCK) Ps[q][k] = ((k / N) == (k % N)) ? g : 0.0;
        }
    __syncthreads();
    double eocc[2] = { 0.0, 0.0 };   // occupancy energies of the densities in use (none for a start density)
    const pdg_scf_options &o = a.o;
    const int hist = o.history, hl = pl.hist_len;
    int *ctl = sm.iv;
    double *cf = sm.small + 32;
    if (tid == 0) { ctl[1] = 0; for (int i = 0; i < hist; i++) ctl[2 + i] = i; }
    int iteration = 0, converged = 0, qdiis = 0, qrca = o.use_rca ? 1 : 0, st = PDG_NOT_CONVERGED;
    bool rca_prev = false;
    double eold = 0.0, deltaeold = 0.0, rms = 0.0, eel = 0.0, e1 = 0.0, e2 = 0.0, eq = 0.0;
    const double *phi = a.phi ? a.phi + (size_t)f * s.n_atoms : nullptr;
    __syncthreads();
    while (iteration < o.maximum_scf_cycles && !converged) {
        for (size_t k = tid; k < NN; k += PDG_BLOCK) Pt[k] = ns == 2 ? Ps[0][k] + Ps[1][k] : 0.5 * Ps[0][k];
        __syncthreads();
        e1 = e2 = 0.0;
        for (int q = 0; q < ns; q++) {
            if (ns == 2) fock_build_spin(a, H, Pt, Ps[q], Fs[q], tei, sm, wsp[q] + pl.G);
            else fock_build_spin(a, H, Ps[0], Pt, Fs[0], tei, sm, wsp[0] + pl.G);
            const double th = sym_trace(N, Ps[q], H, sm), tf = sym_trace(N, Ps[q], Fs[q], sm);
            e1 += th;
            e2 += 0.5 * (tf - th);
        }
        // QC/MM: Lowdin charges of the total density, -phi on the diagonal of both spins' matrices
        double tq = 0.0;
        for (int A = tid; A < s.n_atoms; A += PDG_BLOCK) {
            const int no = s.atom_norb[A], as0 = s.atom_start[A];
            double ps = 0.0;
            for (int m = 0; m < no; m++) ps += Ptot[(size_t)(as0 + m) * N + as0 + m];
            const double q = elem(s, s.atom_elem[A])[PDG_E_ZCORE] - ps;
            if (a.charges) a.charges[(size_t)f * s.n_atoms + A] = q;
            if (phi) {
                tq += q * phi[A];
                for (int m = 0; m < no; m++)
                    for (int r = 0; r < ns; r++) Fs[r][(size_t)(as0 + m) * N + as0 + m] -= phi[A];
            }
        }
        eq = block_sum(tq, sm.red);
        tm.lap(PDG_T_FOCK);
        eel = eocc[0] + eocc[1] + e1 + e2 + eq;
        if (!isfinite(eel)) { st = PDG_NAN; break; }
        converged = (iteration > 0) && (rms <= o.density_tolerance) && (deltaeold <= o.energy_tolerance);
        if (converged) break;
        double deltae = eel - eold, etemp = eel;
        if (valid) {
            if (tid == 0) {
                int mn = ctl[1], newest;
                if (mn < hist) { mn++; newest = ctl[2 + mn - 1]; }
                else { mn = hist; newest = ctl[2]; for (int i = 0; i < hist - 1; i++) ctl[2 + i] = ctl[3 + i]; ctl[2 + hist - 1] = newest; }
                ctl[1] = mn; ctl[20] = newest;
            }
            __syncthreads();
            const int newest = ctl[20], matnum = ctl[1];
            double emx = 0.0, dots[PDG_MAX_HISTORY];
            for (int m = 0; m < PDG_MAX_HISTORY; m++) dots[m] = 0.0;
            for (int q = 0; q < ns; q++) {
                double *wq = wsp[q];
                double *hp = wq + pl.hP + (size_t)newest * hl, *hf = wq + pl.hF + (size_t)newest * hl, *he = wq + pl.hE + (size_t)newest * hl;
                for (int i = w; i < N; i += PDG_WARPS)
                    for (int j = lane; j <= i; j += 32) { hp[i * (i + 1) / 2 + j] = Ps[q][(size_t)i * N + j]; hf[i * (i + 1) / 2 + j] = Fs[q][(size_t)i * N + j]; }
                double *FP = wq + pl.A;
                const double *Fq = Fs[q], *Pq = Ps[q];
                tgemm<true, false>(N, N, N, [&](int i, int k) { return Fq[(size_t)i * N + k]; }, [&](int k, int j) { return Pq[(size_t)k * N + j]; },
                                   false, sm, [&](int i, int j, double v) { FP[(size_t)i * N + j] = v; });
                for (int i = w; i < N; i += PDG_WARPS)
                    for (int j = lane; j < i; j += 32) {
                        const double ev = FP[(size_t)i * N + j] - FP[(size_t)j * N + i];
                        he[i * (i - 1) / 2 + j] = ev;
                        emx = fmax(emx, fabs(ev));
                    }
                __syncthreads();
                const int ne = N * (N - 1) / 2;
                for (int k = tid; k < ne; k += PDG_BLOCK) {
                    const double en_ = he[k];
                    for (int m = 0; m < matnum; m++) dots[m] += wq[pl.hE + (size_t)ctl[2 + m] * hl + k] * en_;
                }
            }
            const double maxerr = (ns == 2 ? 2.0 : 1.0) * block_max(emx, sm.red);   // two density sets: the largest error doubled
            {
                double *rs = sm.ta;
                for (int m = 0; m < matnum; m++) {
                    const double v = warp_sum(dots[m]);
                    if (lane == 0) rs[w * PDG_MAX_HISTORY + m] = v;
                }
                __syncthreads();
                if (tid < matnum) {
                    double t = 0.0;
                    for (int q = 0; q < PDG_WARPS; q++) t += rs[q * PDG_MAX_HISTORY + tid];
                    const double b = 2.0 * t;
                    const int n = ctl[2 + tid];
                    Bm[n * PDG_MAX_HISTORY + newest] = b; Bm[newest * PDG_MAX_HISTORY + n] = b;
                }
            }
            __syncthreads();
            tm.lap(PDG_T_DIIS_SAVE);
            if (iteration > 0) {
                if (o.use_rca) {
                    if (qdiis && maxerr > 0.8) { qdiis = 0; qrca = 1; }
                    else if (iteration > 1 && qrca && maxerr < o.diis_onset) { qdiis = 1; qrca = 0; }
                }
                if (qdiis) {
                    if (w == 0) {
                        int mn = ctl[1], good = 0;
                        while (mn > 1) {
                            const int n1 = mn + 1;
                            double *x = sm.small + 64;
                            const bool okk = warp_small_solve(n1,
                                [&](int i, int j) { return (i < mn && j < mn) ? Bm[ctl[2 + i] * PDG_MAX_HISTORY + ctl[2 + j]] : ((i == mn && j == mn) ? 0.0 : -1.0); },
                                [&](int i) { return i == mn ? -1.0 : 0.0; }, sm.ta, x);
                            double dev = 0.0;
                            for (int i = 0; i < mn; i++) dev += x[i];
                            dev += -1.0;
                            if (okk && fabs(dev) < 1.0e-6) {
                                if (lane < mn) cf[lane] = x[lane];
                                good = 1;
                                break;
                            }
                            mn--;
                            __syncwarp();
                            if (lane == 0) {
                                for (int i = 0; i < mn; i++) ctl[2 + i] = ctl[3 + i];
                                for (int i = mn; i < hist; i++) { ctl[2 + i] = ctl[2 + i - 1] + 1; if (ctl[2 + i] >= hist) ctl[2 + i] -= hist; }
                            }
                            __syncwarp();
                        }
                        if (lane == 0) { ctl[1] = mn; ctl[21] = good; }
                    }
                    __syncthreads();
                    if (ctl[21]) {
                        const int mn = ctl[1];
                        for (int q = 0; q < ns; q++)
                            for (int e = tid; e < hl; e += PDG_BLOCK) {
                                int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
                                while ((i + 1) * (i + 2) / 2 <= e) i++;
                                while (i * (i + 1) / 2 > e) i--;
                                const int j = e - i * (i + 1) / 2;
                                double pp = 0.0, ff = 0.0;
                                for (int m = 0; m < mn; m++) {
                                    const size_t off = (size_t)ctl[2 + m] * hl + e;
                                    pp = fma(cf[m], wsp[q][pl.hP + off], pp); ff = fma(cf[m], wsp[q][pl.hF + off], ff);
                                }
                                Ps[q][(size_t)i * N + j] = pp; Fs[q][(size_t)i * N + j] = ff;
                                Ps[q][(size_t)j * N + i] = pp; Fs[q][(size_t)j * N + i] = ff;
                            }
                        __syncthreads();
                    }
                } else if (o.use_rca && qrca && rca_prev) {
                    // RCA_Iterate over the sets: the four traces summed (DIISSCFConverger.c:661-760)
                    double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
                    for (int q = 0; q < ns; q++) {
                        const double *rP = wsp[q] + pl.rP, *rF = wsp[q] + pl.rF;
                        for (size_t k = tid; k < NN; k += PDG_BLOCK) {
                            t1 += Fs[q][k] * Ps[q][k]; t2 += Fs[q][k] * rP[k]; t3 += rF[k] * Ps[q][k]; t4 += rF[k] * rP[k];
                        }
                    }
                    t1 = block_sum(t1, sm.red); t2 = block_sum(t2, sm.red); t3 = block_sum(t3, sm.red); t4 = block_sum(t4, sm.red);
                    double ca = t1 - t2, cc = t3 - t4, dd = eold;
                    ca += cc + 2.0 * (dd - etemp);
                    double cb = etemp - ca - cc - dd, fmin_ = etemp, mub = 1.0, mu;
                    if (eold < etemp) { fmin_ = eold; mub = 0.0; }
                    if (ca == 0.0) {
                        if (cb == 0.0) mu = mub;
                        else { double mt = -cc / (2.0 * cb); mu = (cb > 0.0 && mt > 0.0 && mt < 1.0) ? mt : mub; }
                    } else {
                        double fac = cb * cb - 3.0 * ca * cc;
                        if (fac >= 0.0) {
                            double m1 = (-cb + sqrt(fac)) / (3.0 * ca), m2 = (-cb - sqrt(fac)) / (3.0 * ca);
                            if (m1 > 0.0 && m1 < 1.0) { double fv = ((ca * m1 + cb) * m1 + cc) * m1 + dd; if (fv < fmin_) { fmin_ = fv; mub = m1; } }
                            if (m2 > 0.0 && m2 < 1.0) { double fv = ((ca * m2 + cb) * m2 + cc) * m2 + dd; if (fv < fmin_) { fmin_ = fv; mub = m2; } }
                        }
                        mu = mub;
                    }
                    mu = fmax(mu, 0.01);
                    const double nu = 1.0 - mu;
                    for (int q = 0; q < ns; q++) {
                        const double *rP = wsp[q] + pl.rP, *rF = wsp[q] + pl.rF;
                        for (size_t k = tid; k < NN; k += PDG_BLOCK) { Ps[q][k] = mu * Ps[q][k] + nu * rP[k]; Fs[q][k] = mu * Fs[q][k] + nu * rF[k]; }
                    }
                    etemp = ((ca * mu + cb) * mu + cc) * mu + dd;
                    __syncthreads();
                }
            }
            rca_prev = false;
            if (o.use_rca) {   // RCA_Save every cycle, as the reference does (DIISSCFConverger.c:231-235)
                for (int q = 0; q < ns; q++) {
                    double *rP = wsp[q] + pl.rP, *rF = wsp[q] + pl.rF;
                    for (size_t k = tid; k < NN; k += PDG_BLOCK) { rP[k] = Ps[q][k]; rF[k] = Fs[q][k]; }
                }
                __syncthreads();
                rca_prev = true;
            }
            iteration++;
        }
        deltaeold = deltae; eold = etemp;
        __syncthreads();
        tm.lap(PDG_T_ITERATE);
        // one density step per set, with its occupancies
        rms = 0.0;
        for (int q = 0; q < ns; q++) {
            rms = fmax(rms, density_step<true>(as, wsp[q], Fs[q], Ps[q], sm, tm, false, q));
            eocc[q] = sm.small[128];
            __syncthreads();
        }
        valid = true;
    }
    if (converged) st = PDG_OK;
    if (tid == 0) {
        double *E = a.energies + (size_t)f * PDG_NENERGY;
        E[0] = eel; E[1] = eel - eq; E[2] = en; E[3] = base; E[4] = eq; E[5] = e1; E[6] = e2; E[7] = rms;
        a.status[f] = st;
        if (a.ncycles) a.ncycles[f] = iteration;
        tm.slot[PDG_T_TOTAL] = (double)(clock64() - t_begin);
    }
}

__global__ void __launch_bounds__(PDG_BLOCK, PDG_SCF_CTAS_PER_SM) k_scf_open(SCFArgs a)
{
    extern __shared__ __align__(128) double shm[];
    scf_frame_open(a, blockIdx.x, shm);
}

// Tensor memory (256 columns) and the completion mbarrier of the purification density step, for CTAs that may
// run it.  A CTA of a kernel that contains tcgen05 code holds the tensor-memory allocation permit until it
// allocates and relinquishes it (or exits), and no other such CTA is placed on its SM meanwhile: CTAs that
// will not allocate give it up at once, so that two CTAs share each SM in every mode.
__device__ __forceinline__ void tc_setup(bool ok, TCState &tc, uint32_t *taddr_s, uint64_t *bar_s)
{
    const int w = threadIdx.x >> 5;
    tc.tmem = 0u; tc.bar = 0u; tc.phase = 0u;
#ifdef PDG_SCF_NO_TENSOR
    return;   // no tcgen05 code in this variant: nothing to allocate or relinquish
#endif
    if (!ok) {
        if (w == 0) asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        return;
    }
    if (w == 0) tc_alloc(tc_smem_addr(taddr_s), 256);
    if (threadIdx.x == 0) mbar_init(tc_smem_addr(bar_s), 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tc.tmem = *taddr_s; tc.bar = tc_smem_addr(bar_s);
}

__device__ __forceinline__ void tc_teardown(bool ok, const TCState &tc)
{
#ifdef PDG_SCF_NO_TENSOR
    return;
#endif
    if (!ok) return;
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc_dealloc(tc.tmem, 256);
}

// One CTA per frame of one system.
__global__ void __launch_bounds__(PDG_BLOCK, PDG_SCF_CTAS_PER_SM) k_scf(SCFArgs a)
{
    extern __shared__ __align__(128) double shm[];
    __shared__ uint32_t tc_taddr_s;
    __shared__ __align__(8) uint64_t tc_bar_s;
    const int N = a.s.n_basis;
    const bool tc_ok = a.fock_only != 1 && a.o.density_step != 0 && N <= 144 && smem_plan(N, a.s.n_vec, a.smem_limit).amat != 0;
    TCState tc;
    tc_setup(tc_ok, tc, &tc_taddr_s, &tc_bar_s);
    scf_frame(a, blockIdx.x, shm, tc, tc_ok);
    tc_teardown(tc_ok, tc);
}

// Persistent SCF over a heterogeneous batch: each CTA takes the next item of `order` (largest first) from the
// queue counter until the batch is exhausted; the tensor memory is allocated once per CTA when any item may
// use the purification step.  Items are independent; the only shared state is the counter (zero at launch).
__global__ void __launch_bounds__(PDG_BLOCK, PDG_SCF_CTAS_PER_SM)
k_scf_batch(SCFArgs a, Batch b, const int *__restrict__ order, int *__restrict__ queue, int tensor_items)
{
    extern __shared__ __align__(128) double shm[];
    __shared__ uint32_t tc_taddr_s;
    __shared__ __align__(8) uint64_t tc_bar_s;
    __shared__ SCFArgs ia;
    __shared__ int next;
    const bool tc_any = tensor_items != 0 && a.o.density_step != 0;
    TCState tc;
    tc_setup(tc_any, tc, &tc_taddr_s, &tc_bar_s);
    for (int round = 0; round < b.n; round++) {
        if (threadIdx.x == 0) next = atomicAdd(queue, 1);
        __syncthreads();
        const int q = next;
        if (q >= b.n) break;
        if (threadIdx.x == 0) {
            const int k = order[q];
            const BatchItem &it = b.items[k];
            ia = a;
            ia.s = it.s; ia.plan = it.plan; ia.n_frames = 1;
            ia.ws = a.ws + it.ws; ia.density = a.density + it.dens;
            ia.phi = a.phi ? a.phi + it.atom : nullptr;
            ia.charges = a.charges ? a.charges + it.atom : nullptr;
            ia.energies = a.energies + (size_t)k * PDG_NENERGY;
            ia.status = a.status + k;
            ia.ncycles = a.ncycles ? a.ncycles + k : nullptr;
        }
        __syncthreads();
        const int N = ia.s.n_basis;
        const bool ok = tc_any && N <= 144 && smem_plan(N, ia.s.n_vec, a.smem_limit).amat != 0;
        scf_frame(ia, 0, shm, tc, ok);
        __syncthreads();
    }
    tc_teardown(tc_any, tc);
}

size_t scf_smem_bytes(int N, int kv) { return smem_plan(N, kv, PDG_SMEM_LIMIT).bytes; }
size_t scf_smem_bytes_limit(int N, int kv, int limit_bytes) { return smem_plan(N, kv, limit_bytes).bytes; }

int scf_occupancy(const DeviceSystem &s, int *threads, int *smem_bytes, int *ctas_per_sm)
{
    const size_t sm = scf_smem_bytes(s.n_basis, s.n_vec);
    if (sm > 48 * 1024) {
        cudaFuncSetAttribute(k_scf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaFuncSetAttribute(k_scf, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    }
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_scf, PDG_BLOCK, sm);
    *threads = PDG_BLOCK; *smem_bytes = (int)sm; *ctas_per_sm = n;
    return e == cudaSuccess ? 0 : 1;
}

void launch_scf(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *phi, const pdg_scf_options &o,
                double *density, int use_density, double *energies, double *charges, int *status, int *ncycles,
                double *ws, int fock_only, double *fock_out, cudaStream_t st, const double *base)
{
    SCFArgs a;
    a.s = s; a.plan = p; a.n_frames = n_frames; a.phi = phi; a.o = o; a.density = density; a.use_density = use_density;
    a.energies = energies; a.charges = charges; a.status = status; a.ncycles = ncycles; a.ws = ws;
    a.fock_only = fock_only; a.fock_out = fock_out;
    a.smem_limit = PDG_SMEM_LIMIT;
    a.base = fock_only ? nullptr : base;
    size_t sm = scf_smem_bytes(s.n_basis, s.n_vec);
    static size_t configured = 0;
    if (sm > 48 * 1024 && sm > configured) {
        cudaFuncSetAttribute(k_scf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        // two SCF CTAs per SM need the largest shared-memory carveout
        cudaFuncSetAttribute(k_scf, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
        configured = sm;
    }
    k_scf<<<n_frames, PDG_BLOCK, sm, st>>>(a);
}

__global__ void k_uhf_densities(long long n, size_t NN, const double *__restrict__ P, double *__restrict__ out)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const long long f = g / (long long)NN, k = g % (long long)NN;
    const double a = P[(2 * f) * NN + k], b = P[(2 * f + 1) * NN + k];
    out[g] = a + b;       // total densities, n_frames x N x N
    out[n + g] = a - b;   // spin densities after them
}

void launch_uhf_densities(int n_frames, int N, const double *P, double *out, cudaStream_t st)
{
    const long long n = (long long)n_frames * N * N;
    k_uhf_densities<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, (size_t)N * N, P, out);
}

void launch_scf_open(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *phi, const pdg_scf_options &o,
                     const OpenOccupancy &oc, double *density, int use_density, double *energies, double *charges, int *status,
                     int *ncycles, double *ws, cudaStream_t st)
{
    SCFArgs a = {};
    a.s = s; a.plan = p; a.n_frames = n_frames; a.phi = phi; a.o = o; a.density = density; a.use_density = use_density;
    a.energies = energies; a.charges = charges; a.status = status; a.ncycles = ncycles; a.ws = ws;
    a.fock_only = 0; a.fock_out = nullptr; a.smem_limit = PDG_SMEM_LIMIT; a.base = nullptr;
    a.n_sets = oc.n_sets; a.occ_type = oc.type; a.occ_factor = oc.factor; a.fermi_beta = oc.beta;
    for (int q = 0; q < 2; q++) {
        a.occ_charge[q] = oc.charge[q]; a.occ_ncard[q] = oc.ncard[q]; a.occ_nfrac[q] = oc.nfrac[q]; a.occ_frac[q] = oc.frac[q];
    }
    const int N = s.n_basis;
    const size_t sm = scf_smem_bytes(N, N);   // every eigenpair (scf_frame_open)
    if (sm > 48 * 1024) {
        cudaFuncSetAttribute(k_scf_open, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaFuncSetAttribute(k_scf_open, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    }
    k_scf_open<<<n_frames, PDG_BLOCK, sm, st>>>(a);
}

void launch_batch_scf(const Batch &b, const int *order, int *queue, int grid, int smem_limit, size_t smem_bytes, int tensor_items,
                      const double *phi, const pdg_scf_options &o, double *density, int use_density, double *energies,
                      double *charges, int *status, int *ncycles, double *ws, cudaStream_t st)
{
    SCFArgs a = {};
    a.n_frames = b.n; a.phi = phi; a.o = o; a.density = density; a.use_density = use_density;
    a.energies = energies; a.charges = charges; a.status = status; a.ncycles = ncycles; a.ws = ws;
    a.fock_only = 0; a.fock_out = nullptr; a.smem_limit = smem_limit;
    k_scf_batch<<<grid, PDG_BLOCK, smem_bytes, st>>>(a, b, order, queue, tensor_items);
}

// Launch attributes of the batch SCF kernel for a dynamic shared-memory size (outside any stream capture).
int configure_batch_scf(size_t smem_bytes)
{
    if (cudaFuncSetAttribute(k_scf_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes) != cudaSuccess) return 1;
    if (cudaFuncSetAttribute(k_scf_batch, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return 1;
    return 0;
}

}   // namespace PDG_SCF_NS
