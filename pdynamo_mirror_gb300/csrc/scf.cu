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

#define TILE 64
#define KCH 16

struct SCFArgs {
    DeviceSystem s; FramePlan plan; int n_frames;
    const double *phi; pdg_scf_options o;
    double *density; int use_density;
    double *energies, *charges; int *status, *ncycles;
    double *ws; int fock_only; double *fock_out;
};

// Shared scratch layout (doubles): red[32] | gemm tiles 2*TILE*KCH | small[256] | d,e,e2,tau,eig (5N) | v,p (2N)
struct Smem {
    double *red, *ta, *tb, *small, *d, *e, *e2, *tau, *eig, *v, *p;
    int *iv;   // ints: [0..63] control, [64..] cluster starts
};

__device__ __forceinline__ Smem carve(double *base, int N)
{
    Smem m;
    m.red = base; m.ta = base + 32; m.tb = m.ta + TILE * KCH; m.small = m.tb + TILE * KCH;
    m.d = m.small + 256; m.e = m.d + N; m.e2 = m.e + N; m.tau = m.e2 + N; m.eig = m.tau + N; m.v = m.eig + N; m.p = m.v + N;
    m.iv = (int *)(m.p + N);
    return m;
}

// C = A * B over M x Nc outputs with inner dimension K; element accessors are strided.  Each thread owns
// a 2 x 4 register tile of a TILE x TILE output tile.  lower_only skips tiles strictly above the diagonal.
// The epilogue receives (i, j, value).
template <typename Epi>
__device__ void block_gemm(int M, int Nc, int K, const double *A, int a_r, int a_c, const double *B, int b_r, int b_c,
                           bool lower_only, Smem &sm, Epi epi)
{
    const int tid = threadIdx.x;
    const int tr = tid / 16, tc = tid % 16;   // 32 x 16 threads -> rows tr*2 + {0,1}, cols tc*4 + {0..3}
    for (int i0 = 0; i0 < M; i0 += TILE)
        for (int j0 = 0; j0 < Nc; j0 += TILE) {
            if (lower_only && j0 > i0 + TILE - 1) continue;
            double acc[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
            for (int k0 = 0; k0 < K; k0 += KCH) {
                __syncthreads();
                for (int t = tid; t < TILE * KCH; t += PDG_BLOCK) {
                    int r = t / KCH, kk = t % KCH, gi = i0 + r, gk = k0 + kk;
                    sm.ta[kk * TILE + r] = (gi < M && gk < K) ? A[(size_t)gi * a_r + (size_t)gk * a_c] : 0.0;
                    int c = t % TILE, kb = t / TILE, gj = j0 + c, gk2 = k0 + kb;
                    sm.tb[kb * TILE + c] = (gj < Nc && gk2 < K) ? B[(size_t)gk2 * b_r + (size_t)gj * b_c] : 0.0;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < KCH; kk++) {
                    double a0 = sm.ta[kk * TILE + tr * 2], a1 = sm.ta[kk * TILE + tr * 2 + 1];
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        double b = sm.tb[kk * TILE + tc * 4 + c];
                        acc[0][c] = fma(a0, b, acc[0][c]);
                        acc[1][c] = fma(a1, b, acc[1][c]);
                    }
                }
            }
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 4; c++) {
                    int gi = i0 + tr * 2 + r, gj = j0 + tc * 4 + c;
                    if (gi < M && gj < Nc) epi(gi, gj, acc[r][c]);
                }
        }
    __syncthreads();
}

// ----------------------------------------------------------------------------------------------------
// F = H + G(P) and the energies tr(PH), tr(PG)/2; then the QC/MM Lowdin term.  Returns eqcmm.
__device__ void fock_build(const SCFArgs &a, int f, const double *H, const double *P, double *F, const double *tei,
                           Smem &sm, double *e1, double *e2, double *eqcmm)
{
    const DeviceSystem &s = a.s;
    const int N = s.n_basis, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // diagonal blocks: one-centre G plus Coulomb from every partner atom
    for (int A = w; A < s.n_atoms; A += PDG_WARPS) {
        int no = s.atom_norb[A], as = s.atom_start[A], na = no * (no + 1) / 2;
        double acc[10];
        for (int k = 0; k < 10; k++) acc[k] = 0.0;
        for (int B = lane; B < s.n_atoms; B += 32) {
            if (B == A) continue;
            int hi = A > B ? A : B, lo = A > B ? B : A;
            int p = hi * (hi - 1) / 2 + lo;
            int nob = s.atom_norb[B], bs = s.atom_start[B], nb = nob * (nob + 1) / 2;
            double pb[10];
            for (int cd = 0; cd < nb; cd++) {
                int c = cd == 0 ? 0 : (cd < 3 ? 1 : (cd < 6 ? 2 : 3)), dd = cd - c * (c + 1) / 2;
                pb[cd] = (c == dd ? 1.0 : 2.0) * P[(size_t)(bs + c) * N + bs + dd];
            }
            const double *blk = tei + s.pair_tei[p];
            if (A > B) {   // A holds the rows of the block
                for (int ab = 0; ab < na; ab++) {
                    double t = 0.0;
                    for (int cd = 0; cd < nb; cd++) t += blk[ab * nb + cd] * pb[cd];
                    acc[ab] += t;
                }
            } else {
                for (int cd = 0; cd < na; cd++) {
                    double t = 0.0;
                    for (int ab = 0; ab < nb; ab++) t += blk[ab * na + cd] * pb[ab];
                    acc[cd] += t;
                }
            }
        }
        for (int k = 0; k < na; k++) acc[k] = warp_sum(acc[k]);
        if (lane < no * no) {
            int m = lane / no, n = lane % no;
            const double *E = elem(s, s.atom_elem[A]);
            double gss = E[PDG_E_GSS], gsp = E[PDG_E_GSP], gpp = E[PDG_E_GPP], gp2 = E[PDG_E_GP2], hsp = E[PDG_E_HSP], hpp = E[PDG_E_HPP];
            const double *PA = P + (size_t)as * N + as;
            double g = 0.0;
            if (no == 1) g = 0.5 * PA[0] * gss;
            else if (m == 0 && n == 0) { g = 0.5 * PA[0] * gss; for (int q = 1; q < 4; q++) g += PA[q * N + q] * (gsp - 0.5 * hsp); }
            else if (m == n) {
                g = PA[0] * (gsp - 0.5 * hsp) + 0.5 * PA[m * N + m] * gpp;
                for (int q = 1; q < 4; q++) if (q != m) g += PA[q * N + q] * (gp2 - 0.5 * hpp);
            } else if (m == 0 || n == 0) g = PA[m * N + n] * (1.5 * hsp - 0.5 * gsp);
            else g = PA[m * N + n] * (1.5 * hpp - 0.5 * gp2);
            int idx = (m >= n) ? m * (m + 1) / 2 + n : n * (n + 1) / 2 + m;
            F[(size_t)(as + m) * N + as + n] = H[(size_t)(as + m) * N + as + n] + g + acc[idx];
        }
    }
    // off-diagonal blocks: exchange, F_ac = H_ac - 1/2 sum_bd (ab|cd) P_bd
    for (int p = w; p < s.n_pairs; p += PDG_WARPS) {
        int i = s.pair_i[p], j = s.pair_j[p];
        int noi = s.atom_norb[i], noj = s.atom_norb[j], is = s.atom_start[i], js = s.atom_start[j];
        int nj = noj * (noj + 1) / 2;
        const double *blk = tei + s.pair_tei[p];
        if (lane < noi * noj) {
            int aa = lane / noj, c = lane % noj;
            double t = 0.0;
            for (int b = 0; b < noi; b++) {
                int ab = aa >= b ? aa * (aa + 1) / 2 + b : b * (b + 1) / 2 + aa;
                for (int d = 0; d < noj; d++) {
                    int cd = c >= d ? c * (c + 1) / 2 + d : d * (d + 1) / 2 + c;
                    t += blk[ab * nj + cd] * P[(size_t)(is + b) * N + js + d];
                }
            }
            double v = H[(size_t)(is + aa) * N + js + c] - 0.5 * t;
            F[(size_t)(is + aa) * N + js + c] = v;
            F[(size_t)(js + c) * N + is + aa] = v;
        }
    }
    __syncthreads();
    double t1 = 0.0, t2 = 0.0;
    for (size_t k = threadIdx.x; k < (size_t)N * N; k += PDG_BLOCK) { double pv = P[k], hv = H[k]; t1 += pv * hv; t2 += pv * (F[k] - hv); }
    *e1 = block_sum(t1, sm.red);
    *e2 = 0.5 * block_sum(t2, sm.red);
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
// Small dense solve by thread 0 (partial pivoting); rejects a reciprocal 1-norm condition below 1e-15
// (SymmetricMatrix_SolveLinearEquations' test, SymmetricMatrix.c:1412-1450).
__device__ bool small_solve(int n, double *A, double *b)
{
    double M[17][17], Inv[17][17], x[17], anorm = 0.0;
    for (int j = 0; j < n; j++) { double t = 0.0; for (int i = 0; i < n; i++) t += fabs(A[i * n + j]); anorm = fmax(anorm, t); }
    for (int i = 0; i < n; i++) { x[i] = b[i]; for (int j = 0; j < n; j++) { M[i][j] = A[i * n + j]; Inv[i][j] = (i == j); } }
    for (int k = 0; k < n; k++) {
        int pv = k;
        for (int i = k + 1; i < n; i++) if (fabs(M[i][k]) > fabs(M[pv][k])) pv = i;
        if (M[pv][k] == 0.0) return false;
        if (pv != k) {
            for (int j = 0; j < n; j++) { double t = M[k][j]; M[k][j] = M[pv][j]; M[pv][j] = t; t = Inv[k][j]; Inv[k][j] = Inv[pv][j]; Inv[pv][j] = t; }
            double t = x[k]; x[k] = x[pv]; x[pv] = t;
        }
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            double fct = M[i][k] / M[k][k];
            if (fct == 0.0) continue;
            for (int j = 0; j < n; j++) { M[i][j] -= fct * M[k][j]; Inv[i][j] -= fct * Inv[k][j]; }
            x[i] -= fct * x[k];
        }
    }
    double inorm = 0.0;
    for (int j = 0; j < n; j++) { double t = 0.0; for (int i = 0; i < n; i++) t += fabs(Inv[i][j] / M[i][i]); inorm = fmax(inorm, t); }
    for (int i = 0; i < n; i++) b[i] = x[i] / M[i][i];
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

__device__ int sturm_count(int N, const double *d, const double *e2, double x, double pivmin)
{
    int c = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) c++;
    for (int i = 1; i < N; i++) {
        q = d[i] - x - e2[i - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0.0) c++;
    }
    return c;
}

// Phase timers: thread 0 accumulates clock64() deltas between block-wide barriers into the frame's
// timer slots (workspace misc area, after the DIIS B matrix).
struct Timer {
    double *slot; long long t;
    __device__ void start() { if (threadIdx.x == 0) t = clock64(); }
    __device__ void lap(int k) { if (threadIdx.x == 0) { long long n = clock64(); slot[k] += (double)(n - t); t = n; } }
};

__device__ double density_step(const SCFArgs &a, double *wsf, const double *F, double *P, Smem &sm, Timer &tm)
{
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int N = s.n_basis, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int kv = s.n_vec;
    double *A = wsf + pl.A, *HV = wsf + pl.HV, *Z = wsf + pl.Z;
    for (size_t k = tid; k < (size_t)N * N; k += PDG_BLOCK) A[k] = F[k];
    __syncthreads();
    // --- Householder tridiagonalisation A = Q T Q^T (lower, dsytd2-style; the full square is updated so
    //     every access is a contiguous row).
    for (int k = 0; k + 2 < N; k++) {
        int m = N - k - 1;
        const double *row = A + (size_t)k * N + k + 1;
        double part = 0.0;
        for (int i = 1 + tid; i < m; i += PDG_BLOCK) part += row[i] * row[i];
        double xn2 = block_sum(part, sm.red);
        double alpha = row[0];
        if (tid == 0) sm.d[k] = A[(size_t)k * N + k];
        if (xn2 == 0.0) {
            if (tid == 0) { sm.e[k] = alpha; sm.tau[k] = 0.0; }
            __syncthreads();
            continue;
        }
        double beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        double tau = (beta - alpha) / beta, scal = 1.0 / (alpha - beta);
        for (int i = tid; i < m; i += PDG_BLOCK) {
            double vi = (i == 0) ? 1.0 : row[i] * scal;
            sm.v[i] = vi;
            HV[(size_t)k * N + i] = vi;
        }
        if (tid == 0) { sm.e[k] = beta; sm.tau[k] = tau; }
        __syncthreads();
        // p = tau A22 v (warp per row)
        for (int i = w; i < m; i += PDG_WARPS) {
            const double *ar = A + (size_t)(k + 1 + i) * N + k + 1;
            double t = 0.0;
            for (int j = lane; j < m; j += 32) t += ar[j] * sm.v[j];
            t = warp_sum(t);
            if (lane == 0) sm.p[i] = tau * t;
        }
        __syncthreads();
        double pv = 0.0;
        for (int i = tid; i < m; i += PDG_BLOCK) pv += sm.p[i] * sm.v[i];
        double K = 0.5 * tau * block_sum(pv, sm.red);
        for (int i = tid; i < m; i += PDG_BLOCK) sm.p[i] -= K * sm.v[i];   // p <- w
        __syncthreads();
        for (int t = tid; t < m * m; t += PDG_BLOCK) {
            int i = t / m, j = t % m;
            A[(size_t)(k + 1 + i) * N + k + 1 + j] -= sm.v[i] * sm.p[j] + sm.p[i] * sm.v[j];
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (N >= 2) { sm.d[N - 2] = A[(size_t)(N - 2) * N + N - 2]; sm.e[N - 2] = A[(size_t)(N - 2) * N + N - 1]; sm.tau[N - 2] = 0.0; }
        sm.d[N - 1] = A[(size_t)(N - 1) * N + N - 1];
        sm.e[N - 1] = 0.0;
    }
    __syncthreads();
    tm.lap(PDG_T_TRIDIAGONAL);
    // --- eigenvalues by bisection, one thread per wanted index (ascending)
    double gl = 1e300, gu = -1e300, emax2 = 0.0;
    for (int i = tid; i < N; i += PDG_BLOCK) {
        double r = (i > 0 ? fabs(sm.e[i - 1]) : 0.0) + (i < N - 1 ? fabs(sm.e[i]) : 0.0);
        gl = fmin(gl, sm.d[i] - r); gu = fmax(gu, sm.d[i] + r);
        if (i < N - 1) { sm.e2[i] = sm.e[i] * sm.e[i]; emax2 = fmax(emax2, sm.e2[i]); }
    }
    gl = -block_max(-gl, sm.red); gu = block_max(gu, sm.red); emax2 = block_max(emax2, sm.red);
    double tnorm = fmax(fabs(gl), fabs(gu));
    double pivmin = 1.0e-290 * fmax(1.0, emax2);
    gl -= 2.2e-16 * tnorm * 4.0 * N + pivmin; gu += 2.2e-16 * tnorm * 4.0 * N + pivmin;
    int first = s.vec_occupied ? 0 : N - kv;
    for (int t = tid; t < kv; t += PDG_BLOCK) {
        int m = first + t;
        double lo = gl, hi = gu;
        for (int it = 0; it < 200; it++) {
            double mid = 0.5 * (lo + hi);
            if (hi - lo <= 2.2e-16 * fmax(fabs(lo), fabs(hi)) + 4.0 * pivmin || mid == lo || mid == hi) break;
            if (sturm_count(N, sm.d, sm.e2, mid, pivmin) <= m) lo = mid; else hi = mid;
        }
        sm.eig[t] = 0.5 * (lo + hi);
    }
    __syncthreads();
    tm.lap(PDG_T_EIGENVALUES);
    // --- clusters (dstein-style): gaps below ortol share re-orthogonalisation; equal values are split
    if (tid == 0) {
        double onenrm = 0.0;
        for (int i = 0; i < N; i++) onenrm = fmax(onenrm, fabs(sm.d[i]) + (i > 0 ? fabs(sm.e[i - 1]) : 0.0) + (i < N - 1 ? fabs(sm.e[i]) : 0.0));
        double ortol = 1.0e-5 * fmax(onenrm, 1.0);
        int nc = 0;
        sm.iv[64] = 0;
        for (int t = 1; t < kv; t++) {
            double pert = 10.0 * fabs(2.2e-16 * sm.eig[t]) + 1e-300;
            if (sm.eig[t] - sm.eig[t - 1] < pert) sm.eig[t] = sm.eig[t - 1] + pert;
            if (sm.eig[t] - sm.eig[t - 1] > ortol) sm.iv[64 + (++nc)] = t;
        }
        sm.iv[64 + (++nc)] = kv;
        sm.iv[0] = nc;
        sm.small[0] = onenrm;
    }
    __syncthreads();
    const int nclusters = sm.iv[0];
    const double tiny = 2.2e-16 * fmax(sm.small[0], 1.0);
    // --- inverse iteration: one warp per cluster, members in order, 3 iterations each
    double *lu = wsf + pl.LU + (size_t)w * 8 * N;
    double *u0 = lu, *u1 = lu + N, *u2 = lu + 2 * N, *lm = lu + 3 * N, *pv = lu + 4 * N, *x = lu + 5 * N;
    for (int c = w; c < nclusters; c += PDG_WARPS) {
        int c0 = sm.iv[64 + c], c1 = sm.iv[64 + c + 1];
        for (int t = c0; t < c1; t++) {
            double sigma = sm.eig[t];
            if (lane == 0) {   // T - sigma I = P L U, partial pivoting (U has two super-diagonals)
                double ak = sm.d[0] - sigma, bk = N > 1 ? sm.e[0] : 0.0;
                for (int k = 0; k < N - 1; k++) {
                    double ck = sm.e[k], an = sm.d[k + 1] - sigma, bn = (k + 1 < N - 1) ? sm.e[k + 1] : 0.0;
                    if (fabs(ak) >= fabs(ck)) {
                        if (ak == 0.0) ak = tiny;
                        double l = ck / ak;
                        u0[k] = ak; u1[k] = bk; u2[k] = 0.0; lm[k] = l; pv[k] = 0.0;
                        ak = an - l * bk; bk = bn;
                    } else {
                        double l = ak / ck;
                        u0[k] = ck; u1[k] = an; u2[k] = bn; lm[k] = l; pv[k] = 1.0;
                        ak = bk - l * an; bk = -l * bn;
                    }
                }
                u0[N - 1] = (ak == 0.0) ? tiny : ak;
                for (int k = 0; k < N; k++) { if (fabs(u0[k]) < tiny) u0[k] = copysign(tiny, u0[k]); u0[k] = 1.0 / u0[k]; }
            }
            for (int i = lane; i < N; i += 32) x[i] = ((hash2(t * 2654435761u + 17u, i) >> 8) * (1.0 / 16777216.0)) * 2.0 - 1.0;
            __syncwarp();
            for (int it = 0; it < 3; it++) {
                if (lane == 0) {
                    for (int k = 0; k < N - 1; k++) {
                        if (pv[k] != 0.0) { double tt = x[k]; x[k] = x[k + 1]; x[k + 1] = tt; }
                        x[k + 1] -= lm[k] * x[k];
                    }
                    x[N - 1] *= u0[N - 1];
                    if (N > 1) x[N - 2] = (x[N - 2] - u1[N - 2] * x[N - 1]) * u0[N - 2];
                    for (int k = N - 3; k >= 0; k--) x[k] = (x[k] - u1[k] * x[k + 1] - u2[k] * x[k + 2]) * u0[k];
                }
                __syncwarp();
                for (int q = c0; q < t; q++) {   // re-orthogonalise against earlier cluster members
                    const double *zq = Z + (size_t)q * N;
                    double dt = 0.0;
                    for (int i = lane; i < N; i += 32) dt += x[i] * zq[i];
                    dt = warp_sum(dt);
                    for (int i = lane; i < N; i += 32) x[i] -= dt * zq[i];
                    __syncwarp();
                }
                double nr = 0.0;
                for (int i = lane; i < N; i += 32) nr += x[i] * x[i];
                nr = warp_sum(nr);
                double sc = 1.0 / sqrt(nr);
                for (int i = lane; i < N; i += 32) x[i] *= sc;
                __syncwarp();
            }
            double *zt = Z + (size_t)t * N;
            for (int i = lane; i < N; i += 32) zt[i] = x[i];
            __syncwarp();
        }
    }
    __syncthreads();
    tm.lap(PDG_T_EIGENVECTORS);
    // --- back-transformation z <- Q z (reflectors applied last to first), one warp per vector
    for (int t = w; t < kv; t += PDG_WARPS) {
        double *zt = Z + (size_t)t * N;
        for (int k = N - 3; k >= 0; k--) {
            double tau = sm.tau[k];
            if (tau == 0.0) continue;
            int m = N - k - 1;
            const double *hv = HV + (size_t)k * N;
            double dt = 0.0;
            for (int i = lane; i < m; i += 32) dt += hv[i] * zt[k + 1 + i];
            dt = warp_sum(dt) * tau;
            for (int i = lane; i < m; i += 32) zt[k + 1 + i] -= dt * hv[i];
            __syncwarp();
        }
    }
    __syncthreads();
    tm.lap(PDG_T_BACKTRANSFORM);
    // --- P = 2 Z^T Z (occupied) or 2 (1 - Z^T Z) (virtual); lower triangle then mirrored
    const bool occ = s.vec_occupied;
    double rms = 0.0;
    block_gemm(N, N, kv, Z, 1, N, Z, N, 1, true, sm, [&](int i, int j, double v) {
        if (j > i) return;
        double pn = occ ? 2.0 * v : ((i == j ? 2.0 : 0.0) - 2.0 * v);
        double dlt = pn - P[(size_t)i * N + j];
        rms += (i == j) ? dlt * dlt : 2.0 * dlt * dlt;
        P[(size_t)i * N + j] = pn;
        if (i != j) P[(size_t)j * N + i] = pn;
    });
    double out = sqrt(block_sum(rms, sm.red)) / (double)N;
    tm.lap(PDG_T_DENSITY);
    return out;
}

// ----------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(PDG_BLOCK, 1) k_scf(SCFArgs a)
{
    extern __shared__ double shm[];
    const DeviceSystem &s = a.s;
    const FramePlan &pl = a.plan;
    const int f = blockIdx.x, tid = threadIdx.x, N = s.n_basis;
    const size_t NN = (size_t)N * N;
    Smem sm = carve(shm, N);
    double *wsf = a.ws + (size_t)f * pl.stride;
    double *H = wsf + pl.H, *F = wsf + pl.F, *P = a.density + (size_t)f * NN;
    const double *tei = wsf + pl.tei;
    double *Bm = wsf + pl.misc;   // DIIS B matrix, PDG_MAX_HISTORY^2
    Timer tm;
    tm.slot = wsf + pl.misc + PDG_MAX_HISTORY * PDG_MAX_HISTORY;
    long long t_begin = clock64();
    if (tid < PDG_NTIMERS) tm.slot[tid] = 0.0;
    __syncthreads();
    tm.start();
    // nuclear energy: sum of the pair terms in pair order
    double en = 0.0;
    for (int p = tid; p < s.n_pairs; p += PDG_BLOCK) en += wsf[pl.pair_e + (size_t)p * PDG_PAIR_E_STRIDE + 20];
    en = block_sum(en, sm.red);
    double base = 0.0;
    for (int A = tid; A < s.n_atoms; A += PDG_BLOCK) { const double *E = elem(s, s.atom_elem[A]); base += E[PDG_E_EHEAT] - E[PDG_E_EISOL]; }
    base = block_sum(base, sm.red);
    bool valid = a.use_density != 0;
    if (!valid) {   // uniform diagonal guess (QCOnePDM.c:326-331)
        double g = (double)s.n_electrons / (double)N;
        for (size_t k = tid; k < NN; k += PDG_BLOCK) P[k] = ((k / N) == (k % N)) ? g : 0.0;
    }
    __syncthreads();
    double e1, e2, eq;
    if (a.fock_only) {
        fock_build(a, f, H, P, F, tei, sm, &e1, &e2, &eq);
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
    double eold = 0.0, deltaeold = 0.0, rms = 0.0, eel = 0.0;
    __syncthreads();
    int ncyc = 0;
    while (iteration < o.maximum_scf_cycles && !converged) {
        fock_build(a, f, H, P, F, tei, sm, &e1, &e2, &eq);
        tm.lap(PDG_T_FOCK);
        ncyc++;
        eel = e1 + e2 + eq;
        if (!isfinite(eel)) { st = PDG_NAN; break; }
        converged = (iteration > 0) && (rms <= o.density_tolerance) && (deltaeold <= o.energy_tolerance);
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
            for (int i = tid / 32; i < N; i += PDG_WARPS)
                for (int j = tid % 32; j <= i; j += 32) { hp[i * (i + 1) / 2 + j] = P[(size_t)i * N + j]; hf[i * (i + 1) / 2 + j] = F[(size_t)i * N + j]; }
            double *FP = wsf + pl.A;
            block_gemm(N, N, N, F, N, 1, P, N, 1, false, sm, [&](int i, int j, double v) { FP[(size_t)i * N + j] = v; });
            double emx = 0.0;
            for (int i = tid / 32; i < N; i += PDG_WARPS)
                for (int j = tid % 32; j < i; j += 32) {
                    double ev = FP[(size_t)i * N + j] - FP[(size_t)j * N + i];
                    he[i * (i - 1) / 2 + j] = ev;
                    emx = fmax(emx, fabs(ev));
                }
            __syncthreads();
            double maxerr = block_max(emx, sm.red);
            double dots[PDG_MAX_HISTORY];
            for (int m = 0; m < PDG_MAX_HISTORY; m++) dots[m] = 0.0;
            const int ne = N * (N - 1) / 2;
            for (int k = tid; k < ne; k += PDG_BLOCK) {
                double en_ = he[k];
                for (int m = 0; m < matnum; m++) dots[m] += wsf[pl.hE + (size_t)ctl[2 + m] * hl + k] * en_;
            }
            for (int m = 0; m < matnum; m++) {
                double b = 2.0 * block_sum(dots[m], sm.red);
                if (tid == 0) { int n = ctl[2 + m]; Bm[n * PDG_MAX_HISTORY + newest] = b; Bm[newest * PDG_MAX_HISTORY + n] = b; }
            }
            __syncthreads();
            tm.lap(PDG_T_DIIS_SAVE);
            if (iteration > 0) {
                if (o.use_rca) {
                    if (qdiis && maxerr > 0.8) { qdiis = 0; qrca = 1; }
                    else if (iteration > 1 && qrca && maxerr < o.diis_onset) { qdiis = 1; qrca = 0; }
                }
                if (qdiis) {
                    if (tid == 0) {   // DIIS_Iterate: bordered solve, drop the oldest until well conditioned
                        int mn = ctl[1];
                        ctl[21] = 0;
                        while (mn > 1) {
                            int n1 = mn + 1;
                            double Am[17 * 17], bv[17];
                            for (int i = 0; i < n1 * n1; i++) Am[i] = 0.0;
                            for (int i = 0; i < mn; i++)
                                for (int j = 0; j < mn; j++) Am[i * n1 + j] = Bm[ctl[2 + i] * PDG_MAX_HISTORY + ctl[2 + j]];
                            for (int i = 0; i < mn; i++) { Am[mn * n1 + i] = -1.0; Am[i * n1 + mn] = -1.0; bv[i] = 0.0; }
                            bv[mn] = -1.0;
                            bool ok = small_solve(n1, Am, bv);
                            bv[mn] = -1.0;
                            double dev = 0.0;
                            for (int i = 0; i < n1; i++) dev += bv[i];
                            if (ok && fabs(dev) < 1.0e-6) { for (int i = 0; i < mn; i++) cf[i] = bv[i]; ctl[21] = 1; break; }
                            mn--;
                            for (int i = 0; i < mn; i++) ctl[2 + i] = ctl[3 + i];
                            for (int i = mn; i < hist; i++) { ctl[2 + i] = ctl[2 + i - 1] + 1; if (ctl[2 + i] >= hist) ctl[2 + i] -= hist; }
                        }
                        ctl[1] = mn;
                    }
                    __syncthreads();
                    if (ctl[21]) {
                        const int mn = ctl[1];
                        for (size_t k = tid; k < NN; k += PDG_BLOCK) {
                            int i = (int)(k / N), j = (int)(k % N);
                            int pkk = (i >= j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
                            double pp = 0.0, ff = 0.0;
                            for (int m = 0; m < mn; m++) {
                                size_t off = (size_t)ctl[2 + m] * hl + pkk;
                                pp += cf[m] * wsf[pl.hP + off]; ff += cf[m] * wsf[pl.hF + off];
                            }
                            P[k] = pp; F[k] = ff;
                        }
                        __syncthreads();
                    }
                } else if (o.use_rca && qrca) {
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
            if (o.use_rca) {
                double *rP = wsf + pl.rP, *rF = wsf + pl.rF;
                for (size_t k = tid; k < NN; k += PDG_BLOCK) { rP[k] = P[k]; rF[k] = F[k]; }
            }
            iteration++;
        }
        deltaeold = deltae; eold = etemp;
        __syncthreads();
        tm.lap(PDG_T_ITERATE);
        rms = density_step(a, wsf, F, P, sm, tm);
        valid = true;
    }
    if (converged) st = PDG_OK;
    if (tid == 0) {
        double *E = a.energies + (size_t)f * PDG_NENERGY;
        E[0] = eel; E[1] = e1 + e2; E[2] = en; E[3] = base; E[4] = eq; E[5] = e1; E[6] = e2; E[7] = rms;
        a.status[f] = st;
        if (a.ncycles) a.ncycles[f] = iteration;
        tm.slot[PDG_T_TOTAL] = (double)(clock64() - t_begin);
        tm.slot[PDG_T_CYCLES] = (double)ncyc;
    }
}

size_t scf_smem_bytes(int N) { return sizeof(double) * (32 + 2 * TILE * KCH + 256 + 7 * (size_t)N) + sizeof(int) * (64 + (size_t)N + 2); }

void launch_scf(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *phi, const pdg_scf_options &o,
                double *density, int use_density, double *energies, double *charges, int *status, int *ncycles,
                double *ws, int fock_only, double *fock_out, cudaStream_t st)
{
    SCFArgs a;
    a.s = s; a.plan = p; a.n_frames = n_frames; a.phi = phi; a.o = o; a.density = density; a.use_density = use_density;
    a.energies = energies; a.charges = charges; a.status = status; a.ncycles = ncycles; a.ws = ws;
    a.fock_only = fock_only; a.fock_out = fock_out;
    size_t sm = scf_smem_bytes(s.n_basis);
    static size_t configured = 0;
    if (sm > 48 * 1024 && sm > configured) {
        cudaFuncSetAttribute(k_scf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        configured = sm;
    }
    k_scf<<<n_frames, PDG_BLOCK, sm, st>>>(a);
}
