// wide.cu - the SCF of ONE large QC region spread over the whole GPU (pdg_wide_*, include/pdg.h).
//
// The single-frame kernel of scf.cu gives one CTA to each frame: right for many small frames, but a 600-atom region
// (N = 1200) would run its O(N^3) density steps on one SM.  Here every phase of one SCF cycle is a grid-wide
// kernel (or a cuBLAS GEMM for the dense products), queued by the host on one stream; the converger's scalar state
// lives on the device, and the host reads one small control record per cycle to decide whether to go on.
//
//   Fock build        F = H + G(P) (QCModelMNDO_Fock, QCModelMNDO.c:700; G of MNDOIntegrals_MakeFockG,
//                     MNDOIntegrals.c:51, as J/K block contractions, one thread per output element), traces and the
//                     Lowdin QC/MM term (QCModelMNDO_QCMMFockLowdin, :1808)
//   DIIS / ODA        DIIS_Fock_Save (DIISSCFConverger.c:385: e = F P - P F by GEMMs on the last step's
//                     eigenvectors), DIIS_Iterate (:530; bordered solve with drop-oldest), RCA_Iterate (:661), the mode
//                     switching of IterateWithoutDensities (:147) and the convergence test (:116)
//   density step      QCOnePDM_MakeFromFock (QCOnePDM.c:403) as in scf.cu but grid-wide: Householder
//                     tridiagonalisation (two kernels per column, replayed from a CUDA graph), FP64 bisection for the
//                     min(n_occ, N - n_occ) wanted eigenvalues, inverse iteration (one thread per vector,
//                     re-orthogonalised inside clusters of close eigenvalues), blocked compact-WY back-transformation
//                     and P = 2 Z Z^T or 2 (1 - Z Z^T) by DGEMM.
// The integrals and the gradients are the batch kernels of integrals.cu run on this one frame (their grids span the
// frame's atom pairs).  Reductions are taken in a fixed order, so results do not depend on timing.
#include "common.cuh"
#include "multipole.cuh"
#include <cublas_v2.h>
#include <vector>
#include <cstring>

namespace wide {

#define WB 256                 // threads per block of the grid-wide kernels
#define WW (WB / 32)
#define WMAXH PDG_MAX_HISTORY
#define WNB 64                 // reflectors per back-transformation block

// Converger state on the device (one per wide object), read by the host after every cycle's control kernel.
struct Ctl {
    int iteration, converged, status, ncyc, valid, have_z, qdiis, qrca, matnum, newest, good, do_extrap, do_oda, done;
    int slots[WMAXH];
    double eold, deltaeold, rms, eel, e1, e2, eq, etemp, deltae, maxerr, mu, enuc, base;
    double cf[WMAXH];
    double B[WMAXH * WMAXH];
};

// Workspace plan (doubles from the base): the frame plan of the integral and gradient kernels first, then the
// regions of the grid-wide SCF.
struct WPlan {
    FramePlan fp;   // only tei, pair_e, pair_g and H (the integral and gradient kernels' regions) are laid out
    size_t F, A, C, rP, rF, hP, hF, hE, Zc, G, colbuf, vbuf, q, tpart, pk, part, d, e, tau, eig, cst, lu, y, vb, sb, tb, wb, ctl;
    // mixed method: the base of the perturbative steps (F0, P0, all eigenvalues, the complementary vectors in FP64), the
    // matrix the last density step was applied to, and FP32 work (float offsets from f32)
    size_t BF, BP, BL, Ft, Zcc, f32;
    size_t D, ZY, V32, Gi, T1, E, Lp, T2, Mp, K, K2, R, EK, Am, U, Sm, WZ2, DQ, P32, f32_total;
    size_t total;
    int kvp;   // vectors rounded up to 32 (interleaved inverse-iteration arrays; wanted or complementary set)
    int parts; // partial-sum slots per reduction
};

__host__ inline WPlan wide_plan(const DeviceSystem &s)
{
    WPlan w;
    std::memset(&w, 0, sizeof(w));
    const size_t N = s.n_basis, NN = N * N, kv = s.n_vec > 0 ? s.n_vec : 1, nc = N > kv ? N - kv : 1;
    w.kvp = (int)((N + 31) & ~size_t(31));
    w.parts = 1024;
    size_t o = 0;
    auto take = [&](size_t n) { size_t r = o; o += align32(n); return r; };
    w.fp.tei = take(s.tei_total);
    w.fp.pair_e = take((size_t)s.n_pairs * PDG_PAIR_E_STRIDE);
    w.fp.pair_g = take((size_t)s.n_pairs * 3);
    w.fp.H = take(NN);
    w.fp.stride = o;
    w.F = take(NN); w.A = take(NN); w.C = take(NN); w.rP = take(NN); w.rF = take(NN);
    w.hP = take(WMAXH * NN); w.hF = take(WMAXH * NN); w.hE = take(WMAXH * NN);
    w.Zc = take(N * kv); w.G = take(N * kv);
    w.colbuf = take(2 * N); w.vbuf = take(2 * N); w.q = take(2 * N); w.tpart = take(2 * (size_t)w.parts); w.pk = take((size_t)s.n_cel + 1);
    w.part = take((size_t)w.parts * 32);
    w.d = take(N); w.e = take(N); w.tau = take(N); w.eig = take(N); w.cst = take(N / 2 + 2);
    w.lu = take(5 * N * (size_t)w.kvp + (N * (size_t)w.kvp + 7) / 8);
    w.y = take(N * (size_t)w.kvp);
    w.vb = take(N * WNB); w.sb = take(WNB * WNB); w.tb = take(WNB * WNB); w.wb = take(2 * WNB * N);   // W and T W: WNB x (up to N columns) each
    w.ctl = take((sizeof(Ctl) + 7) / 8);
    w.BF = take(NN); w.BP = take(NN); w.BL = take(N); w.Ft = take(NN); w.Zcc = take(N * nc);
    size_t f = 0;
    auto tf = [&](size_t n) { size_t r = f; f += (n + 63) & ~size_t(63); return r; };
    w.D = tf(NN); w.ZY = tf(2 * N * kv); w.V32 = tf(N * nc); w.Gi = tf(nc * kv); w.T1 = tf(N * kv); w.E = tf(nc * kv);
    w.Lp = tf(kv * kv); w.T2 = tf(N * nc); w.Mp = tf(nc * nc); w.K = tf(nc * kv); w.K2 = tf(nc * kv); w.R = tf(nc * kv);
    w.EK = tf(kv * kv); w.Am = tf(kv * kv); w.U = tf(kv * kv); w.Sm = tf(N * kv); w.WZ2 = tf(2 * N * kv); w.DQ = tf(NN);
    w.P32 = tf(NN);
    w.f32_total = f;
    w.f32 = take((f + 1) / 2);
    w.total = align32(o);
    return w;
}

// ---------------------------------------------------------------------------------------------------------------
// Deterministic partial sums: every block writes its partials to part[slot * parts + block]; single-block kernels sum
// them in block order.
__device__ __forceinline__ double block_reduce(double v, double *red)
{
    return block_sum(v, red);
}

// ---------------------------------------------------------------------------------------------------------------
// Fock build.  pk: one-centre densities of every atom with the off-diagonal factor 2 (the Coulomb right-hand sides).
__global__ void __launch_bounds__(WB) k_pk(DeviceSystem s, const double *__restrict__ P, double *__restrict__ pk)
{
    const int N = s.n_basis;
    for (int e = blockIdx.x * WB + threadIdx.x; e < s.n_cel; e += gridDim.x * WB) {
        const int A = s.cel[e] >> 4, ab = s.cel[e] & 15, as = s.atom_start[A];
        const int m = MP_DA[ab], n = MP_DB[ab];
        pk[e] = (m == n ? 1.0 : 2.0) * P[(size_t)(as + m) * N + as + n];
    }
}

__global__ void __launch_bounds__(WB) k_fock(DeviceSystem s, const double *__restrict__ H, const double *__restrict__ P,
                                             const double *__restrict__ tei, const double *__restrict__ pk, double *__restrict__ F)
{
    const int N = s.n_basis, n_out = s.n_cel + s.n_xel;
    for (int e = blockIdx.x * WB + threadIdx.x; e < n_out; e += gridDim.x * WB) {
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
}

// tr(P H) and tr(P F) over the lower triangle (off-diagonal and diagonal parts apart, as scf.cu), one warp per row;
// block partials to part slots 0..3.
__global__ void __launch_bounds__(WB) k_traces(int N, const double *__restrict__ P, const double *__restrict__ H,
                                               const double *__restrict__ F, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, gw = blockIdx.x * WW + (threadIdx.x >> 5), nw = gridDim.x * WW;
    double th = 0.0, tf = 0.0, dh = 0.0, df = 0.0;
    for (int i = gw; i < N; i += nw)
        for (int j = lane; j <= i; j += 32) {
            const size_t k = (size_t)i * N + j;
            const double pv = P[k];
            if (j < i) { th = fma(pv, H[k], th); tf = fma(pv, F[k], tf); }
            else { dh = fma(pv, H[k], dh); df = fma(pv, F[k], df); }
        }
    th = block_reduce(th, red); tf = block_reduce(tf, red); dh = block_reduce(dh, red); df = block_reduce(df, red);
    if (threadIdx.x == 0) {
        part[0 * parts + blockIdx.x] = th; part[1 * parts + blockIdx.x] = tf;
        part[2 * parts + blockIdx.x] = dh; part[3 * parts + blockIdx.x] = df;
    }
}

// Lowdin charges q_A = Z_A - sum P_mm and the QC/MM term: F_mm -= phi_A, partial q . phi to part slot 4 (one block).
__global__ void __launch_bounds__(WB) k_lowdin(DeviceSystem s, const double *__restrict__ P, const double *__restrict__ phi,
                                               double *__restrict__ F, double *__restrict__ charges, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    const int N = s.n_basis;
    double tq = 0.0;
    for (int A = threadIdx.x; A < s.n_atoms; A += WB) {
        const int no = s.atom_norb[A], as = s.atom_start[A];
        double ps = 0.0;
        for (int m = 0; m < no; m++) ps += P[(size_t)(as + m) * N + as + m];
        const double q = elem(s, s.atom_elem[A])[PDG_E_ZCORE] - ps;
        if (charges) charges[A] = q;
        if (phi) {
            tq += q * phi[A];
            for (int m = 0; m < no; m++) F[(size_t)(as + m) * N + as + m] -= phi[A];
        }
    }
    tq = block_reduce(tq, red);
    if (threadIdx.x == 0) part[4 * parts] = tq;
}

__device__ __forceinline__ double sum_parts(const double *part, int slot, int parts, int nb)
{
    double t = 0.0;
    for (int b = 0; b < nb; b++) t += part[(size_t)slot * parts + b];
    return t;
}

// The same sum by one warp: lane l adds blocks l, l + 32, ... (loads in flight together), then the fixed shuffle tree;
// every lane gets the result, and every block that calls it gets the same value.
__device__ __forceinline__ double warp_sum_parts(const double *part, int nb)
{
    const int lane = threadIdx.x & 31;
    double t = 0.0;
    for (int b = lane; b < nb; b += 32) t += part[b];
    return warp_sum(t);
}

// Control after the Fock build (one thread): energies, the convergence test (DIISSCFConverger_Converged,
// DIISSCFConverger.c:116-121, signed deltaeold), the DIIS slot of this cycle.
__global__ void k_control_fock(Ctl *c, const double *__restrict__ part, int parts, int nb_traces, pdg_scf_options o, int hist)
{
    if (threadIdx.x >= 32) return;
    const double th = warp_sum_parts(part, nb_traces), tf = warp_sum_parts(part + parts, nb_traces);
    const double dh = warp_sum_parts(part + 2 * (size_t)parts, nb_traces), df = warp_sum_parts(part + 3 * (size_t)parts, nb_traces);
    if (threadIdx.x != 0) return;
    const double e1 = 2.0 * th + dh, e2 = 0.5 * ((2.0 * tf + df) - e1), eq = part[4 * parts];
    c->e1 = e1; c->e2 = e2; c->eq = eq; c->eel = e1 + e2 + eq;
    c->ncyc++;
    if (!isfinite(c->eel)) { c->status = PDG_NAN; c->done = 1; return; }
    c->converged = (c->iteration > 0) && (c->rms <= o.density_tolerance) && (c->deltaeold <= o.energy_tolerance);
    if (c->converged) { c->status = PDG_OK; c->done = 1; return; }
    c->deltae = c->eel - c->eold; c->etemp = c->eel;
    if (c->valid) {
        int mn = c->matnum, newest;
        if (mn < hist) { mn++; newest = c->slots[mn - 1]; }
        else { mn = hist; newest = c->slots[0]; for (int i = 0; i < hist - 1; i++) c->slots[i] = c->slots[i + 1]; c->slots[hist - 1] = newest; }
        c->matnum = mn; c->newest = newest;
    }
}

// DIIS history: P and F into the newest slot (dense).
__global__ void __launch_bounds__(WB) k_pack(size_t NN, const Ctl *c, const double *__restrict__ P, const double *__restrict__ F,
                                             double *__restrict__ hP, double *__restrict__ hF)
{
    const size_t off = (size_t)c->newest * NN;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) { hP[off + k] = P[k]; hF[off + k] = F[k]; }
}

// Error vector from C: e_ij = sg (C_ij - C_ji) for i > j (C = G Z^T with G = F Z, or C = F P), into the newest slot
// (strict lower triangle, dense row-major positions); block maxima to part slot 5.
template <typename T>
__global__ void __launch_bounds__(WB) k_error(int N, const Ctl *c, const T *__restrict__ C, double sg, double *__restrict__ hE,
                                              double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    double *he = hE + (size_t)c->newest * N * N;
    const int lane = threadIdx.x & 31, gw = blockIdx.x * WW + (threadIdx.x >> 5), nw = gridDim.x * WW;
    double mx = 0.0;
    for (int i = gw; i < N; i += nw)
        for (int j = lane; j < i; j += 32) {
            const double ev = sg * ((double)C[(size_t)i * N + j] - (double)C[(size_t)j * N + i]);
            he[(size_t)i * N + j] = ev;
            mx = fmax(mx, fabs(ev));
        }
    mx = block_max(mx, red);
    if (threadIdx.x == 0) part[5 * parts + blockIdx.x] = mx;
}

// B-matrix row: dots of the newest error vector with every stored one (strict lower triangles), block partials to
// part slots 8 + m.
__global__ void __launch_bounds__(WB) k_dots(int N, const Ctl *c, const double *__restrict__ hE, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, gw = blockIdx.x * WW + (threadIdx.x >> 5), nw = gridDim.x * WW;
    const size_t NN = (size_t)N * N;
    const double *en = hE + (size_t)c->newest * NN;
    const int mn = c->matnum;
    double acc[WMAXH];
    for (int m = 0; m < WMAXH; m++) acc[m] = 0.0;
    for (int i = gw; i < N; i += nw)
        for (int j = lane; j < i; j += 32) {
            const size_t k = (size_t)i * N + j;
            const double v = en[k];
            for (int m = 0; m < mn; m++) acc[m] = fma(hE[(size_t)c->slots[m] * NN + k], v, acc[m]);
        }
    for (int m = 0; m < mn; m++) {
        const double t = block_reduce(acc[m], red);
        if (threadIdx.x == 0) part[(size_t)(8 + m) * parts + blockIdx.x] = t;
    }
}

// ODA traces t1..t4 = F.P, F.rP, rF.P, rF.rP (full matrices), block partials to part slots 24..27.
__global__ void __launch_bounds__(WB) k_oda_traces(size_t NN, const double *__restrict__ F, const double *__restrict__ P,
                                                   const double *__restrict__ rF, const double *__restrict__ rP, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) {
        t1 += F[k] * P[k]; t2 += F[k] * rP[k]; t3 += rF[k] * P[k]; t4 += rF[k] * rP[k];
    }
    t1 = block_reduce(t1, red); t2 = block_reduce(t2, red); t3 = block_reduce(t3, red); t4 = block_reduce(t4, red);
    if (threadIdx.x == 0) {
        part[24 * parts + blockIdx.x] = t1; part[25 * parts + blockIdx.x] = t2;
        part[26 * parts + blockIdx.x] = t3; part[27 * parts + blockIdx.x] = t4;
    }
}

// Small dense solve A x = b (n <= 17) by one warp: Gauss-Jordan with partial pivoting, rejecting a reciprocal
// 1-norm condition below 1e-15 (SymmetricMatrix_SolveLinearEquations' test, SymmetricMatrix.c:1412-1450).
__device__ bool warp_solve(int n, const double *Ain, const double *bin, double *M, double *x)
{
    const int lane = threadIdx.x & 31, w2 = 2 * n + 1;
    for (int e = lane; e < n * w2; e += 32) {
        const int i = e / w2, j = e % w2;
        M[e] = j < n ? Ain[i * n + j] : (j < 2 * n ? (j - n == i ? 1.0 : 0.0) : bin[i]);
    }
    __syncwarp();
    double cs = 0.0;
    if (lane < n) for (int i = 0; i < n; i++) cs += fabs(M[i * w2 + lane]);
    const double anorm = warp_max(cs);
    for (int k = 0; k < n; k++) {
        double v = (lane >= k && lane < n) ? fabs(M[lane * w2 + k]) : -1.0;
        int iv = lane;
        for (int off = 16; off > 0; off >>= 1) {
            const double v2 = __shfl_xor_sync(0xffffffffu, v, off);
            const int i2 = __shfl_xor_sync(0xffffffffu, iv, off);
            if (v2 > v || (v2 == v && i2 < iv)) { v = v2; iv = i2; }
        }
        if (v == 0.0) return false;
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
    double ci = 0.0;
    if (lane < n) for (int i = 0; i < n; i++) ci += fabs(M[i * w2 + n + lane] / M[i * w2 + i]);
    const double inorm = warp_max(ci);
    if (lane < n) x[lane] = M[lane * w2 + 2 * n] / M[lane * w2 + lane];
    __syncwarp();
    return anorm * inorm < 1.0e15;
}

// Control after the DIIS save (one warp): the B-matrix row, the mode switch (RCA_ONSET 0.8, diisOnset), the DIIS
// solve with drop-oldest, or the ODA step length from the four traces (DIISSCFConverger.c:661-760).
__global__ void k_control_diis(Ctl *c, const double *__restrict__ part, int parts, int nb, int nb_oda, pdg_scf_options o, int hist)
{
    __shared__ double M[17 * 35], Ab[17 * 17], bb[17], x[17];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    double mx = 0.0;
    for (int b = lane; b < nb; b += 32) mx = fmax(mx, part[5 * (size_t)parts + b]);
    mx = warp_max(mx);
    const int matnum = c->matnum;
    for (int m = 0; m < matnum; m++) {
        const double t = 2.0 * warp_sum_parts(part + (size_t)(8 + m) * parts, nb);
        if (lane == 0) {
            const int n = c->slots[m];
            c->B[n * WMAXH + c->newest] = t; c->B[c->newest * WMAXH + n] = t;
        }
    }
    const double t1 = warp_sum_parts(part + 24 * (size_t)parts, nb_oda), t2 = warp_sum_parts(part + 25 * (size_t)parts, nb_oda);
    const double t3 = warp_sum_parts(part + 26 * (size_t)parts, nb_oda), t4 = warp_sum_parts(part + 27 * (size_t)parts, nb_oda);
    __syncwarp();
    if (lane == 0) {
        c->maxerr = mx;
        c->do_extrap = 0; c->do_oda = 0;
        if (c->iteration > 0 && o.use_rca) {
            if (c->qdiis && c->maxerr > 0.8) { c->qdiis = 0; c->qrca = 1; }
            else if (c->iteration > 1 && c->qrca && c->maxerr < o.diis_onset) { c->qdiis = 1; c->qrca = 0; }
        }
    }
    __syncwarp();
    if (c->iteration > 0 && c->qdiis) {
        int mn = c->matnum, good = 0;
        while (mn > 1) {
            const int n1 = mn + 1;
            for (int e = lane; e < n1 * n1; e += 32) {
                const int i = e / n1, j = e % n1;
                Ab[e] = (i < mn && j < mn) ? c->B[c->slots[i] * WMAXH + c->slots[j]] : ((i == mn && j == mn) ? 0.0 : -1.0);
            }
            if (lane < n1) bb[lane] = lane == mn ? -1.0 : 0.0;
            __syncwarp();
            const bool ok = warp_solve(n1, Ab, bb, M, x);
            double dev = -1.0;
            for (int i = 0; i < mn; i++) dev += x[i];
            if (ok && fabs(dev) < 1.0e-6) {
                if (lane < mn) c->cf[lane] = x[lane];
                good = 1;
                break;
            }
            mn--;
            __syncwarp();
            if (lane == 0) {
                for (int i = 0; i < mn; i++) c->slots[i] = c->slots[i + 1];
                for (int i = mn; i < hist; i++) { c->slots[i] = c->slots[i - 1] + 1; if (c->slots[i] >= hist) c->slots[i] -= hist; }
            }
            __syncwarp();
        }
        if (lane == 0) { c->matnum = mn; c->good = good; c->do_extrap = good; }
    } else if (c->iteration > 0 && o.use_rca && c->qrca && lane == 0) {
        double ca = t1 - t2, cc = t3 - t4, dd = c->eold;
        const double etemp = c->etemp;
        ca += cc + 2.0 * (dd - etemp);
        double cb = etemp - ca - cc - dd, fmin_ = etemp, mub = 1.0, mu;
        if (c->eold < etemp) { fmin_ = c->eold; mub = 0.0; }
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
        c->mu = mu;
        c->etemp = ((ca * mu + cb) * mu + cc) * mu + dd;
        c->do_oda = 1;
    }
    __syncwarp();
    if (lane == 0) {
        if (c->valid) c->iteration++;
        c->deltaeold = c->deltae; c->eold = c->etemp;
    }
}

// DIIS extrapolation P = sum c_m hP_m, F = sum c_m hF_m, or the ODA mixture; then the RCA copies.
__global__ void __launch_bounds__(WB) k_iterate(size_t NN, const Ctl *c, const double *__restrict__ hP, const double *__restrict__ hF,
                                                double *__restrict__ P, double *__restrict__ F, double *__restrict__ rP, double *__restrict__ rF,
                                                int use_rca)
{
    const int ex = c->do_extrap, oda = c->do_oda, mn = c->matnum;
    const double mu = c->mu, nu = 1.0 - c->mu;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) {
        double p = P[k], f = F[k];
        if (ex) {
            double pp = 0.0, ff = 0.0;
            for (int m = 0; m < mn; m++) {
                const size_t off = (size_t)c->slots[m] * NN + k;
                pp = fma(c->cf[m], hP[off], pp); ff = fma(c->cf[m], hF[off], ff);
            }
            p = pp; f = ff;
        } else if (oda) {
            p = mu * p + nu * rP[k]; f = mu * f + nu * rF[k];
        }
        P[k] = p; F[k] = f;
        if (use_rca) { rP[k] = p; rF[k] = f; }
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Householder tridiagonalisation of the dense symmetric A (N x N, both triangles kept; dsytd2 'L'), one grid-wide
// kernel per column.  With A(k) the matrix after k steps, step k forms the reflector v_k, tau_k from column k of A(k)
// (rows k+1 ..), the product q_k = A(k)22 v_k over rows and columns k+1 .., w_k = tau_k q_k - K_k v_k with
// K_k = tau_k^2 (q_k . v_k) / 2, and A(k+1)22 = A(k)22 - v_k w_k^T - w_k v_k^T.  Launch k finishes step k - 1 and
// starts step k in one pass over the rows:
//   * every block forms w_{k-1} from q_{k-1} (and the block partials of q_{k-1} . v_{k-1}) of launch k - 1, then
//     column k of A(k) from the copy of column k of A(k-1) that launch k - 1 left (its rows k ..) minus the rank-2
//     terms of step k - 1, and from it the reflector v_k (dlarfg; identical in every block);
//   * one warp per row i > k: the row's columns > k are updated by step k - 1 and, in the same pass, multiplied by
//     v_k (q_k, and the block partials of q_k . v_k); the row's column k takes v_k (the back-transformation reads the
//     reflectors there); row k + 1, updated, is copied out as the next launch's column.
// q, the reflector, the column copy and the partials are double-buffered by the parity of k, since launch k reads
// launch k - 1's and writes its own.
__device__ void reflector(int m, const double *__restrict__ x, double *v, double *red, double *tau_out, double *e_out)
{
    const double alpha = x[0];
    double part = 0.0;
    for (int i = 1 + threadIdx.x; i < m; i += WB) part = fma(x[i], x[i], part);
    const double xn2 = block_sum(part, red);
    double tau = 0.0, e = alpha, scal = 0.0;
    if (xn2 != 0.0) {
        const double beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
        tau = (beta - alpha) / beta; e = beta; scal = 1.0 / (alpha - beta);
    }
    for (int i = threadIdx.x; i < m; i += WB) v[i] = (i == 0) ? 1.0 : (tau != 0.0 ? x[i] * scal : 0.0);
    *tau_out = tau; *e_out = e;
    __syncthreads();
}

// v_{k-1} and w_{k-1} (N - k entries each, indexed from row k) into shared memory; false for k = 0.
__device__ bool previous_step(int N, int k, const double *__restrict__ vbuf, const double *__restrict__ qbuf, const double *__restrict__ tau,
                              const double *__restrict__ tpart, int parts, int nb, double *vp, double *wp)
{
    if (k == 0) return false;
    const int pp = (k - 1) & 1, mp = N - k;
    const double t = tau[k - 1];
    __shared__ double qv_s;
    if (threadIdx.x < 32) {
        const double qv = warp_sum_parts(tpart + pp * parts, nb);
        if (threadIdx.x == 0) qv_s = qv;
    }
    __syncthreads();
    const double K = 0.5 * t * t * qv_s;
    for (int i = threadIdx.x; i < mp; i += WB) { const double vi = vbuf[pp * N + i]; vp[i] = vi; wp[i] = fma(-K, vi, t * qbuf[pp * N + i]); }
    __syncthreads();
    return true;
}

__global__ void __launch_bounds__(WB) k_tri_step(int N, int k, double *__restrict__ A, double *__restrict__ colbuf, double *__restrict__ vbuf,
                                                 double *__restrict__ qbuf, double *__restrict__ d, double *__restrict__ e,
                                                 double *__restrict__ tau, double *__restrict__ tpart, int parts, int nb)
{
    extern __shared__ double sm[];
    __shared__ double red[32];
    double *vp = sm, *wp = sm + N, *c = sm + 2 * N, *vk = sm + 3 * N;
    const int lane = threadIdx.x & 31, par = k & 1, mp = N - k, m = N - k - 1, c0 = k + 1;
    const bool upd = previous_step(N, k, vbuf, qbuf, tau, tpart, parts, nb, vp, wp);
    // column k of A(k), rows k .. N-1 (index r = row - k)
    const double *cb = colbuf + par * N + k;
    for (int r = threadIdx.x; r < mp; r += WB) c[r] = upd ? fma(-vp[r], wp[0], fma(-wp[r], vp[0], cb[r])) : cb[r];
    __syncthreads();
    double tk, ek;
    reflector(m, c + 1, vk, red, &tk, &ek);
    if (blockIdx.x == 0) {
        for (int i = threadIdx.x; i < m; i += WB) vbuf[par * N + i] = vk[i];
        if (threadIdx.x == 0) { tau[k] = tk; e[k] = ek; d[k] = c[0]; }
    }
    double pv = 0.0;
    const int gw = blockIdx.x * WW + (threadIdx.x >> 5), nw = gridDim.x * WW;
    double *next = colbuf + (1 - par) * N + c0;   // row k+1 of A(k+1)... of A(k) from column k+1 on: launch k+1's column
    for (int i = gw; i < m; i += nw) {
        double *row = A + (size_t)(c0 + i) * N + c0;
        const double vi = upd ? vp[i + 1] : 0.0, wi = upd ? wp[i + 1] : 0.0;   // row c0 + i is entry i + 1 of step k - 1
        double sacc = 0.0;
        // eight loads of the row in flight per lane before the arithmetic that uses them
        for (int j0 = lane; j0 < m; j0 += 256) {
            double a[8];
#pragma unroll
            for (int u = 0; u < 8; u++) { const int j = j0 + 32 * u; a[u] = j < m ? row[j] : 0.0; }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int j = j0 + 32 * u;
                if (j < m) {
                    double av = a[u];
                    if (upd) { av = fma(-vi, wp[j + 1], fma(-wi, vp[j + 1], av)); row[j] = av; }
                    if (i == 0) next[j] = av;
                    sacc = fma(av, vk[j], sacc);
                }
            }
        }
        sacc = warp_sum(sacc);
        if (lane == 0) {
            qbuf[par * N + i] = sacc;
            pv = fma(sacc, vk[i], pv);
            if (i >= 1) A[(size_t)(c0 + i) * N + k] = vk[i];   // the reflector, below the subdiagonal of column k
        }
    }
    pv = block_sum(pv, red);
    if (threadIdx.x == 0) tpart[par * parts + blockIdx.x] = pv;
}

// After the last step (k = N - 3): step N - 3's update of the trailing 2 x 2 block gives d[N-2], e[N-2], d[N-1].
__global__ void __launch_bounds__(WB) k_tri_last(int N, const double *__restrict__ A, const double *__restrict__ colbuf,
                                                 const double *__restrict__ vbuf, const double *__restrict__ qbuf, double *__restrict__ d,
                                                 double *__restrict__ e, double *__restrict__ tau, const double *__restrict__ tpart, int parts, int nb)
{
    extern __shared__ double sm[];
    double *vp = sm, *wp = sm + N;
    if (blockIdx.x) return;
    const int k = N - 2;
    const bool upd = previous_step(N, k, vbuf, qbuf, tau, tpart, parts, nb, vp, wp);
    if (threadIdx.x == 0) {
        const double *cb = colbuf + (k & 1) * N + k;
        const double a00 = cb[0], a10 = cb[1], a11 = A[(size_t)(N - 1) * N + N - 1];
        d[N - 2] = upd ? a00 - 2.0 * vp[0] * wp[0] : a00;
        e[N - 2] = upd ? a10 - vp[1] * wp[0] - wp[1] * vp[0] : a10;
        d[N - 1] = upd ? a11 - 2.0 * vp[1] * wp[1] : a11;
        tau[N - 2] = 0.0;
        e[N - 1] = 0.0;
    }
}

// Start: A = F and the first column (row 0 of the symmetric F).
__global__ void __launch_bounds__(WB) k_tri_start(int N, const double *__restrict__ F, double *__restrict__ A, double *__restrict__ colbuf)
{
    const size_t NN = (size_t)N * N;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) A[k] = F[k];
    for (int i = blockIdx.x * WB + threadIdx.x; i < N; i += gridDim.x * WB) colbuf[i] = F[i];
}

// ---------------------------------------------------------------------------------------------------------------
// Eigenvalues of the tridiagonal T (d, e) by FP64 bisection on Sturm counts (as dstebz): eigenvalue of index
// first + t, t < nv, one thread each; the result in eig[t].
__device__ __forceinline__ int sturm(int N, const double *d, const double *e, double x, double pivmin)
{
    int c = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    c += (q < 0.0);
    for (int i = 1; i < N; i++) {
        // e^2 / q with the reciprocal from an FP32 seed and two FP64 Newton steps (relative error ~1e-16; only the sign
        // of each pivot counts): a fraction of the FP64 instructions of a division.  Pivots outside the float range
        // take the division.
        double r;
        const double aq = fabs(q);
        if (aq > 1.0e-30 && aq < 1.0e30) {
            r = (double)__frcp_rn((float)q);
            r = r * fma(-q, r, 2.0);
            r = r * fma(-q, r, 2.0);
        } else r = 1.0 / q;
        q = (d[i] - x) - e[i - 1] * e[i - 1] * r;
        if (fabs(q) < pivmin) q = -pivmin;
        c += (q < 0.0);
    }
    return c;
}

// The Sturm count in FP32, for the multisection rounds whose bracket is still wide (the count is exact wherever x is
// farther than ~1e-6 ||T|| from every eigenvalue).
__device__ __forceinline__ int sturm32(int N, const double *d, const double *e, double x, float pivmin)
{
    int c = 0;
    const float xf = (float)x;
    float q = (float)d[0] - xf;
    if (fabsf(q) < pivmin) q = -pivmin;
    c += (q < 0.0f);
    for (int i = 1; i < N; i++) {
        const float ef = (float)e[i - 1];
        q = ((float)d[i] - xf) - __fdividef(ef * ef, q);
        if (fabsf(q) < pivmin) q = -pivmin;
        c += (q < 0.0f);
    }
    return c;
}

// One warp per eigenvalue: multisection instead of bisection.  An FP64 warp instruction costs the same however many
// lanes are active, so the 32 lanes evaluate 31 interior points of the bracket at once (the cost of one bisection
// step) and the bracket shrinks 32-fold per round: about 11 rounds to round-off instead of 55 bisection steps.
#define MS_WARPS 4
__global__ void __launch_bounds__(32 * MS_WARPS) k_bisect(int N, int first, int nv, const double *__restrict__ d,
                                                          const double *__restrict__ e, double *__restrict__ eig)
{
    const int lane = threadIdx.x & 31, t = blockIdx.x * MS_WARPS + (threadIdx.x >> 5);
    if (t >= nv) return;
    double lo = 1e300, hi = -1e300, emax = 0.0;
    for (int i = lane; i < N; i += 32) {
        const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < N - 1 ? fabs(e[i]) : 0.0);
        lo = fmin(lo, d[i] - r); hi = fmax(hi, d[i] + r);
        if (i < N - 1) emax = fmax(emax, e[i] * e[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    }
    const double tnorm = fmax(fabs(lo), fabs(hi));
    const double pivmin = fmax(1e-300, 2.2250738585072014e-308 * fmax(1.0, emax));
    lo -= 2.2e-16 * tnorm * N + 2.0 * pivmin; hi += 2.2e-16 * tnorm * N + 2.0 * pivmin;
    const int idx = first + t;   // the eigenvalue with exactly idx eigenvalues below it
    // FP32 counts while the bracket is wider than 1e-4 ||T|| (its interior points stay far from the eigenvalue in
    // FP32 terms only then), with a margin of 1e-5 ||T|| kept on both sides of the FP32 bracket; FP64 after that
    const float piv32 = 1.0e-30f;
    for (int round = 0; round < 8 && hi - lo > 1.0e-4 * tnorm; round++) {
        const double x = lo + (hi - lo) * (double)(lane + 1) * (1.0 / 32.0);
        const bool above = lane == 31 ? true : sturm32(N, d, e, x, piv32) > idx;
        const unsigned b = __ballot_sync(0xffffffffu, above);
        const int l = __ffs(b) - 1;
        const double xl = __shfl_sync(0xffffffffu, x, l), xp = l > 0 ? __shfl_sync(0xffffffffu, x, max(l - 1, 0)) : lo;
        hi = fmin(hi, xl + 1.0e-5 * tnorm); lo = fmax(lo, xp - 1.0e-5 * tnorm);
    }
    // the FP64 counts at the widened bracket's ends confirm it; if not, the whole Gershgorin interval again
    {
        const bool ok_lo = lane != 0 || sturm(N, d, e, lo, pivmin) <= idx, ok_hi = lane != 1 || sturm(N, d, e, hi, pivmin) > idx;
        if (!__all_sync(0xffffffffu, ok_lo && ok_hi)) {
            lo = -tnorm - 2.2e-16 * tnorm * N - 2.0 * pivmin; hi = tnorm + 2.2e-16 * tnorm * N + 2.0 * pivmin;
        }
    }
    for (int round = 0; round < 40; round++) {
        if (hi - lo <= 2.2e-16 * fmax(fabs(lo), fabs(hi)) + pivmin) break;
        const double x = lo + (hi - lo) * (double)(lane + 1) * (1.0 / 32.0);   // lane 31: hi itself
        const bool above = lane == 31 ? true : sturm(N, d, e, x, pivmin) > idx;
        const unsigned b = __ballot_sync(0xffffffffu, above);
        const int l = __ffs(b) - 1;   // first point with more than idx eigenvalues below it
        const double xl = __shfl_sync(0xffffffffu, x, l), xp = l > 0 ? __shfl_sync(0xffffffffu, x, max(l - 1, 0)) : lo;
        if (xl >= hi && xp <= lo) break;   // no progress (round-off)
        hi = xl; lo = xp;
    }
    if (lane == 0) eig[t] = 0.5 * (lo + hi);
}

// Inverse iteration for the nv wanted eigenvectors, one thread per vector: the LU factors of T - lambda I with row
// interchanges (stored interleaved by vector, so the threads' accesses coalesce), four solves from a hashed start
// vector with rescaling between them, then normalisation.  Output: the vectors as columns of Zc (N x nv, column-major),
// in the tridiagonal basis.  Vectors of well-separated eigenvalues come out orthogonal to about eps ||T|| / gap; those of
// close eigenvalues are orthonormalised afterwards within their cluster (k_cluster_gs).
__device__ __forceinline__ unsigned int whash(unsigned int a, unsigned int b)
{
    unsigned int h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    return h;
}

__global__ void __launch_bounds__(32) k_invit(int N, int nv, int ld, const double *__restrict__ d, const double *__restrict__ e,
                                              const double *__restrict__ eig, double tnorm, double *__restrict__ lu,
                                              unsigned char *__restrict__ pv, double *__restrict__ y, double *__restrict__ Zc)
{
    const int t = blockIdx.x * 32 + threadIdx.x;
    if (t >= nv) return;
    const double sigma = eig[t], tiny = 1e-14 * tnorm + 1e-300;
    double *u0 = lu, *u1 = lu + (size_t)N * ld, *u2 = lu + 2 * (size_t)N * ld, *lm = lu + 3 * (size_t)N * ld;
    double ak = d[0] - sigma, bk = N > 1 ? e[0] : 0.0;
    for (int k = 0; k < N - 1; k++) {
        const double ck = e[k], an = d[k + 1] - sigma, bn = k + 1 < N - 1 ? e[k + 1] : 0.0;
        const bool sw = fabs(ak) < fabs(ck);
        double piv = sw ? ck : ak;
        if (fabs(piv) < tiny) piv = copysign(tiny, piv);
        const double r = 1.0 / piv, l = (sw ? ak : ck) * r;
        const double uu1 = sw ? an : bk, uu2 = sw ? bn : 0.0;
        u0[(size_t)k * ld + t] = r; u1[(size_t)k * ld + t] = uu1; u2[(size_t)k * ld + t] = uu2; lm[(size_t)k * ld + t] = l;
        pv[(size_t)k * ld + t] = sw;
        ak = fma(-l, uu1, sw ? bk : an);
        bk = fma(-l, uu2, sw ? 0.0 : bn);
    }
    if (fabs(ak) < tiny) ak = copysign(tiny, ak);
    u0[(size_t)(N - 1) * ld + t] = 1.0 / ak;
    for (int i = 0; i < N; i++) y[(size_t)i * ld + t] = ((whash(t * 2654435761u + 17u, i) >> 8) * (1.0 / 16777216.0)) * 2.0 - 1.0;
    double sc = 1.0;
    for (int it = 0; it < 4; it++) {
        // forward: interchanges and L; the operands of eight steps are loaded ahead of the dependent recurrence
        double c = y[t] * sc;
        int k = 0;
        for (; k + 8 <= N - 1; k += 8) {
            double xn[8], l[8]; bool sw[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                xn[u] = y[(size_t)(k + 1 + u) * ld + t] * sc; l[u] = lm[(size_t)(k + u) * ld + t]; sw[u] = pv[(size_t)(k + u) * ld + t];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const double yk = sw[u] ? xn[u] : c, cn = sw[u] ? c : xn[u];
                y[(size_t)(k + u) * ld + t] = yk;
                c = fma(-l[u], yk, cn);
            }
        }
        for (; k < N - 1; k++) {
            const double xn = y[(size_t)(k + 1) * ld + t] * sc, l = lm[(size_t)k * ld + t];
            const bool sw = pv[(size_t)k * ld + t];
            const double yk = sw ? xn : c, cn = sw ? c : xn;
            y[(size_t)k * ld + t] = yk;
            c = fma(-l, yk, cn);
        }
        // back substitution with U, eight rows loaded ahead
        double x1 = c * u0[(size_t)(N - 1) * ld + t], x2 = 0.0, mx = fabs(x1);
        y[(size_t)(N - 1) * ld + t] = x1;
        k = N - 2;
        for (; k - 7 >= 0; k -= 8) {
            double yy[8], a0[8], a1[8], a2[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const size_t o = (size_t)(k - u) * ld + t;
                yy[u] = y[o]; a0[u] = u0[o]; a1[u] = u1[o]; a2[u] = u2[o];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const double x0 = fma(-a2[u], x2, fma(-a1[u], x1, yy[u])) * a0[u];
                y[(size_t)(k - u) * ld + t] = x0; x2 = x1; x1 = x0; mx = fmax(mx, fabs(x0));
            }
        }
        for (; k >= 0; k--) {
            const size_t o = (size_t)k * ld + t;
            const double x0 = fma(-u2[o], x2, fma(-u1[o], x1, y[o])) * u0[o];
            y[o] = x0; x2 = x1; x1 = x0; mx = fmax(mx, fabs(x0));
        }
        sc = mx > 0.0 ? 1.0 / mx : 1.0;   // folded into the next forward pass
    }
    double nr = 0.0;
    for (int i = 0; i < N; i++) { const double v = y[(size_t)i * ld + t] * sc; nr = fma(v, v, nr); }
    const double s = sc / sqrt(nr);
    double *z = Zc + (size_t)t * N;
    for (int i = 0; i < N; i++) z[i] = y[(size_t)i * ld + t] * s;
}

// Gram-Schmidt inside every cluster of close eigenvalues, one block per cluster: each member in turn is
// orthogonalised against the cluster's earlier members by classical Gram-Schmidt done twice (the dots of a pass in
// parallel over the warps, then one combined update over the components) and normalised.  The span of a cluster's
// vectors is its invariant subspace to within the contamination from farther eigenvalues, and the density depends on
// the span only.  Blocks whose index is not a cluster start return at once.
__global__ void __launch_bounds__(WB) k_cluster_gs(int N, int nv, const int *__restrict__ cstart, double *__restrict__ Zc)
{
    extern __shared__ double dots[];   // one per earlier member
    __shared__ double red[32];
    const int c0 = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (c0 >= nv || cstart[c0] != c0) return;
    int c1 = c0 + 1;
    while (c1 < nv && cstart[c1] == c0) c1++;
    if (c1 - c0 < 2) return;
    for (int t = c0 + 1; t < c1; t++) {
        double *zt = Zc + (size_t)t * N;
        const int nq = t - c0;
        for (int pass = 0; pass < 2; pass++) {
            for (int q = w; q < nq; q += WW) {
                const double *zq = Zc + (size_t)(c0 + q) * N;
                double dt = 0.0;
                for (int i = lane; i < N; i += 32) dt = fma(zt[i], zq[i], dt);
                dt = warp_sum(dt);
                if (lane == 0) dots[q] = dt;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < N; i += WB) {
                double v = zt[i];
                for (int q = 0; q < nq; q++) v = fma(-dots[q], Zc[(size_t)(c0 + q) * N + i], v);
                zt[i] = v;
            }
            __syncthreads();
        }
        double nr = 0.0;
        for (int i = threadIdx.x; i < N; i += WB) nr = fma(zt[i], zt[i], nr);
        nr = block_sum(nr, red);
        const double sc = 1.0 / sqrt(nr);
        for (int i = threadIdx.x; i < N; i += WB) zt[i] *= sc;
        __syncthreads();
    }
}

// Cluster starts (one thread; nv <= N): cstart[t] = first index of t's cluster; returns the largest cluster size.
__global__ void k_clusters(int nv, const double *__restrict__ eig, double gap, int *__restrict__ cstart, int *__restrict__ maxsize)
{
    if (threadIdx.x || blockIdx.x) return;
    int s0 = 0, big = nv > 0 ? 1 : 0;
    for (int t = 0; t < nv; t++) {
        if (t > 0 && eig[t] - eig[t - 1] > gap) s0 = t;
        cstart[t] = s0;
        big = max(big, t - s0 + 1);
    }
    *maxsize = big;
}

// Back-transformation block: Vb (m x nb, column-major, unit diagonal at row j of column j, zeros above) from the
// reflectors stored in A below the subdiagonal of columns k0 .. k0 + nb - 1; rows counted from k0 + 1.
__global__ void __launch_bounds__(WB) k_vblock(int N, int k0, int nb, const double *__restrict__ A, double *__restrict__ Vb)
{
    const int m = N - k0 - 1;
    for (int e = blockIdx.x * WB + threadIdx.x; e < m * nb; e += gridDim.x * WB) {
        const int j = e / m, r = e % m;   // column j (reflector k0 + j), row r (matrix row k0 + 1 + r)
        double v = 0.0;
        if (r == j) v = 1.0;
        else if (r > j) v = A[(size_t)(k0 + 1 + r) * N + k0 + j];
        Vb[(size_t)j * m + r] = v;
    }
}

// T of the compact WY form I - V T V^T (upper triangular, dlarft 'Forward' 'Columnwise') from S = V^T V and tau: one
// block of WNB threads, column by column, thread i forming T[i][j] = -tau_j sum_{l=i}^{j-1} T[i][l] S[l][j] for i < j.
// T is written column-major (WNB x WNB, zeros below the diagonal), ready for DGEMM.
__global__ void __launch_bounds__(WNB) k_tblock(int nb, const double *__restrict__ S, const double *__restrict__ tau, int k0, double *__restrict__ T)
{
    __shared__ double Ts[WNB * WNB];   // row-major
    const int i = threadIdx.x;
    if (blockIdx.x) return;
    for (int e = i; e < WNB * WNB; e += WNB) Ts[e] = 0.0;
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        const double tj = tau[k0 + j];
        double s = 0.0;
        if (i < j)
            for (int l = i; l < j; l++) s = fma(Ts[i * WNB + l], S[j * nb + l], s);   // S column-major: S[l][j] = S[j * nb + l]
        __syncthreads();
        if (i < j) Ts[i * WNB + j] = -tj * s;
        if (i == j) Ts[j * WNB + j] = tj;
        __syncthreads();
    }
    for (int e = i; e < nb * nb; e += WNB) { const int r = e % nb, c = e / nb; T[e] = Ts[r * WNB + c]; }   // column-major, ld nb
}

// P = 2 C (occupied vectors) or 2 (1 - C) (virtual), C = Zc Zc^T; block partials of the squared change to part slot 6.
__global__ void __launch_bounds__(WB) k_density(int N, int occ, const double *__restrict__ C, double *__restrict__ P,
                                                double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    const size_t NN = (size_t)N * N;
    double r = 0.0;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) {
        const int i = (int)(k / N), j = (int)(k % N);
        const double v = C[(size_t)min(i, j) * N + max(i, j)];   // C symmetric; take one triangle for both entries
        const double pn = occ ? 2.0 * v : ((i == j ? 2.0 : 0.0) - 2.0 * v);
        const double dl = pn - P[k];
        r = fma(dl, dl, r);
        P[k] = pn;
    }
    r = block_reduce(r, red);
    if (threadIdx.x == 0) part[6 * parts + blockIdx.x] = r;
}

__global__ void k_control_density(Ctl *c, const double *__restrict__ part, int parts, int nb, int N)
{
    if (threadIdx.x >= 32 || blockIdx.x) return;
    const double r = warp_sum_parts(part + 6 * (size_t)parts, nb);
    if (threadIdx.x) return;
    c->rms = sqrt(r) / (double)N;
    c->valid = 1;
    c->have_z = 1;
}

// Uniform diagonal guess (QCOnePDM.c:326-331).
__global__ void __launch_bounds__(WB) k_guess(int N, double g, double *__restrict__ P)
{
    const size_t NN = (size_t)N * N;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) P[k] = (k / N == k % N) ? g : 0.0;
}

// Nuclear energy (pair terms in pair order) and the heat-of-formation baseline, one block.
__global__ void __launch_bounds__(WB) k_init_ctl(DeviceSystem s, const double *__restrict__ pair_e, int valid, int hist, int use_rca, Ctl *c)
{
    __shared__ double red[32];
    double en = 0.0;
    for (int p = threadIdx.x; p < s.n_pairs; p += WB) en += pair_e[(size_t)p * PDG_PAIR_E_STRIDE + 20];
    en = block_sum(en, red);
    double base = 0.0;
    for (int A = threadIdx.x; A < s.n_atoms; A += WB) { const double *E = elem(s, s.atom_elem[A]); base += E[PDG_E_EHEAT] - E[PDG_E_EISOL]; }
    base = block_sum(base, red);
    if (threadIdx.x == 0) {
        memset(c, 0, sizeof(Ctl));
        c->enuc = en; c->base = base; c->valid = valid; c->status = PDG_NOT_CONVERGED;
        c->qrca = use_rca ? 1 : 0;   // ODA (RCA) until the DIIS onset, as the reference starts (DIISSCFConverger.c:147)
        for (int i = 0; i < hist; i++) c->slots[i] = i;
    }
}

__global__ void k_finish(const Ctl *c, double *__restrict__ energies, int *__restrict__ status, int *__restrict__ ncycles)
{
    if (threadIdx.x || blockIdx.x) return;
    energies[0] = c->eel; energies[1] = c->e1 + c->e2; energies[2] = c->enuc; energies[3] = c->base; energies[4] = c->eq;
    energies[5] = c->e1; energies[6] = c->e2; energies[7] = c->rms;
    *status = c->status;
    if (ncycles) *ncycles = c->iteration;
}

// ---------------------------------------------------------------------------------------------------------------
// Mixed method (perturbative density steps; not in the reference).  FP32 elementwise helpers.
__global__ void __launch_bounds__(WB) k_f32_diff(size_t n, const double *__restrict__ a, const double *__restrict__ b, float *__restrict__ out)
{
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < n; k += (size_t)gridDim.x * WB) out[k] = (float)(a[k] - (b ? b[k] : 0.0));
}
__global__ void __launch_bounds__(WB) k_f32_sum(size_t n, const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out)
{
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < n; k += (size_t)gridDim.x * WB) out[k] = a[k] + b[k];
}
// Gi (nc x kv, column-major) = 1 / (lambda_a - mu_i); BL = wanted eigenvalues, then the complementary ones
__global__ void __launch_bounds__(WB) k_gaps(int kv, int nc, const double *__restrict__ BL, float *__restrict__ Gi)
{
    for (int e = blockIdx.x * WB + threadIdx.x; e < kv * nc; e += gridDim.x * WB) {
        const int a = e / nc, i = e % nc;
        Gi[e] = (float)(1.0 / (BL[a] - BL[kv + i]));
    }
}
// K2 = (E + R) o Gi; block maxima of |K2 - K| and |K2| to part slots 28, 29
__global__ void __launch_bounds__(WB) k_sweep(size_t n, const float *__restrict__ E, const float *__restrict__ R, const float *__restrict__ Gi,
                                              const float *__restrict__ K, float *__restrict__ K2, int first, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    float dm = 0.f, km = 0.f;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < n; k += (size_t)gridDim.x * WB) {
        const float kn = (E[k] + (first ? 0.f : R[k])) * Gi[k];
        dm = fmaxf(dm, fabsf(kn - (first ? 0.f : K[k]))); km = fmaxf(km, fabsf(kn));
        K2[k] = kn;
    }
    const double d = block_max((double)dm, red), m = block_max((double)km, red);
    if (threadIdx.x == 0) { part[28 * (size_t)parts + blockIdx.x] = d; part[29 * (size_t)parts + blockIdx.x] = m; }
}
__global__ void k_sweep_max(const double *__restrict__ part, int parts, int nb, double *__restrict__ out)
{
    if (threadIdx.x >= 32 || blockIdx.x) return;
    double d = 0.0, m = 0.0;
    for (int b = threadIdx.x; b < nb; b += 32) { d = fmax(d, part[28 * (size_t)parts + b]); m = fmax(m, part[29 * (size_t)parts + b]); }
    d = warp_max(d); m = warp_max(m);
    if (threadIdx.x == 0) { out[0] = d; out[1] = m; }
}
// y += alpha x (FP32)
__global__ void __launch_bounds__(WB) k_f32_axpy(size_t n, float alpha, const float *__restrict__ x, float *__restrict__ y)
{
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < n; k += (size_t)gridDim.x * WB) y[k] = fmaf(alpha, x[k], y[k]);
}
// P = P0 + c dQ (dQ column-major N x N, taken from one triangle for both entries); block partials of the squared change
__global__ void __launch_bounds__(WB) k_pert_density(int N, double c, const double *__restrict__ BP, const float *__restrict__ DQ,
                                                     double *__restrict__ P, double *__restrict__ part, int parts)
{
    __shared__ double red[32];
    const size_t NN = (size_t)N * N;
    double r = 0.0;
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < NN; k += (size_t)gridDim.x * WB) {
        const int i = (int)(k / N), j = (int)(k % N);
        const double v = (double)DQ[(size_t)min(i, j) * N + max(i, j)];
        const double pn = BP[k] + c * v;
        const double dl = pn - P[k];
        r = fma(dl, dl, r);
        P[k] = pn;
    }
    r = block_reduce(r, red);
    if (threadIdx.x == 0) part[6 * (size_t)parts + blockIdx.x] = r;
}
__global__ void __launch_bounds__(WB) k_copy(size_t n, const double *__restrict__ a, double *__restrict__ b)
{
    for (size_t k = (size_t)blockIdx.x * WB + threadIdx.x; k < n; k += (size_t)gridDim.x * WB) b[k] = a[k];
}
__global__ void k_set_have_z(Ctl *c, int v) { if (threadIdx.x == 0 && blockIdx.x == 0) c->have_z = v; }

}  // namespace wide

// =================================================================================================================
// Host side.
using namespace wide;

// Phases of the per-call device timing (pdg_wide_phase_times).
enum { WPH_INTEGRALS, WPH_FOCK, WPH_DIIS, WPH_TRIDIAGONAL, WPH_EIGENVALUES, WPH_EIGENVECTORS, WPH_BACKTRANSFORM, WPH_DENSITY,
       WPH_GRADIENTS, WPH_N };

struct pdg_wide {
    DeviceSystem s;
    WPlan w;
    // phase timing: events recorded on the stream in order, each closing the phase it is tagged with
    int timing = 0, n_marks = 0;
    std::vector<cudaEvent_t> events;
    std::vector<int> tags;
    float phase_ms[WPH_N] = {};
    int grid;                      // blocks of the grid-wide kernels (the SM count)
    cublasHandle_t blas = nullptr;
    cudaGraphExec_t tri = nullptr; // the tridiagonalisation (2 (N - 2) kernels), replayed every density step
    cudaStream_t tri_stream = nullptr;
    double *tri_ws = nullptr;      // workspace base the graph was captured on
    Ctl host;                      // last control record read back
    // mixed method: the base of the perturbative steps is valid for this workspace
    int base_ok = 0;
    double *base_ws = nullptr;
    double sweep[2];               // last perturbative sweep: max change of K, max |K|
    int pert_steps = 0, fp64_steps = 0;   // density steps of the last call
};

static int cublas_ok(cublasStatus_t st, const char *what);

size_t wide_workspace_bytes(const DeviceSystem &s) { return sizeof(double) * wide_plan(s).total; }
size_t wide_workspace_size(const pdg_wide *W) { return sizeof(double) * W->w.total; }

int wide_create(const DeviceSystem &s, pdg_wide **out)
{
    pdg_wide *W = new pdg_wide();
    W->s = s;
    W->w = wide_plan(s);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    W->grid = sms > 0 ? sms : 148;
    if (W->grid > W->w.parts) W->grid = W->w.parts;
    if (cublasCreate(&W->blas) != CUBLAS_STATUS_SUCCESS) { delete W; return PDG_CUDA_ERROR; }
    cublasSetMathMode(W->blas, CUBLAS_DEFAULT_MATH);
    *out = W;
    return PDG_OK;
}

static void mark(pdg_wide *W, cudaStream_t st, int phase)
{
    if (!W->timing || W->n_marks >= (int)W->events.size()) return;
    cudaEventRecord(W->events[W->n_marks], st);
    W->tags[W->n_marks++] = phase;
}

int wide_timing(pdg_wide *W, int enable)
{
    if (enable && W->events.empty()) {
        W->events.resize(4096);
        W->tags.resize(4096);
        for (cudaEvent_t &e : W->events)
            if (cudaEventCreate(&e) != cudaSuccess) return PDG_CUDA_ERROR;
    }
    W->timing = enable ? 1 : 0;
    return PDG_OK;
}

int wide_phase_times(pdg_wide *W, float *ms)
{
    for (int k = 0; k < WPH_N; k++) ms[k] = W->phase_ms[k];
    ms[WPH_N] = (float)W->fp64_steps;
    ms[WPH_N + 1] = (float)W->pert_steps;
    return PDG_OK;
}

// After a timed call: the device time between consecutive marks, summed per phase.
static void collect(pdg_wide *W)
{
    for (int k = 0; k < WPH_N; k++) W->phase_ms[k] = 0.0f;
    if (!W->timing || W->n_marks < 2) return;
    cudaEventSynchronize(W->events[W->n_marks - 1]);
    for (int k = 1; k < W->n_marks; k++) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, W->events[k - 1], W->events[k]) == cudaSuccess) W->phase_ms[W->tags[k]] += t;
    }
}

void wide_destroy(pdg_wide *W)
{
    if (!W) return;
    for (cudaEvent_t e : W->events)
        if (e) cudaEventDestroy(e);
    if (W->tri) cudaGraphExecDestroy(W->tri);
    if (W->blas) cublasDestroy(W->blas);
    delete W;
}

// C (m x n, column-major, ld m) = op(A) op(B) + beta C with FP64 GEMM on the given stream.
static cublasStatus_t dgemm(pdg_wide *W, cudaStream_t st, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                            double alpha, const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc)
{
    cublasSetStream(W->blas, st);
    return cublasDgemm(W->blas, ta, tb, m, n, k, &alpha, A, lda, B, ldb, &beta, C, ldc);
}

static cublasStatus_t sgemm(pdg_wide *W, cudaStream_t st, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                            float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
    cublasSetStream(W->blas, st);
    return cublasSgemm(W->blas, ta, tb, m, n, k, &alpha, A, lda, B, ldb, &beta, C, ldc);
}

// The tridiagonalisation of A (plan regions of this workspace) as one CUDA graph, captured on first use.
static int tri_graph(pdg_wide *W, double *ws, cudaStream_t st)
{
    const int N = W->s.n_basis;
    if (W->tri && W->tri_ws == ws) return PDG_OK;
    if (W->tri) { cudaGraphExecDestroy(W->tri); W->tri = nullptr; }
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return PDG_CUDA_ERROR;
    const WPlan &p = W->w;
    double *A = ws + p.A, *colbuf = ws + p.colbuf, *vbuf = ws + p.vbuf, *q = ws + p.q, *tpart = ws + p.tpart;
    double *d = ws + p.d, *e = ws + p.e, *tau = ws + p.tau;
    const size_t sm_step = 4 * sizeof(double) * (size_t)N, sm_last = 2 * sizeof(double) * (size_t)N;
    cudaFuncSetAttribute(k_tri_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_step);
    cudaFuncSetAttribute(k_tri_last, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_last);
    cudaGraph_t g;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    for (int k = 0; k + 2 < N; k++)
        k_tri_step<<<W->grid, WB, sm_step, cap>>>(N, k, A, colbuf, vbuf, q, d, e, tau, tpart, p.parts, W->grid);
    k_tri_last<<<1, WB, sm_last, cap>>>(N, A, colbuf, vbuf, q, d, e, tau, tpart, p.parts, W->grid);
    cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (ce != cudaSuccess) return PDG_CUDA_ERROR;
    ce = cudaGraphInstantiate(&W->tri, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) { W->tri = nullptr; return PDG_CUDA_ERROR; }
    W->tri_ws = ws;
    return PDG_OK;
}

// Eigenpairs [first, first + nv) of the tridiagonal T in d, e (eigenvalues to eig_out): bisection, inverse iteration with
// cluster re-orthogonalisation, and the blocked back-transformation by the reflectors stored in A; the vectors end as the
// columns of Zout (N x nv, column-major).  tn: the Gershgorin bound of T.
static int wide_eigenvectors(pdg_wide *W, double *ws, int first, int nv, double *Zout, double *eig_out, double tn, cudaStream_t st)
{
    const WPlan &p = W->w;
    const int N = W->s.n_basis, G = W->grid;
    double *A = ws + p.A;
    k_bisect<<<(nv + MS_WARPS - 1) / MS_WARPS, 32 * MS_WARPS, 0, st>>>(N, first, nv, ws + p.d, ws + p.e, eig_out);
    mark(W, st, WPH_EIGENVALUES);
    // Inverse iteration at an eigenvalue converged to round-off leaves a vector's overlap with another eigenvector at
    // about eps ||T|| / gap: below 3e-10 for gaps above 1e-6 ||T||, so only closer eigenvalues form clusters, whose
    // vectors are orthonormalised after the iteration.
    int *cstart = (int *)(ws + p.cst), *maxsize = cstart + N;
    k_clusters<<<1, 1, 0, st>>>(nv, eig_out, 1.0e-6 * tn, cstart, maxsize);
    double *lu = ws + p.lu;
    unsigned char *pv = (unsigned char *)(lu + 5 * (size_t)N * p.kvp);
    k_invit<<<(nv + 31) / 32, 32, 0, st>>>(N, nv, p.kvp, ws + p.d, ws + p.e, eig_out, tn, lu, pv, ws + p.y, Zout);
    k_cluster_gs<<<nv, WB, sizeof(double) * (size_t)nv, st>>>(N, nv, cstart, Zout);
    mark(W, st, WPH_EIGENVECTORS);
    // back-transformation Zout <- Q Zout, blocks of WNB reflectors from the last to the first
    const int nref = N - 2;
    for (int k0 = ((nref - 1) / WNB) * WNB; k0 >= 0 && nref > 0; k0 -= WNB) {
        const int nb = min(WNB, nref - k0), m = N - k0 - 1;
        double *Vb = ws + p.vb, *S = ws + p.sb, *T = ws + p.tb, *Wm = ws + p.wb;
        k_vblock<<<G, WB, 0, st>>>(N, k0, nb, A, Vb);
        if (dgemm(W, st, CUBLAS_OP_T, CUBLAS_OP_N, nb, nb, m, 1.0, Vb, m, Vb, m, 0.0, S, nb) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
        k_tblock<<<1, WNB, 0, st>>>(nb, S, ws + p.tau, k0, T);
        double *W2 = Wm + (size_t)WNB * N;
        for (int c0 = 0; c0 < nv; c0 += N) {   // the W buffers hold WNB x N: columns in chunks of N
            const int nvc = min(N, nv - c0);
            if (dgemm(W, st, CUBLAS_OP_T, CUBLAS_OP_N, nb, nvc, m, 1.0, Vb, m, Zout + (size_t)c0 * N + k0 + 1, N, 0.0, Wm, nb) != CUBLAS_STATUS_SUCCESS ||
                dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_N, nb, nvc, nb, 1.0, T, nb, Wm, nb, 0.0, W2, nb) != CUBLAS_STATUS_SUCCESS ||
                dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_N, m, nvc, nb, -1.0, Vb, m, W2, nb, 1.0, Zout + (size_t)c0 * N + k0 + 1, N) != CUBLAS_STATUS_SUCCESS)
                return PDG_CUDA_ERROR;
        }
    }
    mark(W, st, WPH_BACKTRANSFORM);
    return cudaGetLastError() == cudaSuccess ? PDG_OK : PDG_CUDA_ERROR;
}

// One FP64 density step: P <- density of the wanted eigenvectors of F; the vectors stay in Zc for the DIIS save.  With
// make_base (the mixed method) it also keeps the base of the following perturbative steps: F0 = F, P0 = P, the wanted
// vectors in FP32, the complementary eigenpairs (from the same tridiagonal form, vectors rounded to FP32) and the
// reciprocal gaps.
static int wide_density_step(pdg_wide *W, double *ws, double *P, cudaStream_t st, bool make_base)
{
    const DeviceSystem &s = W->s;
    const WPlan &p = W->w;
    const int N = s.n_basis, kv = s.n_vec, nc = N - kv, G = W->grid;
    double *F = ws + p.F, *A = ws + p.A, *C = ws + p.C, *Zc = ws + p.Zc, *part = ws + p.part;
    k_tri_start<<<G, WB, 0, st>>>(N, F, A, ws + p.colbuf);
    int rc = tri_graph(W, ws, st);
    if (rc) return rc;
    if (cudaGraphLaunch(W->tri, st) != cudaSuccess) return PDG_CUDA_ERROR;
    mark(W, st, WPH_TRIDIAGONAL);
    double bounds[2];
    {
        // Gershgorin bound of T, for the cluster gap and the pivot floor
        std::vector<double> hd(N), he(N);
        if (cudaMemcpyAsync(hd.data(), ws + p.d, sizeof(double) * N, cudaMemcpyDeviceToHost, st) != cudaSuccess) return PDG_CUDA_ERROR;
        if (cudaMemcpyAsync(he.data(), ws + p.e, sizeof(double) * N, cudaMemcpyDeviceToHost, st) != cudaSuccess) return PDG_CUDA_ERROR;
        if (cudaStreamSynchronize(st) != cudaSuccess) return PDG_CUDA_ERROR;
        double lo = 1e300, hi = -1e300;
        for (int i = 0; i < N; i++) {
            const double r = (i > 0 ? fabs(he[i - 1]) : 0.0) + (i < N - 1 ? fabs(he[i]) : 0.0);
            lo = fmin(lo, hd[i] - r); hi = fmax(hi, hd[i] + r);
        }
        bounds[0] = lo; bounds[1] = hi;
    }
    const double tn = fmax(fabs(bounds[0]), fabs(bounds[1]));
    // the wanted eigenpairs: the lowest n_occ (occupied) or the highest N - n_occ (virtual)
    if ((rc = wide_eigenvectors(W, ws, s.vec_occupied ? 0 : N - kv, kv, Zc, ws + p.eig, tn, st))) return rc;
    // C = Zc Zc^T (column-major N x N: symmetric, so also row-major), P from it
    if (dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_T, N, N, kv, 1.0, Zc, N, Zc, N, 0.0, C, N) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
    k_density<<<G, WB, 0, st>>>(N, s.vec_occupied, C, P, part, p.parts);
    k_control_density<<<1, 32, 0, st>>>((Ctl *)(ws + p.ctl), part, p.parts, G, N);
    mark(W, st, WPH_DENSITY);
    if (make_base && nc > 0) {
        float *f32 = (float *)(ws + p.f32);
        const size_t NN = (size_t)N * N;
        k_copy<<<G, WB, 0, st>>>(NN, F, ws + p.BF);
        k_copy<<<G, WB, 0, st>>>(NN, P, ws + p.BP);
        k_copy<<<1, WB, 0, st>>>((size_t)kv, ws + p.eig, ws + p.BL);
        k_f32_diff<<<G, WB, 0, st>>>((size_t)N * kv, Zc, nullptr, f32 + p.ZY);
        if ((rc = wide_eigenvectors(W, ws, s.vec_occupied ? kv : 0, nc, ws + p.Zcc, ws + p.BL + kv, tn, st))) return rc;
        k_f32_diff<<<G, WB, 0, st>>>((size_t)N * nc, ws + p.Zcc, nullptr, f32 + p.V32);
        k_gaps<<<G, WB, 0, st>>>(kv, nc, ws + p.BL, f32 + p.Gi);
        W->base_ok = 1;
        W->base_ws = ws;
        mark(W, st, WPH_DENSITY);
    }
    return cudaGetLastError() == cudaSuccess ? PDG_OK : PDG_CUDA_ERROR;
}

// Perturbative density step around the base (the device counterpart of scf.cu's density_step_pert, every product a
// cuBLAS SGEMM): for F = F0 + dF, the wanted invariant subspace is spanned by the columns of Z0 + V K, K (nc x kv)
// solving E + M' K - K L' - K E^T K = (lambda_a - mu_i) K_ia with E = V^T dF Z0, L' = Z0^T dF Z0, M' = V^T dF V (fixed-
// point sweeps from K = E / (lambda - mu)); the new projector differs from Z0 Z0^T by dQ = Z0 W^T + Y (Z0 + W)^T, Y = V K,
// U = (1 + K^T K)^-1 - 1 = -A + A^2 - A^3 (A = K^T K), W = Y + (Z0 + Y) U; P = P0 + 2 dQ (occupied) or P0 - 2 dQ.  Every FP32
// product has a small factor (dF, K, Y, W).  Returns 1 when it produced P, 0 when the base does not carry the step (the
// sweeps do not settle or |K| >= 3e-2: the caller runs an FP64 step, which makes a new base).
static int wide_pert_step(pdg_wide *W, double *ws, double *P, cudaStream_t st, int *done)
{
    const DeviceSystem &s = W->s;
    const WPlan &p = W->w;
    const int N = s.n_basis, kv = s.n_vec, nc = N - kv, G = W->grid;
    const size_t NN = (size_t)N * N;
    float *f = (float *)(ws + p.f32);
    float *D = f + p.D, *Z0 = f + p.ZY, *Yc = f + p.ZY + (size_t)N * kv, *V = f + p.V32, *Gi = f + p.Gi, *T1 = f + p.T1, *E = f + p.E;
    float *Lp = f + p.Lp, *T2 = f + p.T2, *Mp = f + p.Mp, *K = f + p.K, *K2 = f + p.K2, *R = f + p.R, *EK = f + p.EK, *Am = f + p.Am;
    float *U = f + p.U, *Sm = f + p.Sm, *Wc = f + p.WZ2, *WZ = f + p.WZ2 + (size_t)N * kv, *DQ = f + p.DQ;
    double *part = ws + p.part, *mx = ws + p.part + 30 * (size_t)p.parts;
    const cublasOperation_t Nn = CUBLAS_OP_N, Tt = CUBLAS_OP_T;
    *done = 0;
    if (nc <= 0) return PDG_OK;
    k_f32_diff<<<G, WB, 0, st>>>(NN, ws + p.F, ws + p.BF, D);
    if (sgemm(W, st, Nn, Nn, N, kv, N, 1.f, D, N, Z0, N, 0.f, T1, N) ||                 // T1 = dF Z0
        sgemm(W, st, Tt, Nn, nc, kv, N, 1.f, V, N, T1, N, 0.f, E, nc) ||                // E = V^T T1
        sgemm(W, st, Tt, Nn, kv, kv, N, 1.f, Z0, N, T1, N, 0.f, Lp, kv) ||              // L' = Z0^T T1
        sgemm(W, st, Nn, Nn, N, nc, N, 1.f, D, N, V, N, 0.f, T2, N) ||                  // T2 = dF V
        sgemm(W, st, Tt, Nn, nc, nc, N, 1.f, V, N, T2, N, 0.f, Mp, nc))                 // M' = V^T T2
        return PDG_CUDA_ERROR;
    k_sweep<<<G, WB, 0, st>>>((size_t)nc * kv, E, R, Gi, K, K, 1, part, p.parts);     // K = E / (lambda - mu)
    bool settled = false;
    double kmax = 0.0;
    for (int it = 0; it < 12 && !settled; it++) {
        if (sgemm(W, st, Tt, Nn, kv, kv, nc, 1.f, E, nc, K, nc, 0.f, EK, kv)) return PDG_CUDA_ERROR;   // E^T K
        k_f32_axpy<<<1, WB, 0, st>>>((size_t)kv * kv, 1.f, Lp, EK);                                      // L' + E^T K
        if (sgemm(W, st, Nn, Nn, nc, kv, nc, 1.f, Mp, nc, K, nc, 0.f, R, nc) ||                          // M' K
            sgemm(W, st, Nn, Nn, nc, kv, kv, -1.f, K, nc, EK, kv, 1.f, R, nc))                           // - K (L' + E^T K)
            return PDG_CUDA_ERROR;
        k_sweep<<<G, WB, 0, st>>>((size_t)nc * kv, E, R, Gi, K, K2, 0, part, p.parts);
        k_sweep_max<<<1, 32, 0, st>>>(part, p.parts, G, mx);
        if (cudaMemcpyAsync(W->sweep, mx, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PDG_CUDA_ERROR;
        if (cudaStreamSynchronize(st) != cudaSuccess) return PDG_CUDA_ERROR;
        float *tmp = K; K = K2; K2 = tmp;
        kmax = W->sweep[1];
        settled = W->sweep[0] <= 1.0e-5 * W->sweep[1] + 1.0e-30;
    }
    // |K| bounds the FP32 rounding carried into P (~1e-7 |K| per product) and the error of U = -A + A^2 - A^3 (|K|^8):
    // 3e-2 keeps both below the 1e-8 tolerance (3e-9 and 7e-13), and lets the base carry several MD steps
    if (!settled || !(kmax < 3.0e-2)) return PDG_OK;
    if (sgemm(W, st, Nn, Nn, N, kv, nc, 1.f, V, N, K, nc, 0.f, Yc, N) ||               // Y = V K
        sgemm(W, st, Tt, Nn, kv, kv, nc, 1.f, K, nc, K, nc, 0.f, Am, kv) ||            // A = K^T K
        sgemm(W, st, Nn, Nn, kv, kv, kv, 1.f, Am, kv, Am, kv, 0.f, EK, kv) ||           // A^2
        sgemm(W, st, Nn, Nn, kv, kv, kv, -1.f, Am, kv, EK, kv, 0.f, U, kv))            // -A^3
        return PDG_CUDA_ERROR;
    k_f32_axpy<<<1, WB, 0, st>>>((size_t)kv * kv, 1.f, EK, U);                           // A^2 - A^3
    k_f32_axpy<<<1, WB, 0, st>>>((size_t)kv * kv, -1.f, Am, U);                          // U = -A + A^2 - A^3
    k_f32_sum<<<G, WB, 0, st>>>((size_t)N * kv, Z0, Yc, Sm);                             // S = Z0 + Y
    if (cudaMemcpyAsync(Wc, Yc, sizeof(float) * (size_t)N * kv, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return PDG_CUDA_ERROR;
    if (sgemm(W, st, Nn, Nn, N, kv, kv, 1.f, Sm, N, U, kv, 1.f, Wc, N)) return PDG_CUDA_ERROR;   // W = Y + S U
    k_f32_sum<<<G, WB, 0, st>>>((size_t)N * kv, Z0, Wc, WZ);                                       // Z0 + W
    // dQ = [Z0 | Y] [W | Z0 + W]^T
    if (sgemm(W, st, Nn, Tt, N, N, 2 * kv, 1.f, Z0, N, Wc, N, 0.f, DQ, N)) return PDG_CUDA_ERROR;
    k_pert_density<<<G, WB, 0, st>>>(N, s.vec_occupied ? 2.0 : -2.0, ws + p.BP, DQ, P, part, p.parts);
    k_control_density<<<1, 32, 0, st>>>((Ctl *)(ws + p.ctl), part, p.parts, G, N);
    mark(W, st, WPH_DENSITY);
    *done = 1;
    return cudaGetLastError() == cudaSuccess ? PDG_OK : PDG_CUDA_ERROR;
}

int wide_energy_gradients(pdg_wide *W, const double *xyz, const double *phi, const pdg_scf_options &o, double *P, int use_density,
                          double *energies, double *gradients, double *charges, int *status, int *ncycles, double *ws, cudaStream_t st)
{
    const DeviceSystem &s = W->s;
    const WPlan &p = W->w;
    const int N = s.n_basis, G = W->grid, hist = o.history;
    const size_t NN = (size_t)N * N;
    Ctl *ctl = (Ctl *)(ws + p.ctl);
    double *F = ws + p.F, *H = ws + p.fp.H, *part = ws + p.part, *C = ws + p.C;
    W->n_marks = 0;
    mark(W, st, WPH_INTEGRALS);
    // integrals (the frame kernels of integrals.cu on this one frame)
    launch_pair_integrals(s, p.fp, 1, xyz, ws, st);
    launch_assemble_h(s, p.fp, 1, ws, st);
    if (!use_density) k_guess<<<G, WB, 0, st>>>(N, (double)s.n_electrons / (double)N, P);
    k_init_ctl<<<1, WB, 0, st>>>(s, ws + p.fp.pair_e, use_density ? 1 : 0, hist, o.use_rca, ctl);
    if (cudaGetLastError() != cudaSuccess) return PDG_CUDA_ERROR;
    mark(W, st, WPH_INTEGRALS);
    const int nb_tr = G;
    const bool mixed = o.density_step != 0;
    bool have_ft = false;   // F~ of the last density step is in the workspace (mixed method)
    W->pert_steps = W->fp64_steps = 0;
    for (int cycle = 0; cycle <= o.maximum_scf_cycles; cycle++) {
        // Fock build, energies, convergence test
        k_pk<<<G, WB, 0, st>>>(s, P, ws + p.pk);
        k_fock<<<G * 4, WB, 0, st>>>(s, H, P, ws + p.fp.tei, ws + p.pk, F);
        k_traces<<<nb_tr, WB, 0, st>>>(N, P, H, F, part, p.parts);
        k_lowdin<<<1, WB, 0, st>>>(s, P, phi, F, charges, part, p.parts);
        k_control_fock<<<1, 32, 0, st>>>(ctl, part, p.parts, nb_tr, o, hist);
        mark(W, st, WPH_FOCK);
        if (cudaMemcpyAsync(&W->host, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PDG_CUDA_ERROR;
        if (cudaStreamSynchronize(st) != cudaSuccess) return PDG_CUDA_ERROR;
        if (W->host.done || W->host.iteration >= o.maximum_scf_cycles) break;
        // DIIS save: history, error vector e = F P - P F, B-matrix row
        if (W->host.valid) {
            k_pack<<<G, WB, 0, st>>>(NN, ctl, P, F, ws + p.hP, ws + p.hF);
            double sg = 1.0;
            if (have_ft) {
                // mixed method: P is the projector of F~ (the matrix its density step was applied to), so F P - P F =
                // dF P - P dF with dF = F - F~, small once the SCF settles: its FP32 product carries ~1e-7 |dF|
                float *f32 = (float *)(ws + p.f32);
                k_f32_diff<<<G, WB, 0, st>>>(NN, F, ws + p.Ft, f32 + p.D);
                k_f32_diff<<<G, WB, 0, st>>>(NN, P, nullptr, f32 + p.P32);
                if (sgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, 1.f, f32 + p.D, N, f32 + p.P32, N, 0.f, f32 + p.DQ, N) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
                k_error<float><<<G, WB, 0, st>>>(N, ctl, f32 + p.DQ, -1.0, ws + p.hE, part, p.parts);
            } else if (W->host.have_z) {
                // P = 2 Zc Zc^T (or 2 (1 - Zc Zc^T)): F P - P F = sg (G Zc^T - Zc G^T), G = F Zc
                if (dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_N, N, s.n_vec, N, 1.0, F, N, ws + p.Zc, N, 0.0, ws + p.G, N) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
                // C (column-major) = G Zc^T, i.e. row-major C^T: the error kernel reads C_ij - C_ji, so the sign flips
                if (dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_T, N, N, s.n_vec, 1.0, ws + p.G, N, ws + p.Zc, N, 0.0, C, N) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
                sg = s.vec_occupied ? -2.0 : 2.0;
            } else {
                // C (column-major) = F P, row-major (F P)^T = P F: e = FP - PF = C^T - C, read as -(C_ij - C_ji)
                if (dgemm(W, st, CUBLAS_OP_N, CUBLAS_OP_N, N, N, N, 1.0, F, N, P, N, 0.0, C, N) != CUBLAS_STATUS_SUCCESS) return PDG_CUDA_ERROR;
                sg = -1.0;
            }
            if (!have_ft) k_error<double><<<G, WB, 0, st>>>(N, ctl, C, sg, ws + p.hE, part, p.parts);
            k_dots<<<G, WB, 0, st>>>(N, ctl, ws + p.hE, part, p.parts);
            if (o.use_rca) k_oda_traces<<<G, WB, 0, st>>>(NN, F, P, ws + p.rF, ws + p.rP, part, p.parts);
            k_control_diis<<<1, 32, 0, st>>>(ctl, part, p.parts, G, G, o, hist);
            k_iterate<<<G, WB, 0, st>>>(NN, ctl, ws + p.hP, ws + p.hF, P, F, ws + p.rP, ws + p.rF, o.use_rca);
        } else {
            // no valid density yet (the diagonal guess): nothing to save; the reference does not count this cycle
            k_control_diis<<<1, 32, 0, st>>>(ctl, part, p.parts, 0, 0, o, hist);
        }
        mark(W, st, WPH_DIIS);
        int rc;
        if (mixed) {
            k_copy<<<G, WB, 0, st>>>(NN, F, ws + p.Ft);
            int done = 0;
            if (W->base_ok && W->base_ws == ws && (rc = wide_pert_step(W, ws, P, st, &done))) return rc;
            if (!done && (rc = wide_density_step(W, ws, P, st, true))) return rc;
            have_ft = true;
            if (done) W->pert_steps++; else W->fp64_steps++;
        } else {
            if ((rc = wide_density_step(W, ws, P, st, false))) return rc;
            W->fp64_steps++;
        }
    }
    k_finish<<<1, 1, 0, st>>>(ctl, energies, status, ncycles);
    if (gradients) {
        // the mixed method takes the sp-sp and sp-s pair gradient terms in FP32 (assembled and summed in FP64)
        launch_pair_gradients(s, p.fp, 1, xyz, P, ws, st, mixed);
        launch_reduce_gradients(s, p.fp, 1, ws, gradients, st);
    }
    mark(W, st, WPH_GRADIENTS);
    if (cudaGetLastError() != cudaSuccess) return PDG_CUDA_ERROR;
    collect(W);
    return PDG_OK;
}
