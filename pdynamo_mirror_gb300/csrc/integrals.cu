// integrals.cu - per-atom-pair integral and gradient kernels (FP64).
//
// k_pair_integrals   one warp per (frame, atom pair i > j): local-frame multipole TEIs and electron-core
//                    terms (multipole.cuh), rotation to the molecular frame, STO-6G overlap -> resonance
//                    block of H, core-core energy.  Replaces the pair body of QCModelMNDO_Integrals
//                    (QCModelMNDO.c:1062-1112) with MNDOIntegrals_MolecularFrame2CIntegrals (MNDOIntegrals.c:147).
// k_assemble_h       one warp per (frame, atom): diagonal blocks of H = U + sum of electron-core terms.
// k_pair_gradients   one warp per (frame, atom pair): dE/dR of the pair (QCModelMNDO_Gradients,
//                    QCModelMNDO.c:732-840 with MNDOIntegrals_MolecularFrame2CIntegralsD, MNDOIntegrals.c:274,
//                    and QCModelMNDOState_GetGradientDensityTerms, QCModelMNDOState.c:178).
// k_reduce_gradients one warp per (frame, atom): sums the pair terms in a fixed order (deterministic).
#include "common.cuh"
#include "multipole.cuh"

#define PI_D 3.14159265358979323846
#define EXPONENT_TOLERANCE 25.0
#define PRIMITIVE_OVERLAP_TOLERANCE (2.30258509299405 * 18.0)

// Core-core repulsion and d/dr, non-diatomic branch (MNDOIntegralUtilities.c:35-150, :152-281).
__device__ double core_core(const double *a, const double *b, double r, double *dedr)
{
    const double B2A = PDG_BOHRS_TO_ANGSTROMS;
    int za = (int)a[PDG_E_Z], zb = (int)b[PDG_E_Z];
    double s8 = a[PDG_E_PO + 8] + b[PDG_E_PO + 8];
    double gam = rsqrt(r * r + s8 * s8), dgdr = -r * gam * gam * gam;
    double alpa = a[PDG_E_ALP], alpb = b[PDG_E_ALP];
    double exi = exp(-alpa * r), exj = exp(-alpb * r);
    double scale = exi + exj;
    int nt = za + zb;
    if (nt == 8 || nt == 9) {
        if (za == 7 || za == 8) scale += (B2A * r - 1.0) * exi;
        if (zb == 7 || zb == 8) scale += (B2A * r - 1.0) * exj;
    }
    double zz = a[PDG_E_ZCORE] * b[PDG_E_ZCORE];
    double enuc = zz * gam;
    scale = fabs(scale * enuc);
    double dd;
    if (za == 1 && (zb == 7 || zb == 8)) {
        dd = dgdr * (1.0 + exi + B2A * r * exj) - gam * (alpa * exi + B2A * (alpb * r - 1.0) * exj);
    } else if ((za == 7 || za == 8) && zb == 1) {
        dd = dgdr * (1.0 + exj + B2A * r * exi) - gam * (alpb * exj + B2A * (alpa * r - 1.0) * exi);
    } else {
        dd = dgdr * (1.0 + exi + exj) - gam * (alpa * exi + alpb * exj);
    }
    double de = zz * dd, an = 0.0, gg = a[PDG_E_GPHOT] * b[PDG_E_GPHOT];
    for (int t = 0; t < 2; t++) {
        const double *e = t ? b : a;
        int ng = (int)e[PDG_E_NG];
        for (int i = 0; i < ng; i++) {
            double d = r - e[PDG_E_FN3 + i], ax = e[PDG_E_FN2 + i] * d * d;
            if (ax <= EXPONENT_TOLERANCE) {
                double ex = exp(-ax);
                scale += gg * zz / r * e[PDG_E_FN1 + i] * ex;
                an += e[PDG_E_FN1 + i] * (1.0 / (r * r) + e[PDG_E_FN2 + i] * 2.0 * d / r) * ex;
            }
        }
    }
    de -= an * gg * zz;
    int npa = (int)a[PDG_E_NPDDG], npb = (int)b[PDG_E_NPDDG];
    if (npa > 0 && npb > 0) {
        const double PDDG_EXPONENT = 10.0 * B2A * B2A;
        double zaf = a[PDG_E_ZCORE] / (a[PDG_E_ZCORE] + b[PDG_E_ZCORE]), zbf = b[PDG_E_ZCORE] / (a[PDG_E_ZCORE] + b[PDG_E_ZCORE]), ap = 0.0;
        for (int i = 0; i < npa; i++)
            for (int j = 0; j < npb; j++) {
                double d = r - a[PDG_E_PDDGE + i] - b[PDG_E_PDDGE + j], ex = exp(-PDDG_EXPONENT * d * d);
                double c = zaf * a[PDG_E_PDDGC + i] + zbf * b[PDG_E_PDDGC + j];
                scale += c * ex;
                ap += c * 2.0 * PDDG_EXPONENT * d * ex;
            }
        de -= ap;
    }
    if (dedr) *dedr = de;
    return enuc + scale;
}

// STO-6G overlap of the shells of atoms i and j (orbital order s, pz, px, py) and, optionally, its
// derivative with respect to atom i (GaussianBasis_2Overlap / _2OverlapD, GaussianBasisCore.c:469,570).
// Each lane takes every 32nd primitive pair; results are warp-reduced into S[16] and SD[48].
__device__ void pair_overlap(const double *Ei, const double *Ej, double abx, double aby, double abz,
                             bool derivs, int lane, double *S, double *SD)
{
    const int ORB[3] = { 2, 3, 1 };
    double s[16], sd[48];
    for (int k = 0; k < 16; k++) s[k] = 0.0;
    if (derivs) for (int k = 0; k < 48; k++) sd[k] = 0.0;
    double AB[3] = { abx, aby, abz }, R2 = abx * abx + aby * aby + abz * abz;
    int nsi = (int)Ei[PDG_E_NSHELL], nsj = (int)Ej[PDG_E_NSHELL];
    int npi[2] = { (int)Ei[PDG_E_NPRIM_S], (int)Ei[PDG_E_NPRIM_P] }, npj[2] = { (int)Ej[PDG_E_NPRIM_S], (int)Ej[PDG_E_NPRIM_P] };
    int base = 0;
    for (int sa = 0; sa < nsi; sa++)
        for (int sb = 0; sb < nsj; sb++) {
            int n = npi[sa] * npj[sb];
            for (int t = lane - base % 32 < 0 ? lane - base % 32 + 32 : lane - base % 32; t < n; t += 32) {
                int p = t / npj[sb], q = t % npj[sb];
                double a = Ei[(sa ? PDG_E_EXP_P : PDG_E_EXP_S) + p], b = Ej[(sb ? PDG_E_EXP_P : PDG_E_EXP_S) + q], g = a + b;
                double fac = a * b * R2 / g;
                if (fac > PRIMITIVE_OVERLAP_TOLERANCE) continue;
                double tg = PI_D / g;
                double s0 = Ei[(sa ? PDG_E_CCBF_P : PDG_E_CCBF_S) + p] * Ej[(sb ? PDG_E_CCBF_P : PDG_E_CCBF_S) + q] * tg * sqrt(tg) * exp(-fac);
                double PA[3], PB[3], h = 0.5 / g;
                for (int k = 0; k < 3; k++) { PA[k] = b / g * AB[k]; PB[k] = -a / g * AB[k]; }
                if (sa == 0 && sb == 0) {
                    s[0] += s0;
                    if (derivs) for (int k = 0; k < 3; k++) sd[k * 16] += 2.0 * a * PA[k] * s0;
                } else if (sa == 1 && sb == 0) {
                    for (int i = 0; i < 3; i++) {
                        s[ORB[i] * 4] += PA[i] * s0;
                        if (derivs) for (int k = 0; k < 3; k++) sd[k * 16 + ORB[i] * 4] += (2.0 * a * (PA[i] * PA[k] + (i == k) * h) - (i == k)) * s0;
                    }
                } else if (sa == 0 && sb == 1) {
                    for (int j = 0; j < 3; j++) {
                        s[ORB[j]] += PB[j] * s0;
                        if (derivs) for (int k = 0; k < 3; k++) sd[k * 16 + ORB[j]] += 2.0 * a * (PA[k] * PB[j] + (k == j) * h) * s0;
                    }
                } else {
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++) {
                            s[ORB[i] * 4 + ORB[j]] += (PA[i] * PB[j] + (i == j) * h) * s0;
                            if (derivs)
                                for (int k = 0; k < 3; k++) {
                                    double dpp = PA[i] * PA[k] * PB[j] + ((i == k) * PB[j] + (i == j) * PA[k] + (k == j) * PA[i]) * h;
                                    sd[k * 16 + ORB[i] * 4 + ORB[j]] += (2.0 * a * dpp - (i == k) * PB[j]) * s0;
                                }
                        }
                }
            }
            base += n;
        }
    for (int k = 0; k < 16; k++) S[k] = warp_sum(s[k]);
    if (derivs) for (int k = 0; k < 48; k++) SD[k] = warp_sum(sd[k]);
}

// Warp-private shared scratch (doubles).
#define PI_WARPS 8
#define PI_SM 640

__global__ void __launch_bounds__(PI_WARPS * 32)
k_pair_integrals(DeviceSystem s, FramePlan plan, int n_frames, const double *__restrict__ xyz,
                 const double *__restrict__ terms, double *__restrict__ ws)
{
    __shared__ double smem[PI_WARPS][PI_SM];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long gw = (long)blockIdx.x * PI_WARPS + w;
    if (gw >= (long)n_frames * s.n_pairs) return;
    int f = (int)(gw / s.n_pairs), p = (int)(gw % s.n_pairs);
    double *W = smem[w];
    double *St = W, *L = W + 96, *ci = W + 196, *cj = W + 206, *X = W + 216, *C = W + 316, *Y = W + 416;
    int i = s.pair_i[p], j = s.pair_j[p];
    int eli = s.atom_elem[i], elj = s.atom_elem[j];
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    int noi = s.atom_norb[i], noj = s.atom_norb[j];
    int ni = noi * (noi + 1) / 2, nj = noj * (noj + 1) / 2;
    bool spi = noi > 1, spj = noj > 1;
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    double x = R[3 * j] - R[3 * i], y = R[3 * j + 1] - R[3 * i + 1], z = R[3 * j + 2] - R[3 * i + 2];
    double r = sqrt(x * x + y * y + z * z);
    double *wsf = ws + (size_t)f * plan.stride;

    const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
    for (int k = lane; k < MP_TERMS_USED; k += 32) {
        double a = ta[k];
        St[k] = (a < 0.0) ? 0.0 : rsqrt((r + to[k]) * (r + to[k]) + a);
    }
    for (int k = lane; k < 120; k += 32) L[k] = 0.0;   // L, ci, cj
    Rotation rot;
    make_rotation(x, y, z, r, noi > noj ? noi : noj, false, rot);
    for (int k = lane; k < 100; k += 32) C[k] = ctrans(rot.T, k / 10, k % 10);
    __syncwarp();
    if (lane == 0) multipole_combine(St, spi, spj, L, ci, cj);
    __syncwarp();
    // X = C_i L  (ni x nj),  Y = X C_j^T (ni x nj)
    for (int k = lane; k < ni * nj; k += 32) {
        int ab = k / nj, q = k % nj;
        double v = 0.0;
        for (int m = 0; m < ni; m++) v += C[ab * 10 + m] * L[m * 10 + q];
        X[k] = v;
    }
    __syncwarp();
    double *tei = wsf + plan.tei + s.pair_tei[p];
    for (int k = lane; k < ni * nj; k += 32) {
        int ab = k / nj, cd = k % nj;
        double v = 0.0;
        for (int q = 0; q < nj; q++) v += X[ab * nj + q] * C[cd * 10 + q];
        tei[k] = (fabs(v) > PDG_TEI_UNDERFLOW) ? v : 0.0;   // BlockStorage underflow, QCModelMNDO.c:1029
    }
    // electron-core terms rotated to the molecular frame, scaled by -Z of the other core
    double *pe = wsf + plan.pair_e + (size_t)p * PDG_PAIR_E_STRIDE;
    if (lane < ni) {
        double v = 0.0;
        for (int m = 0; m < ni; m++) v += C[lane * 10 + m] * ci[m];
        pe[lane] = -Ej[PDG_E_ZCORE] * v;
    }
    if (lane >= 16 && lane - 16 < nj) {
        int cd = lane - 16;
        double v = 0.0;
        for (int m = 0; m < nj; m++) v += C[cd * 10 + m] * cj[m];
        pe[10 + cd] = -Ei[PDG_E_ZCORE] * v;
    }
    // resonance integrals H_ab = S_ab (beta_a + beta_b) / 2 (QCModelMNDO.c:1075-1092)
    double Sv[16];
    pair_overlap(Ei, Ej, x, y, z, false, lane, Sv, nullptr);
    int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    double *H = wsf + plan.H;
    if (lane < noi * noj) {
        int a = lane / noj, b = lane % noj;
        double v = Sv[a * 4 + b] * 0.5 * (Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]);
        H[(size_t)(is + a) * N + js + b] = v;
        H[(size_t)(js + b) * N + is + a] = v;
    }
    if (lane == 0) pe[20] = core_core(Ei, Ej, r, nullptr);
}

__global__ void __launch_bounds__(256) k_assemble_h(DeviceSystem s, FramePlan plan, int n_frames, double *__restrict__ ws)
{
    const int lane = threadIdx.x & 31;
    long gw = (long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (gw >= (long)n_frames * s.n_atoms) return;
    int f = (int)(gw / s.n_atoms), A = (int)(gw % s.n_atoms);
    double *wsf = ws + (size_t)f * plan.stride;
    double acc[10];
    for (int k = 0; k < 10; k++) acc[k] = 0.0;
    for (int B = lane; B < s.n_atoms; B += 32) {
        if (B == A) continue;
        int hi = A > B ? A : B, lo = A > B ? B : A;
        int p = hi * (hi - 1) / 2 + lo;
        const double *pe = wsf + plan.pair_e + (size_t)p * PDG_PAIR_E_STRIDE + (A > B ? 0 : 10);
        for (int k = 0; k < 10; k++) acc[k] += pe[k];
    }
    for (int k = 0; k < 10; k++) acc[k] = warp_sum(acc[k]);
    int no = s.atom_norb[A], st = s.atom_start[A], N = s.n_basis;
    const double *E = elem(s, s.atom_elem[A]);
    double *H = wsf + plan.H;
    if (lane < no * no) {
        int a = lane / no, b = lane % no;
        double v = acc[pk(a, b)] + (a == b ? E[PDG_E_USPD + a] : 0.0);
        H[(size_t)(st + a) * N + st + b] = v;
    }
}

void launch_pair_integrals(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *xyz, double *ws, cudaStream_t st)
{
    long warps = (long)n_frames * s.n_pairs;
    if (warps > 0) {
        int blocks = (int)((warps + PI_WARPS - 1) / PI_WARPS);
        k_pair_integrals<<<blocks, PI_WARPS * 32, 0, st>>>(s, p, n_frames, xyz, s.terms, ws);
    }
}

void launch_assemble_h(const DeviceSystem &s, const FramePlan &p, int n_frames, double *ws, cudaStream_t st)
{
    long warps = (long)n_frames * s.n_atoms;
    k_assemble_h<<<(int)((warps + 7) / 8), 256, 0, st>>>(s, p, n_frames, ws);
}

// ---------------------------------------------------------------------------------------------------
// Gradients.
#define PG_WARPS 4
#define PG_SM 1408

__global__ void __launch_bounds__(PG_WARPS * 32)
k_pair_gradients(DeviceSystem s, FramePlan plan, int n_frames, const double *__restrict__ xyz,
                 const double *__restrict__ terms, const double *__restrict__ density, double *__restrict__ ws)
{
    __shared__ double smem[PG_WARPS][PG_SM];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long gw = (long)blockIdx.x * PG_WARPS + w;
    if (gw >= (long)n_frames * s.n_pairs) return;
    int f = (int)(gw / s.n_pairs), p = (int)(gw % s.n_pairs);
    double *W = smem[w];
    double *St = W, *dSt = W + 96, *L = W + 192, *dL = W + 292, *ci = W + 392, *cj = W + 402, *dci = W + 412, *dcj = W + 422;
    double *C = W + 432, *CD = W + 532, *G = W + 832, *W1 = W + 932, *W2 = W + 1032, *W3 = W + 1132;
    double *oneI = W + 1232, *oneJ = W + 1242;
    int i = s.pair_i[p], j = s.pair_j[p];
    int eli = s.atom_elem[i], elj = s.atom_elem[j];
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    int noi = s.atom_norb[i], noj = s.atom_norb[j];
    int ni = noi * (noi + 1) / 2, nj = noj * (noj + 1) / 2;
    bool spi = noi > 1, spj = noj > 1;
    int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    const double *P = density + (size_t)f * N * N;
    double v3[3] = { R[3 * j] - R[3 * i], R[3 * j + 1] - R[3 * i + 1], R[3 * j + 2] - R[3 * i + 2] };
    double r = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
    double eng[3] = { 0.0, 0.0, 0.0 };

    // one-centre density vectors (off-diagonal elements doubled) and the two-centre density
    // Gamma = 1/4 aa bb (P_mk P_nl + P_nk P_ml) - oneI (x) oneJ  (QCModelMNDOState.c:196-250)
    if (lane < ni) { int a = MP_DA[lane], b = MP_DB[lane]; oneI[lane] = (a == b ? 1.0 : 2.0) * P[(size_t)(is + a) * N + is + b]; }
    if (lane >= 16 && lane - 16 < nj) { int k = lane - 16, a = MP_DA[k], b = MP_DB[k]; oneJ[k] = (a == b ? 1.0 : 2.0) * P[(size_t)(js + a) * N + js + b]; }
    __syncwarp();
    for (int k = lane; k < ni * nj; k += 32) {
        int kl = k / nj, mn = k % nj;
        int l = MP_DA[kl], kk = MP_DB[kl], n = MP_DA[mn], m = MP_DB[mn];   // kl = (l >= kk), mn = (n >= m)
        double aa = (kk == l) ? 1.0 : 2.0, bb = (m == n) ? 1.0 : 2.0;
        int K = is + kk, Lx = is + l, M = js + m, Nn = js + n;
        double fv = P[(size_t)M * N + K] * P[(size_t)Nn * N + Lx] + P[(size_t)Nn * N + K] * P[(size_t)M * N + Lx];
        G[k] = 0.25 * aa * bb * fv - oneI[kl] * oneJ[mn];
    }
    if (r >= 5.0e-3) {
        const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
        for (int k = lane; k < MP_TERMS_USED; k += 32) {
            double a = ta[k];
            if (a < 0.0) { St[k] = 0.0; dSt[k] = 0.0; continue; }
            double ro = r + to[k], sv = rsqrt(ro * ro + a);
            St[k] = sv; dSt[k] = -ro * sv * sv * sv;
        }
        for (int k = lane; k < 240; k += 32) L[k] = 0.0;     // L, dL, ci, cj, dci, dcj (contiguous)
        Rotation rot;
        make_rotation(v3[0], v3[1], v3[2], r, noi > noj ? noi : noj, true, rot);
        for (int k = lane; k < 100; k += 32) {
            int ab = k / 10, mn = k % 10;
            C[k] = ctrans(rot.T, ab, mn);
            for (int x = 0; x < 3; x++) CD[x * 100 + k] = rot.active ? ctrans_d(rot.T, rot.D[x], ab, mn) : 0.0;
        }
        __syncwarp();
        if (lane == 0) multipole_combine(St, spi, spj, L, ci, cj);
        if (lane == 1) multipole_combine(dSt, spi, spj, dL, dci, dcj);
        __syncwarp();
        // W1 = L C_j^T, W2 = C_i L, W3 = dL C_j^T
        for (int k = lane; k < ni * nj; k += 32) {
            int a = k / nj, b = k % nj;
            double w1 = 0.0, w3 = 0.0, w2 = 0.0;
            for (int q = 0; q < nj; q++) { w1 += L[a * 10 + q] * C[b * 10 + q]; w3 += dL[a * 10 + q] * C[b * 10 + q]; }
            for (int m = 0; m < ni; m++) w2 += C[a * 10 + m] * L[m * 10 + b];
            W1[k] = w1; W2[k] = w2; W3[k] = w3;
        }
        __syncwarp();
        double t0 = 0.0, ti[3] = { 0, 0, 0 }, tj[3] = { 0, 0, 0 };
        for (int k = lane; k < ni * nj; k += 32) {
            int ab = k / nj, cd = k % nj;
            double g = G[k], u0 = 0.0, ui[3] = { 0, 0, 0 }, uj[3] = { 0, 0, 0 };
            for (int m = 0; m < ni; m++) {
                double w1 = W1[m * nj + cd];
                u0 += C[ab * 10 + m] * W3[m * nj + cd];
                if (spi) for (int x = 0; x < 3; x++) ui[x] += CD[x * 100 + ab * 10 + m] * w1;
            }
            if (spj) for (int q = 0; q < nj; q++) { double w2 = W2[ab * nj + q]; for (int x = 0; x < 3; x++) uj[x] += w2 * CD[x * 100 + cd * 10 + q]; }
            t0 += g * u0;
            for (int x = 0; x < 3; x++) { ti[x] += g * ui[x]; tj[x] += g * uj[x]; }
        }
        // electron-core parts
        double o0 = 0.0, oi[3] = { 0, 0, 0 };
        if (lane < ni) {
            double u = 0.0, ux[3] = { 0, 0, 0 };
            for (int m = 0; m < ni; m++) {
                u += C[lane * 10 + m] * dci[m];
                if (spi) for (int x = 0; x < 3; x++) ux[x] += CD[x * 100 + lane * 10 + m] * ci[m];
            }
            o0 += oneI[lane] * u * (-Ej[PDG_E_ZCORE]);
            for (int x = 0; x < 3; x++) oi[x] += oneI[lane] * ux[x] * (-Ej[PDG_E_ZCORE]);
        }
        if (lane >= 16 && lane - 16 < nj) {
            int cd = lane - 16;
            double u = 0.0, ux[3] = { 0, 0, 0 };
            for (int m = 0; m < nj; m++) {
                u += C[cd * 10 + m] * dcj[m];
                if (spj) for (int x = 0; x < 3; x++) ux[x] += CD[x * 100 + cd * 10 + m] * cj[m];
            }
            o0 += oneJ[cd] * u * (-Ei[PDG_E_ZCORE]);
            for (int x = 0; x < 3; x++) oi[x] += oneJ[cd] * ux[x] * (-Ei[PDG_E_ZCORE]);
        }
        t0 = warp_sum(t0); o0 = warp_sum(o0);
        for (int x = 0; x < 3; x++) { ti[x] = warp_sum(ti[x]); tj[x] = warp_sum(tj[x]); oi[x] = warp_sum(oi[x]); }
        double dcore = 0.0;
        core_core(Ei, Ej, r, &dcore);
        // eng = -s (dcore + doei0f + dtei0f) + doei1 + dtei1   (MNDOIntegrals.c:392-418)
        for (int x = 0; x < 3; x++) {
            double sx = v3[x] / r;
            eng[x] = -sx * dcore - sx * o0 + sx * t0 - oi[x] + ti[x] + tj[x];
        }
    }
    // resonance integral derivatives: sum (beta_a + beta_b) P_ab dS_ab (QCModelMNDO.c:800-823)
    double Sv[16], SDv[48];
    pair_overlap(Ei, Ej, v3[0], v3[1], v3[2], true, lane, Sv, SDv);
    for (int a = 0; a < noi; a++)
        for (int b = 0; b < noj; b++) {
            double bp = (Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]) * P[(size_t)(is + a) * N + js + b];
            for (int x = 0; x < 3; x++) eng[x] += bp * SDv[x * 16 + a * 4 + b];
        }
    if (lane == 0) {
        double *pg = ws + (size_t)f * plan.stride + plan.pair_g + (size_t)p * 3;
        pg[0] = eng[0]; pg[1] = eng[1]; pg[2] = eng[2];
    }
}

__global__ void __launch_bounds__(256) k_reduce_gradients(DeviceSystem s, FramePlan plan, int n_frames,
                                                          const double *__restrict__ ws, double *__restrict__ grad)
{
    const int lane = threadIdx.x & 31;
    long gw = (long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (gw >= (long)n_frames * s.n_atoms) return;
    int f = (int)(gw / s.n_atoms), A = (int)(gw % s.n_atoms);
    const double *pg = ws + (size_t)f * plan.stride + plan.pair_g;
    double g[3] = { 0, 0, 0 };
    for (int B = lane; B < s.n_atoms; B += 32) {
        if (B == A) continue;
        int hi = A > B ? A : B, lo = A > B ? B : A;
        int p = hi * (hi - 1) / 2 + lo;
        double sg = (A > B) ? 1.0 : -1.0;   // pair term added to atom i, subtracted from atom j
        for (int x = 0; x < 3; x++) g[x] += sg * pg[(size_t)p * 3 + x];
    }
    for (int x = 0; x < 3; x++) g[x] = warp_sum(g[x]);
    if (lane < 3) grad[((size_t)f * s.n_atoms + A) * 3 + lane] = g[lane];
}

void launch_pair_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *xyz,
                           const double *density, double *ws, cudaStream_t st)
{
    long warps = (long)n_frames * s.n_pairs;
    if (warps > 0)
        k_pair_gradients<<<(int)((warps + PG_WARPS - 1) / PG_WARPS), PG_WARPS * 32, 0, st>>>(s, p, n_frames, xyz, s.terms, density, ws);
}

void launch_reduce_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *ws, double *grad, cudaStream_t st)
{
    long warps = (long)n_frames * s.n_atoms;
    k_reduce_gradients<<<(int)((warps + 7) / 8), 256, 0, st>>>(s, p, n_frames, ws, grad);
}
