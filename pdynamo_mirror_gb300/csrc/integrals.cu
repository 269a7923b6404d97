// integrals.cu - per-atom-pair integral and gradient kernels (FP64).
//
// k_pair_integrals   one warp per batch of 32 atom pairs (i > j) of a frame: core-core energy and the
//                    rotation's direction cosines one thread per pair, then per pair across the lanes:
//                    local-frame multipole TEIs and electron-core terms (multipole.cuh), rotation to the
//                    molecular frame, STO-6G overlap (overlap.cuh) -> resonance block of H.  Replaces the pair body of QCModelMNDO_Integrals
//                    (QCModelMNDO.c:1062-1112) with MNDOIntegrals_MolecularFrame2CIntegrals (MNDOIntegrals.c:147).
// k_assemble_h       one warp per (frame, atom): diagonal blocks of H = U + sum of electron-core terms.
// k_pair_gradients   one warp per batch of 32 atom pairs, laid out as k_pair_integrals: dE/dR of the pair (QCModelMNDO_Gradients,
//                    QCModelMNDO.c:732-840 with MNDOIntegrals_MolecularFrame2CIntegralsD, MNDOIntegrals.c:274,
//                    and QCModelMNDOState_GetGradientDensityTerms, QCModelMNDOState.c:178).
// k_reduce_gradients one warp per (frame, atom): sums the pair terms in a fixed order (deterministic).
#include "common.cuh"
#include "multipole.cuh"
#include "overlap.cuh"

#define PI_D 3.14159265358979323846
#define EXPONENT_TOLERANCE 25.0

// PM6's diatomic core-core term and d/dr (MNDOIntegralUtilities.c:45-96 energy, :164-218 derivative): Z_a Z_b gamma
// times 1 + 2 x_ab exp(-a_ab r_A r) for X-H pairs (X = C, N, O) or 1 + 2 x_ab exp(-a_ab r (1 + 0.0003 r_A^5)) for the
// others, plus 9.28 exp(-5.98 r_A) for C-C and -0.0007 exp(-(r_A - 2.9)^2) for Si-O, plus the unpolarisable core
// 1e-8 eV ((Z_a^1/3 + Z_b^1/3) / r_A)^12 (r_A: r in Angstroms).
__device__ double core_core_pm6(const double *a, const double *b, int za, int zb, double r, double gam, double dgdr, double *dedr)
{
    const double B2A = PDG_BOHRS_TO_ANGSTROMS, rA = r * B2A;
    const int kb = (int)b[PDG_E_INDEX];
    double scale = 1.0, dscale = 0.0;
    const double xij = 2.0 * a[PDG_E_DIAT_X + kb], aij = a[PDG_E_DIAT_A + kb];
    if (xij != 0.0) {
        const bool xh = (za == 1 && (zb == 6 || zb == 7 || zb == 8)) || (zb == 1 && (za == 6 || za == 7 || za == 8));
        if (xh) {
            const double f3 = xij * exp(-aij * r * r * B2A);
            dscale -= 2.0 * aij * r * B2A * f3;
            scale += f3;
        } else {
            const double r2 = rA * rA, dd = 0.0003 * r2 * r2 * rA, f3 = xij * exp(-aij * r * (1.0 + dd));
            dscale -= aij * (1.0 + 6.0 * dd) * f3;
            scale += f3;
        }
    }
    if (za == 6 && zb == 6) {
        const double f3 = 9.28 * exp(-5.98 * rA);
        dscale -= 5.98 * B2A * f3;
        scale += f3;
    }
    if ((za == 8 && zb == 14) || (za == 14 && zb == 8)) {
        const double dd = rA - 2.9, f3 = -0.0007 * exp(-dd * dd);
        dscale -= 2.0 * dd * B2A * f3;
        scale += f3;
    }
    const double zz = a[PDG_E_ZCORE] * b[PDG_E_ZCORE];
    const double UNPOLARIZABLE_CORE = 1.0e-08 / 27.21;   // 1e-8 eV in Hartree, as the reference writes it
    const double u = (cbrt(a[PDG_E_ZCORE]) + cbrt(b[PDG_E_ZCORE])) / rA, u2 = u * u, u4 = u2 * u2, u12 = u4 * u4 * u4;
    *dedr = zz * (dgdr * scale + gam * dscale) - 12.0 * UNPOLARIZABLE_CORE * u12 / r;
    return zz * gam * scale + UNPOLARIZABLE_CORE * u12;
}

// Core-core repulsion and d/dr (MNDOIntegralUtilities.c:35-150, :152-281): the diatomic branch for PM6 elements,
// else the exponential one; then the AM1/PM3 Gaussians and the PDDG terms.
__device__ double core_core(const double *a, const double *b, double r, double *dedr)
{
    const double B2A = PDG_BOHRS_TO_ANGSTROMS;
    int za = (int)a[PDG_E_Z], zb = (int)b[PDG_E_Z];
    double s8 = a[PDG_E_PO + 8] + b[PDG_E_PO + 8];
    double gam = rsqrt(r * r + s8 * s8), dgdr = -r * gam * gam * gam;
    if (a[PDG_E_DIAT] != 0.0 && b[PDG_E_DIAT] != 0.0) {
        double de, enuc = core_core_pm6(a, b, za, zb, r, gam, dgdr, &de), scale = 0.0, an = 0.0;
        const double zz = a[PDG_E_ZCORE] * b[PDG_E_ZCORE], gg = a[PDG_E_GPHOT] * b[PDG_E_GPHOT];
        for (int t = 0; t < 2; t++) {
            const double *e = t ? b : a;
            const int ng = (int)e[PDG_E_NG];
            for (int i = 0; i < ng; i++) {
                const double d = r - e[PDG_E_FN3 + i], ax = e[PDG_E_FN2 + i] * d * d;
                if (ax <= EXPONENT_TOLERANCE) {
                    const double ex = exp(-ax);
                    scale += gg * zz / r * e[PDG_E_FN1 + i] * ex;
                    an += e[PDG_E_FN1 + i] * (1.0 / (r * r) + e[PDG_E_FN2 + i] * 2.0 * d / r) * ex;
                }
            }
        }
        if (dedr) *dedr = de - an * gg * zz;
        return enuc + scale;
    }
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

// Warp-private shared scratch (doubles).
#define PI_WARPS 8
#define PI_SM 640

__device__ __forceinline__ int overlap_used(int noi, int noj)
{
    return 1 | (noi > 1 ? 2 : 0) | (noj > 1 ? 4 : 0) | (noi > 1 && noj > 1 ? 8 : 0);
}

// A warp takes a batch of up to 32 entries of its frame's (or batch item's) list of pairs that are not s-s.
template <bool BATCH>
__global__ void __launch_bounds__(PI_WARPS * 32)
k_pair_integrals(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt, const double *__restrict__ xyz, double *__restrict__ ws)
{
    __shared__ double smem[PI_WARPS][PI_SM];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    FrameView fv;
    int ub;
    if (!locate<BATCH, PDG_WORK_GEN>(sys0, plan0, n_frames, bt, (long)blockIdx.x * PI_WARPS + w, fv, ub)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const double *terms = s.terms;
    const int b0 = ub * 32, nb = min(32, s.n_gen - b0);
    double *W = smem[w];
    double *St = W, *L = W + 96, *ci = W + 196, *cj = W + 206, *X = W + 216, *C = W + 316;
    const double *R = xyz + 3 * fv.atom;
    double *wsf = ws + fv.ws;
    const int N = s.n_basis;
    double *H = wsf + plan.H;
    // one thread per pair: geometry, core-core energy, direction cosines
    int mi = 0, mj = 0;
    double mx = 0.0, my = 0.0, mz = 0.0, mr = 1.0;
    RotScalars mq = {};
    if (lane < nb) {
        const int p = s.pairs_gen[b0 + lane];
        mi = s.pair_i[p]; mj = s.pair_j[p];
        mx = R[3 * mj] - R[3 * mi]; my = R[3 * mj + 1] - R[3 * mi + 1]; mz = R[3 * mj + 2] - R[3 * mi + 2];
        mr = sqrt(mx * mx + my * my + mz * mz);
        wsf[plan.pair_e + (size_t)p * PDG_PAIR_E_STRIDE + 20] = core_core(elem(s, s.atom_elem[mi]), elem(s, s.atom_elem[mj]), mr, nullptr);
        rot_scalars(mx, my, mz, mr, max(s.atom_norb[mi], s.atom_norb[mj]), false, mq);
    }
    for (int t = 0; t < nb; t++) {
        const int p = s.pairs_gen[b0 + t];
        const int i = __shfl_sync(0xffffffffu, mi, t), j = __shfl_sync(0xffffffffu, mj, t);
        const double x = __shfl_sync(0xffffffffu, mx, t), y = __shfl_sync(0xffffffffu, my, t), z = __shfl_sync(0xffffffffu, mz, t);
        const double r = __shfl_sync(0xffffffffu, mr, t);
        const RotScalars q = rot_shfl(mq, t, false);
        const int eli = s.atom_elem[i], elj = s.atom_elem[j];
        const double *Ei = elem(s, eli), *Ej = elem(s, elj);
        const int noi = s.atom_norb[i], noj = s.atom_norb[j];
        const int ni = noi * (noi + 1) / 2, nj = noj * (noj + 1) / 2;
        const bool spi = noi > 1, spj = noj > 1;
        const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
        for (int k = lane; k < MP_TERMS_USED; k += 32) {
            const double a = ta[k];
            St[k] = (a < 0.0) ? 0.0 : rsqrt((r + to[k]) * (r + to[k]) + a);
        }
        for (int k = lane; k < 120; k += 32) L[k] = 0.0;   // L, ci, cj
        Rotation rot;
        rot_assemble(q, false, rot);
        for (int k = lane; k < 100; k += 32) C[k] = ctrans(rot.T, k / 10, k % 10);
        __syncwarp();
        {   // the local values as the sparse linear map of the terms, a few outputs per lane (L, ci, cj contiguous)
            const MultipoleMap &mpm = *(const MultipoleMap *)s.mp_map;
            for (int o = lane; o < mpm.n; o += 32) {
                const int *tk = mpm.term + o * MP_MAP_NNZ;
                const double *wk = mpm.w + o * MP_MAP_NNZ;
                double v = 0.0;
                for (int k = 0; k < mpm.nnz[o]; k++) v = fma(wk[k], St[tk[k]], v);
                L[mpm.out[o]] = v;
            }
        }
        __syncwarp();
        // X = C_i L  (ni x nj),  TEI = X C_j^T (ni x nj)
        for (int k = lane; k < ni * nj; k += 32) {
            const int ab = k / nj, qq = k % nj;
            double v = 0.0;
            for (int m = 0; m < ni; m++) v += C[ab * 10 + m] * L[m * 10 + qq];
            X[k] = v;
        }
        __syncwarp();
        double *tei = wsf + plan.tei + s.pair_tei[p];
        for (int k = lane; k < ni * nj; k += 32) {
            const int ab = k / nj, cd = k % nj;
            double v = 0.0;
            for (int qq = 0; qq < nj; qq++) v += X[ab * nj + qq] * C[cd * 10 + qq];
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
            const int cd = lane - 16;
            double v = 0.0;
            for (int m = 0; m < nj; m++) v += C[cd * 10 + m] * cj[m];
            pe[10 + cd] = -Ei[PDG_E_ZCORE] * v;
        }
        // resonance integrals H_ab = S_ab (beta_a + beta_b) / 2 (QCModelMNDO.c:1075-1092)
        const int eo = eli * s.n_elements + elj;
        double Fo[5], Do[5];
        if (s.ovl_tab) overlap_sums_table(s, eo, sqrt(x * x + y * y + z * z), Fo, nullptr);
        else overlap_sums(s.ovl + (size_t)s.ovl_off[eo] * OV_REC, s.ovl_n[eo], x * x + y * y + z * z, false, overlap_used(noi, noj), Fo, Do);
        const int is = s.atom_start[i], js = s.atom_start[j];
        if (lane < noi * noj) {
            const int a = lane / noj, b = lane % noj;
            const double AB[3] = { x, y, z };
            const double v = overlap_element(a, b, AB, Fo) * 0.5 * (Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]);
            H[(size_t)(is + a) * N + js + b] = v;
            H[(size_t)(js + b) * N + is + a] = v;
        }
        __syncwarp();
    }
}

// s-s pairs (two one-orbital atoms), one thread per pair: the (ss|ss) integral and the two electron-core
// terms (the single multipole terms 0, MP_CORE_I and MP_CORE_J; no rotation), the resonance integral from
// the ss radial sum, and the core-core energy.  Same results as the general kernel, without its warp-wide
// machinery for a pair that has one integral.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_pair_integrals_ss(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt,
                                                          const double *__restrict__ xyz, double *__restrict__ ws)
{
    FrameView fv;
    int u;
    if (!locate<BATCH, PDG_WORK_SS>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 256 + threadIdx.x, fv, u)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const double *terms = s.terms;
    const int p = s.pairs_ss[u];
    const int i = s.pair_i[p], j = s.pair_j[p], eli = s.atom_elem[i], elj = s.atom_elem[j];
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    const double *R = xyz + 3 * fv.atom;
    const double x = R[3 * j] - R[3 * i], y = R[3 * j + 1] - R[3 * i + 1], z = R[3 * j + 2] - R[3 * i + 2];
    const double R2 = x * x + y * y + z * z, r = sqrt(R2);
    double *wsf = ws + fv.ws;
    const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
    const double s0 = rsqrt((r + to[0]) * (r + to[0]) + ta[0]);
    const double ci = rsqrt((r + to[MP_CORE_I]) * (r + to[MP_CORE_I]) + ta[MP_CORE_I]);
    const double cj = rsqrt((r + to[MP_CORE_J]) * (r + to[MP_CORE_J]) + ta[MP_CORE_J]);
    wsf[plan.tei + s.pair_tei[p]] = (fabs(s0) > PDG_TEI_UNDERFLOW) ? s0 : 0.0;
    double *pe = wsf + plan.pair_e + (size_t)p * PDG_PAIR_E_STRIDE;
    pe[0] = -Ej[PDG_E_ZCORE] * ci;
    pe[10] = -Ei[PDG_E_ZCORE] * cj;
    pe[20] = core_core(Ei, Ej, r, nullptr);
    const int eo = eli * s.n_elements + elj;
    double S = 0.0;
    if (s.ovl_tab) {
        double Fo[5];
        overlap_sums_table(s, eo, r, Fo, nullptr);
        S = Fo[0];
    } else {
        const double *rec = s.ovl + (size_t)s.ovl_off[eo] * OV_REC;
        for (int t = 0; t < s.ovl_n[eo]; t++) {
            const double fac = rec[OV_REC * t] * R2;
            if (fac <= PRIMITIVE_OVERLAP_TOLERANCE) S = fma(rec[OV_REC * t + 1], exp(-fac), S);
        }
    }
    const int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    const double v = S * 0.5 * (Ei[PDG_E_BETA] + Ej[PDG_E_BETA]);
    double *H = wsf + plan.H;
    H[(size_t)is * N + js] = v;
    H[(size_t)js * N + is] = v;
}


// ---------------------------------------------------------------------------------------------------
// sp-s pairs (one atom with s and p orbitals, the other with s only), one thread per pair.  In the local
// frame the sp atom has five distributions with non-zero integrals against the s atom's ss (ss, s-sigma,
// sigma-sigma, pi-pi, pi'-pi'), so every molecular-frame value of the pair is a five-term sum over the
// distribution transform C built from the p-shell rotation T; the same holds for the electron-core
// terms, and for the gradients with dC/dx and the r-derivatives of the five local values.

__constant__ const int8_t SPS_MN[5] = { L_SS, L_PZS, L_PZPZ, L_PXPX, L_PYPY };

// The five local values on the sp side and the electron-core vector of the sp atom's electrons (from the
// multipole terms s_k, or their r-derivatives), and the s atom's electron-core term.
// sp_i: the sp atom is i (terms 1-6, core terms MP_CORE_I..), else j (terms 7-12, MP_CORE_J..).
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

template <typename Real>
__device__ __forceinline__ void sps_local(const double *to, const double *ta, double r, bool sp_i, bool deriv, Real *Lv,
                                          Real *cv, Real &c_s)
{
    auto term = [&](int k) -> Real {
        const double a = ta[k];
        if (a < 0.0) return Real(0);
        const Real ro = (Real)(r + to[k]), sv = rsq(ro * ro + (Real)a);
        return deriv ? -ro * sv * sv * sv : sv;
    };
    const int b = sp_i ? 1 : 7;
    const Real r0 = term(0), s1 = term(b), s2 = term(b + 1), s3 = term(b + 2), s4 = term(b + 3), s5 = term(b + 4), s6 = term(b + 5);
    const Real dz = Real(-0.5) * (s1 - s2), qzz = Real(0.25) * (s3 + s4) - Real(0.5) * s5, qxx = Real(0.5) * (s6 - s5);
    Lv[0] = r0; Lv[1] = dz; Lv[2] = r0 + qzz; Lv[3] = r0 + qxx; Lv[4] = r0 + qxx;
    const int c0 = sp_i ? MP_CORE_I : MP_CORE_J;
    const Real c1 = term(c0 + 1), c2 = term(c0 + 2), c3 = term(c0 + 3), c4 = term(c0 + 4), c5 = term(c0 + 5), c6 = term(c0 + 6);
    const Real c7 = term(c0 + 7);
    const Real cq = Real(0.25) * (c3 + c4) - Real(0.5) * c5, cx = Real(0.5) * (c6 - c5);
    cv[0] = term(c0); cv[1] = Real(-0.5) * (c1 - c2); cv[2] = c7 + cq; cv[3] = c7 + cx; cv[4] = c7 + cx;
    c_s = term(sp_i ? MP_CORE_J : MP_CORE_I);
}

// Overlap radial sums of one pair by one thread (overlap_sums without the warp).
template <typename Real>
__device__ __forceinline__ void overlap_sums_thread(const Real *__restrict__ rec, int nrec, Real R2, bool derivs, Real *F, Real *D)
{
    Real f0 = 0, f1 = 0, f2 = 0, f3 = 0, f4 = 0, d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0;
    for (int t = 0; t < nrec; t++) {
        const Real *q = rec + OV_REC * t;
        const Real abg = q[0], fac = abg * R2;
        if (fac > (Real)PRIMITIVE_OVERLAP_TOLERANCE) continue;
        const Real e = ov_exp(-fac);
        const int ty = (int)q[3];
        const Real t1 = q[1] * e, t2 = q[2] * e;
        f0 += ty == OV_SS ? t1 : Real(0); f1 += ty == OV_PS ? t1 : Real(0); f2 += ty == OV_SP ? t1 : Real(0); f3 += ty == OV_PP ? t1 : Real(0);
        f4 += t2;
        if (derivs) {
            const Real a2 = abg + abg, u1 = a2 * t1;
            d0 += ty == OV_SS ? u1 : Real(0); d1 += ty == OV_PS ? u1 : Real(0); d2 += ty == OV_SP ? u1 : Real(0); d3 += ty == OV_PP ? u1 : Real(0);
            d4 = fma(a2, t2, d4);
        }
    }
    F[0] = f0; F[1] = f1; F[2] = f2; F[3] = f3; F[4] = f4;
    D[0] = d0; D[1] = d1; D[2] = d2; D[3] = d3; D[4] = d4;
}

template <bool BATCH>
__global__ void __launch_bounds__(128) k_pair_integrals_sps(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt,
                                                           const double *__restrict__ xyz, double *__restrict__ ws)
{
    FrameView fv;
    int u;
    if (!locate<BATCH, PDG_WORK_SPS>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 128 + threadIdx.x, fv, u)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const int p = s.pairs_sps[u];
    const int i = s.pair_i[p], j = s.pair_j[p], eli = s.atom_elem[i], elj = s.atom_elem[j];
    const bool sp_i = s.atom_norb[i] > 1;
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    const double *R = xyz + 3 * fv.atom;
    const double x = R[3 * j] - R[3 * i], y = R[3 * j + 1] - R[3 * i + 1], z = R[3 * j + 2] - R[3 * i + 2];
    const double R2 = x * x + y * y + z * z, r = sqrt(R2);
    double *wsf = ws + fv.ws;
    double *pe = wsf + plan.pair_e + (size_t)p * PDG_PAIR_E_STRIDE;
    pe[20] = core_core(Ei, Ej, r, nullptr);
    const double *to = s.terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
    double Lv[5], cv[5], c_s;
    sps_local(to, ta, r, sp_i, false, Lv, cv, c_s);
    RotScalars q;
    rot_scalars(x, y, z, r, 4, false, q);
    Rotation rot;
    rot_assemble(q, false, rot);
    double *tei = wsf + plan.tei + s.pair_tei[p];
    const double zs = sp_i ? Ej[PDG_E_ZCORE] : Ei[PDG_E_ZCORE], zp = sp_i ? Ei[PDG_E_ZCORE] : Ej[PDG_E_ZCORE];
    double *pe_sp = pe + (sp_i ? 0 : 10);
#pragma unroll
    for (int ab = 0; ab < 10; ab++) {
        double v = 0.0, c = 0.0;
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const double t = ctrans(rot.T, ab, SPS_MN[k]);
            v = fma(t, Lv[k], v);
            c = fma(t, cv[k], c);
        }
        tei[ab] = (fabs(v) > PDG_TEI_UNDERFLOW) ? v : 0.0;   // the block is 10 x 1 or 1 x 10: the same order
        pe_sp[ab] = -zs * c;                                // electrons of the sp atom in the core of the s atom
    }
    pe[sp_i ? 10 : 0] = -zp * c_s;                          // electrons of the s atom in the core of the sp atom
    // resonance integrals H_ab = S_ab (beta_a + beta_b) / 2
    const int eo = eli * s.n_elements + elj;
    double Fo[5], Do[5];
    if (s.ovl_tab) overlap_sums_table(s, eo, r, Fo, nullptr);
    else overlap_sums_thread(s.ovl + (size_t)s.ovl_off[eo] * OV_REC, s.ovl_n[eo], R2, false, Fo, Do);
    const double AB[3] = { x, y, z };
    const int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    double *H = wsf + plan.H;
    for (int o = 0; o < 4; o++) {
        const int a = sp_i ? o : 0, b = sp_i ? 0 : o;
        const double v = overlap_element(a, b, AB, Fo) * 0.5 * (Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]);
        H[(size_t)(is + a) * N + js + b] = v;
        H[(size_t)(js + b) * N + is + a] = v;
    }
}

template <bool BATCH>
__global__ void __launch_bounds__(256) k_assemble_h(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt, double *__restrict__ ws)
{
    const int lane = threadIdx.x & 31;
    FrameView fv;
    int A;
    if (!locate<BATCH, PDG_WORK_ATOM>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 8 + (threadIdx.x >> 5), fv, A)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    double *wsf = ws + fv.ws;
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
    const Batch none = {};
    long warps = (long)n_frames * ((s.n_gen + 31) / 32);
    if (warps > 0) {
        int blocks = (int)((warps + PI_WARPS - 1) / PI_WARPS);
        k_pair_integrals<false><<<blocks, PI_WARPS * 32, 0, st>>>(s, p, n_frames, none, xyz, ws);
    }
    const long nss = (long)n_frames * s.n_ss;
    if (nss > 0) k_pair_integrals_ss<false><<<(int)((nss + 255) / 256), 256, 0, st>>>(s, p, n_frames, none, xyz, ws);
    const long nsps = (long)n_frames * s.n_sps;
    if (nsps > 0) k_pair_integrals_sps<false><<<(int)((nsps + 127) / 128), 128, 0, st>>>(s, p, n_frames, none, xyz, ws);
}

void launch_assemble_h(const DeviceSystem &s, const FramePlan &p, int n_frames, double *ws, cudaStream_t st)
{
    const Batch none = {};
    long warps = (long)n_frames * s.n_atoms;
    k_assemble_h<false><<<(int)((warps + 7) / 8), 256, 0, st>>>(s, p, n_frames, none, ws);
}

void launch_batch_integrals(const Batch &b, const double *xyz, double *ws, cudaStream_t st)
{
    const DeviceSystem s0 = {};
    const FramePlan p0 = {};
    if (b.total[PDG_WORK_GEN] > 0)
        k_pair_integrals<true><<<(b.total[PDG_WORK_GEN] + PI_WARPS - 1) / PI_WARPS, PI_WARPS * 32, 0, st>>>(s0, p0, 0, b, xyz, ws);
    if (b.total[PDG_WORK_SS] > 0)
        k_pair_integrals_ss<true><<<(b.total[PDG_WORK_SS] + 255) / 256, 256, 0, st>>>(s0, p0, 0, b, xyz, ws);
    if (b.total[PDG_WORK_SPS] > 0)
        k_pair_integrals_sps<true><<<(b.total[PDG_WORK_SPS] + 127) / 128, 128, 0, st>>>(s0, p0, 0, b, xyz, ws);
    k_assemble_h<true><<<(b.total[PDG_WORK_ATOM] + 7) / 8, 256, 0, st>>>(s0, p0, 0, b, ws);
}

// ---------------------------------------------------------------------------------------------------
// Gradients.
#define PG_WARPS 4
#define PG_SM 1408

// Real = double: the reference's FP64 arithmetic.  Real = float (the mixed method): the pair's multipole terms,
// rotation, density products, contractions, overlap sums and the lane sums in FP32, the core-core term and the
// assembly of the pair gradient in FP64 (per-pair errors ~1e-7 Hartree/Bohr, summed per atom in FP64).  The FP32
// variant over frames asks for four blocks per SM, so that a 304-frame batch of the water box (2432 warps) runs in
// one wave (the batch variant, with its larger per-item bookkeeping, three).
template <bool BATCH, typename Real> struct PairGradOcc { static constexpr int blocks = sizeof(Real) == 4 ? (BATCH ? 3 : 4) : 1; };

template <bool BATCH, typename Real>
__global__ void __launch_bounds__(PG_WARPS * 32, PairGradOcc<BATCH, Real>::blocks)
k_pair_gradients(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt, const double *__restrict__ xyz,
                 const double *__restrict__ density, double *__restrict__ ws)
{
    __shared__ Real smem[PG_WARPS][PG_SM];
    constexpr bool F32 = sizeof(Real) == 4;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    FrameView fv;
    int ub;
    if (!locate<BATCH, PDG_WORK_GEN>(sys0, plan0, n_frames, bt, (long)blockIdx.x * PG_WARPS + w, fv, ub)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const double *terms = s.terms;
    const int b0 = ub * 32, nb = min(32, s.n_gen - b0);
    Real *W = smem[w];
    Real *St = W, *dSt = W + 96, *L = W + 192, *dL = W + 292, *ci = W + 392, *cj = W + 402, *dci = W + 412, *dcj = W + 422;
    Real *C = W + 432, *CD = W + 532, *G = W + 832, *W1 = W + 932, *W2 = W + 1032, *W3 = W + 1132;
    Real *oneI = W + 1232, *oneJ = W + 1242, *Wres = W + 1252;
    const int N = s.n_basis;
    // lane sums: in FP64 for the FP64 variant, in FP32 (then widened) for the FP32 one
    auto lane_sum = [](Real v) -> double {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return (double)v;
    };
    const double *R = xyz + 3 * fv.atom;
    const double *P = density + fv.dens;
    const double *Sp = s.spin ? s.spin + fv.dens : nullptr;   // spin density (spin-unrestricted states)
    // one thread per pair: geometry, core-core derivative, direction cosines and their derivatives
    int mi = 0, mj = 0;
    double mx = 0.0, my = 0.0, mz = 0.0, mr = 1.0, mdc = 0.0;
    RotScalars mq = {};
    if (lane < nb) {
        const int p = s.pairs_gen[b0 + lane];
        mi = s.pair_i[p]; mj = s.pair_j[p];
        mx = R[3 * mj] - R[3 * mi]; my = R[3 * mj + 1] - R[3 * mi + 1]; mz = R[3 * mj + 2] - R[3 * mi + 2];
        mr = sqrt(mx * mx + my * my + mz * mz);
        core_core(elem(s, s.atom_elem[mi]), elem(s, s.atom_elem[mj]), mr, &mdc);
        rot_scalars(mx, my, mz, mr, max(s.atom_norb[mi], s.atom_norb[mj]), true, mq);
    }
    for (int t = 0; t < nb; t++) {
        const int p = s.pairs_gen[b0 + t];
        const int i = __shfl_sync(0xffffffffu, mi, t), j = __shfl_sync(0xffffffffu, mj, t);
        const double v3[3] = { __shfl_sync(0xffffffffu, mx, t), __shfl_sync(0xffffffffu, my, t), __shfl_sync(0xffffffffu, mz, t) };
        const double r = __shfl_sync(0xffffffffu, mr, t), dcore = __shfl_sync(0xffffffffu, mdc, t);
        const RotScalars q = rot_shfl(mq, t, true);
        const int eli = s.atom_elem[i], elj = s.atom_elem[j];
        const double *Ei = elem(s, eli), *Ej = elem(s, elj);
        const int noi = s.atom_norb[i], noj = s.atom_norb[j];
        const int ni = noi * (noi + 1) / 2, nj = noj * (noj + 1) / 2;
        const bool spi = noi > 1, spj = noj > 1;
        const int is = s.atom_start[i], js = s.atom_start[j];
        double eng[3] = { 0.0, 0.0, 0.0 };
        // one-centre density vectors (off-diagonal elements doubled) and the two-centre density
        // Gamma = 1/4 aa bb (P_mk P_nl + P_nk P_ml) - oneI (x) oneJ  (QCModelMNDOState.c:196-250)
        if (lane < ni) { const int a = MP_DA[lane], b = MP_DB[lane]; oneI[lane] = (Real)((a == b ? 1.0 : 2.0) * P[(size_t)(is + a) * N + is + b]); }
        if (lane >= 16 && lane - 16 < nj) { const int k = lane - 16, a = MP_DA[k], b = MP_DB[k]; oneJ[k] = (Real)((a == b ? 1.0 : 2.0) * P[(size_t)(js + a) * N + js + b]); }
        // resonance weights (beta_a + beta_b) P_ab (QCModelMNDO.c:800-823)
        if (lane < 16) {
            const int a = lane / 4, b = lane % 4;
            Wres[lane] = (a < noi && b < noj) ? (Real)((Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]) * P[(size_t)(is + a) * N + js + b]) : Real(0);
        }
        __syncwarp();
        for (int k = lane; k < ni * nj; k += 32) {
            const int kl = k / nj, mn = k % nj;
            const int l = MP_DA[kl], kk = MP_DB[kl], n = MP_DA[mn], m = MP_DB[mn];   // kl = (l >= kk), mn = (n >= m)
            const double aa = (kk == l) ? 1.0 : 2.0, bb = (m == n) ? 1.0 : 2.0;
            const int K = is + kk, Lx = is + l, M = js + m, Nn = js + n;
            if constexpr (F32) {
                const float pa = (float)P[(size_t)M * N + K], pb = (float)P[(size_t)Nn * N + Lx];
                const float pc = (float)P[(size_t)Nn * N + K], pd = (float)P[(size_t)M * N + Lx];
                float fv = pa * pb + pc * pd;
                // open shells: the spin density's products join the exchange part (QCModelMNDOState.c:178-260)
                if (Sp) fv += (float)Sp[(size_t)M * N + K] * (float)Sp[(size_t)Nn * N + Lx] + (float)Sp[(size_t)Nn * N + K] * (float)Sp[(size_t)M * N + Lx];
                G[k] = 0.25f * (float)(aa * bb) * fv - oneI[kl] * oneJ[mn];
            } else {
                double fv = P[(size_t)M * N + K] * P[(size_t)Nn * N + Lx] + P[(size_t)Nn * N + K] * P[(size_t)M * N + Lx];
                // open shells: the spin density's products join the exchange part (QCModelMNDOState.c:178-260)
                if (Sp) fv += Sp[(size_t)M * N + K] * Sp[(size_t)Nn * N + Lx] + Sp[(size_t)Nn * N + K] * Sp[(size_t)M * N + Lx];
                G[k] = (Real)(0.25 * aa * bb * fv) - oneI[kl] * oneJ[mn];
            }
        }
        if (r >= 5.0e-3) {
            const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
            for (int k = lane; k < MP_TERMS_USED; k += 32) {
                const double a = ta[k];
                if (a < 0.0) { St[k] = Real(0); dSt[k] = Real(0); continue; }
                const Real ro = (Real)(r + to[k]), sv = rsq(ro * ro + (Real)a);
                St[k] = sv; dSt[k] = -ro * sv * sv * sv;
            }
            for (int k = lane; k < 240; k += 32) L[k] = Real(0);     // L, dL, ci, cj, dci, dcj (contiguous)
            RotationT<Real> rot;
            rot_assemble(q, true, rot);
            for (int k = lane; k < 100; k += 32) {
                const int ab = k / 10, mn = k % 10;
                C[k] = ctrans(rot.T, ab, mn);
                for (int xx = 0; xx < 3; xx++) CD[xx * 100 + k] = rot.active ? ctrans_d(rot.T, rot.D[xx], ab, mn) : Real(0);
            }
            __syncwarp();
            {   // L, ci, cj and their r-derivatives as the sparse linear map of the terms, a few outputs per lane
                const MultipoleMap &mpm = *(const MultipoleMap *)s.mp_map;
                for (int o = lane; o < mpm.n; o += 32) {
                    const int *tk = mpm.term + o * MP_MAP_NNZ;
                    const Real *wk = sizeof(Real) == sizeof(double) ? (const Real *)(mpm.w + o * MP_MAP_NNZ) : (const Real *)(s.mp_w32 + o * MP_MAP_NNZ);
                    Real v = 0, dv = 0;
                    for (int k = 0; k < mpm.nnz[o]; k++) { v = fma(wk[k], St[tk[k]], v); dv = fma(wk[k], dSt[tk[k]], dv); }
                    const int out = mpm.out[o];
                    if (out < 100) { L[out] = v; dL[out] = dv; }
                    else if (out < 110) { ci[out - 100] = v; dci[out - 100] = dv; }
                    else { cj[out - 110] = v; dcj[out - 110] = dv; }
                }
            }
            __syncwarp();
            // W1 = L C_j^T, W2 = C_i L, W3 = dL C_j^T
            for (int k = lane; k < ni * nj; k += 32) {
                const int a = k / nj, b = k % nj;
                Real w1 = 0, w3 = 0, w2 = 0;
                for (int qq = 0; qq < nj; qq++) { w1 += L[a * 10 + qq] * C[b * 10 + qq]; w3 += dL[a * 10 + qq] * C[b * 10 + qq]; }
                for (int m = 0; m < ni; m++) w2 += C[a * 10 + m] * L[m * 10 + b];
                W1[k] = w1; W2[k] = w2; W3[k] = w3;
            }
            __syncwarp();
            Real t0 = 0, ti[3] = { 0, 0, 0 }, tj[3] = { 0, 0, 0 };
            for (int k = lane; k < ni * nj; k += 32) {
                const int ab = k / nj, cd = k % nj;
                const Real g = G[k];
                Real u0 = 0, ui[3] = { 0, 0, 0 }, uj[3] = { 0, 0, 0 };
                for (int m = 0; m < ni; m++) {
                    const Real w1 = W1[m * nj + cd];
                    u0 += C[ab * 10 + m] * W3[m * nj + cd];
                    if (spi) for (int xx = 0; xx < 3; xx++) ui[xx] += CD[xx * 100 + ab * 10 + m] * w1;
                }
                if (spj) for (int qq = 0; qq < nj; qq++) { const Real w2 = W2[ab * nj + qq]; for (int xx = 0; xx < 3; xx++) uj[xx] += w2 * CD[xx * 100 + cd * 10 + qq]; }
                t0 += g * u0;
                for (int xx = 0; xx < 3; xx++) { ti[xx] += g * ui[xx]; tj[xx] += g * uj[xx]; }
            }
            // electron-core parts
            Real o0 = 0, oi[3] = { 0, 0, 0 };
            const Real zj = (Real)Ej[PDG_E_ZCORE], zi = (Real)Ei[PDG_E_ZCORE];
            if (lane < ni) {
                Real u = 0, ux[3] = { 0, 0, 0 };
                for (int m = 0; m < ni; m++) {
                    u += C[lane * 10 + m] * dci[m];
                    if (spi) for (int xx = 0; xx < 3; xx++) ux[xx] += CD[xx * 100 + lane * 10 + m] * ci[m];
                }
                o0 += oneI[lane] * u * (-zj);
                for (int xx = 0; xx < 3; xx++) oi[xx] += oneI[lane] * ux[xx] * (-zj);
            }
            if (lane >= 16 && lane - 16 < nj) {
                const int cd = lane - 16;
                Real u = 0, ux[3] = { 0, 0, 0 };
                for (int m = 0; m < nj; m++) {
                    u += C[cd * 10 + m] * dcj[m];
                    if (spj) for (int xx = 0; xx < 3; xx++) ux[xx] += CD[xx * 100 + cd * 10 + m] * cj[m];
                }
                o0 += oneJ[cd] * u * (-zi);
                for (int xx = 0; xx < 3; xx++) oi[xx] += oneJ[cd] * ux[xx] * (-zi);
            }
            const double T0 = lane_sum(t0), O0 = lane_sum(o0);
            double TI[3], TJ[3], OI[3];
            for (int xx = 0; xx < 3; xx++) { TI[xx] = lane_sum(ti[xx]); TJ[xx] = lane_sum(tj[xx]); OI[xx] = lane_sum(oi[xx]); }
            // eng = -s (dcore + doei0f + dtei0f) + doei1 + dtei1   (MNDOIntegrals.c:392-418)
            for (int xx = 0; xx < 3; xx++) {
                const double sx = v3[xx] / r;
                eng[xx] = -sx * dcore - sx * O0 + sx * T0 - OI[xx] + TI[xx] + TJ[xx];
            }
        }
        // resonance integral derivatives: sum (beta_a + beta_b) P_ab dS_ab / dR_i
        const int eo = eli * s.n_elements + elj;
        Real Fo[5], Do[5], gr[3];
        const Real *orec = sizeof(Real) == sizeof(double) ? (const Real *)s.ovl : (const Real *)s.ovl32;
        const Real ab3[3] = { (Real)v3[0], (Real)v3[1], (Real)v3[2] };
        overlap_sums(orec + (size_t)s.ovl_off[eo] * OV_REC, s.ovl_n[eo], (Real)(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]), true,
                     overlap_used(noi, noj), Fo, Do);
        overlap_gradient(Wres, noi, noj, ab3, Fo, Do, gr);
        if (lane == 0) {
            double *pg = ws + fv.ws + plan.pair_g + (size_t)p * 3;
            pg[0] = eng[0] + (double)gr[0]; pg[1] = eng[1] + (double)gr[1]; pg[2] = eng[2] + (double)gr[2];
        }
        __syncwarp();
    }
}

// s-s pairs, one thread per pair: the gradient terms of k_pair_gradients for a pair with one orbital on each
// atom (no rotation, Gamma = P_ij^2 / 2 - P_ii P_jj), with the resonance term from the ss radial sums.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_pair_gradients_ss(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt,
                                                          const double *__restrict__ xyz, const double *__restrict__ density,
                                                          double *__restrict__ ws)
{
    FrameView fv;
    int u;
    if (!locate<BATCH, PDG_WORK_SS>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 256 + threadIdx.x, fv, u)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const double *terms = s.terms;
    const int p = s.pairs_ss[u];
    const int i = s.pair_i[p], j = s.pair_j[p], eli = s.atom_elem[i], elj = s.atom_elem[j];
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    const double *R = xyz + 3 * fv.atom;
    const double v3[3] = { R[3 * j] - R[3 * i], R[3 * j + 1] - R[3 * i + 1], R[3 * j + 2] - R[3 * i + 2] };
    const double R2 = v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2], r = sqrt(R2);
    const int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    const double *P = density + fv.dens;
    const double pii = P[(size_t)is * N + is], pjj = P[(size_t)js * N + js], pij = P[(size_t)is * N + js];
    const double sij = s.spin ? s.spin[fv.dens + (size_t)is * N + js] : 0.0;   // spin density (open shells)
    double eng[3] = { 0.0, 0.0, 0.0 };
    if (r >= 5.0e-3) {
        double dcore = 0.0;
        core_core(Ei, Ej, r, &dcore);
        const double *to = terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
        const double ro = r + to[0], sv = rsqrt(ro * ro + ta[0]), ds0 = -ro * sv * sv * sv;
        const double roi = r + to[MP_CORE_I], svi = rsqrt(roi * roi + ta[MP_CORE_I]), dci = -roi * svi * svi * svi;
        const double roj = r + to[MP_CORE_J], svj = rsqrt(roj * roj + ta[MP_CORE_J]), dcj = -roj * svj * svj * svj;
        const double gam = 0.5 * (pij * pij + sij * sij) - pii * pjj;
        const double t0 = gam * ds0;
        const double o0 = pii * dci * (-Ej[PDG_E_ZCORE]) + pjj * dcj * (-Ei[PDG_E_ZCORE]);
        for (int x = 0; x < 3; x++) {
            const double sx = v3[x] / r;
            eng[x] = -sx * dcore - sx * o0 + sx * t0;
        }
    }
    const int eo = eli * s.n_elements + elj;
    double D = 0.0;
    if (s.ovl_tab) {
        double Fo[5], Do[5];
        overlap_sums_table(s, eo, r, Fo, Do);
        D = Do[0];
    } else {
        const double *rec = s.ovl + (size_t)s.ovl_off[eo] * OV_REC;
        for (int t = 0; t < s.ovl_n[eo]; t++) {
            const double abg = rec[OV_REC * t], fac = abg * R2;
            if (fac <= PRIMITIVE_OVERLAP_TOLERANCE) D = fma((abg + abg) * rec[OV_REC * t + 1], exp(-fac), D);
        }
    }
    const double w = (Ei[PDG_E_BETA] + Ej[PDG_E_BETA]) * pij;
    double *pg = ws + fv.ws + plan.pair_g + (size_t)p * 3;
    for (int x = 0; x < 3; x++) pg[x] = eng[x] + v3[x] * w * D;
}


// sp-s pairs, one thread per pair: the gradient terms of k_pair_gradients for a pair with one sp and one s
// atom (Gamma over the sp atom's ten distributions, the five local values, dC/dx of the sp side only).
// Real = float (the mixed method): local values, rotation, contraction and overlap sums in FP32; the core-core
// term and the assembly of the pair gradient in FP64.
template <bool BATCH, typename Real>
__global__ void __launch_bounds__(128) k_pair_gradients_sps(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt,
                                                           const double *__restrict__ xyz, const double *__restrict__ density,
                                                           double *__restrict__ ws)
{
    FrameView fv;
    int u;
    if (!locate<BATCH, PDG_WORK_SPS>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 128 + threadIdx.x, fv, u)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const FramePlan &plan = BATCH ? fv.plan : plan0;
    const int p = s.pairs_sps[u];
    const int i = s.pair_i[p], j = s.pair_j[p], eli = s.atom_elem[i], elj = s.atom_elem[j];
    const bool sp_i = s.atom_norb[i] > 1;
    const double *Ei = elem(s, eli), *Ej = elem(s, elj);
    const double *R = xyz + 3 * fv.atom;
    const double v3[3] = { R[3 * j] - R[3 * i], R[3 * j + 1] - R[3 * i + 1], R[3 * j + 2] - R[3 * i + 2] };
    const double R2 = v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2], r = sqrt(R2);
    const int N = s.n_basis, is = s.atom_start[i], js = s.atom_start[j];
    const int as = sp_i ? is : js, bs = sp_i ? js : is;   // first orbital of the sp atom, the s orbital
    const double *P = density + fv.dens;
    // one-centre densities (off-diagonal elements doubled) and Gamma over the sp atom's distributions:
    // Gamma_ab = 1/4 aa (P_{s,a} P_{s,b} + P_{s,b} P_{s,a}) - one_sp[ab] one_s  (QCModelMNDOState.c:196-250)
    const double one_s = P[(size_t)bs * N + bs];
    const double *Sp = s.spin ? s.spin + fv.dens : nullptr;   // spin density (open shells)
    Real one_sp[10], gam[10];
#pragma unroll
    for (int ab = 0; ab < 10; ab++) {
        const int a = MP_DA[ab], b = MP_DB[ab];
        const double f = (a == b) ? 1.0 : 2.0, o = f * P[(size_t)(as + a) * N + as + b];
        one_sp[ab] = (Real)o;
        double x = P[(size_t)bs * N + as + a] * P[(size_t)bs * N + as + b];
        if (Sp) x += Sp[(size_t)bs * N + as + a] * Sp[(size_t)bs * N + as + b];
        gam[ab] = (Real)(0.5 * f * x - o * one_s);
    }
    double eng[3] = { 0.0, 0.0, 0.0 };
    if (r >= 5.0e-3) {
        double dcore = 0.0;
        core_core(Ei, Ej, r, &dcore);
        const double *to = s.terms + (size_t)(eli * s.n_elements + elj) * 2 * MP_NTERMS, *ta = to + MP_NTERMS;
        Real Lv[5], cv[5], dLv[5], dcv[5], c_s, dc_s;
        sps_local(to, ta, r, sp_i, false, Lv, cv, c_s);
        sps_local(to, ta, r, sp_i, true, dLv, dcv, dc_s);
        RotScalars q;
        rot_scalars(v3[0], v3[1], v3[2], r, 4, true, q);
        RotationT<Real> rot;
        rot_assemble(q, true, rot);
        const Real zs = (Real)(sp_i ? Ej[PDG_E_ZCORE] : Ei[PDG_E_ZCORE]), zp = (Real)(sp_i ? Ei[PDG_E_ZCORE] : Ej[PDG_E_ZCORE]);
        Real t0 = 0, o0 = 0, tr[3] = { 0, 0, 0 }, orr[3] = { 0, 0, 0 };
#pragma unroll
        for (int ab = 0; ab < 10; ab++) {
            Real u0 = 0, w0 = 0, ur[3] = { 0, 0, 0 }, wr[3] = { 0, 0, 0 };
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const Real c = ctrans(rot.T, ab, SPS_MN[k]);
                u0 = fma(c, dLv[k], u0);
                w0 = fma(c, dcv[k], w0);
#pragma unroll
                for (int xx = 0; xx < 3; xx++) {
                    const Real cd = ctrans_d(rot.T, rot.D[xx], ab, SPS_MN[k]);
                    ur[xx] = fma(cd, Lv[k], ur[xx]);
                    wr[xx] = fma(cd, cv[k], wr[xx]);
                }
            }
            t0 = fma(gam[ab], u0, t0);
            o0 = fma(one_sp[ab] * w0, -zs, o0);
#pragma unroll
            for (int xx = 0; xx < 3; xx++) { tr[xx] = fma(gam[ab], ur[xx], tr[xx]); orr[xx] = fma(one_sp[ab] * wr[xx], -zs, orr[xx]); }
        }
        o0 = fma((Real)one_s * dc_s, -zp, o0);
        // eng = -s (dcore + doei0f + dtei0f) + doei1 + dtei1   (MNDOIntegrals.c:392-418)
        for (int xx = 0; xx < 3; xx++) {
            const double sx = v3[xx] / r;
            eng[xx] = -sx * dcore - sx * (double)o0 + sx * (double)t0 - (double)orr[xx] + (double)tr[xx];
        }
    }
    // resonance integral derivatives: sum (beta_a + beta_b) P_ab dS_ab / dR_i
    const int noi = s.atom_norb[i], noj = s.atom_norb[j];
    Real Wres[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int a = k / 4, b = k % 4;
        Wres[k] = (a < noi && b < noj) ? (Real)((Ei[PDG_E_BETA + a] + Ej[PDG_E_BETA + b]) * P[(size_t)(is + a) * N + js + b]) : Real(0);
    }
    const int eo = eli * s.n_elements + elj;
    Real Fo[5], Do[5], gr[3];
    const Real *orec = sizeof(Real) == sizeof(double) ? (const Real *)s.ovl : (const Real *)s.ovl32;
    const Real ab3[3] = { (Real)v3[0], (Real)v3[1], (Real)v3[2] };
    overlap_sums_thread(orec + (size_t)s.ovl_off[eo] * OV_REC, s.ovl_n[eo], (Real)R2, true, Fo, Do);
    overlap_gradient(Wres, noi, noj, ab3, Fo, Do, gr);
    double *pg = ws + fv.ws + plan.pair_g + (size_t)p * 3;
    for (int x = 0; x < 3; x++) pg[x] = eng[x] + (double)gr[x];
}

template <bool BATCH>
__global__ void __launch_bounds__(256) k_reduce_gradients(DeviceSystem sys0, FramePlan plan0, int n_frames, Batch bt,
                                                          const double *__restrict__ ws, double *__restrict__ grad)
{
    const int lane = threadIdx.x & 31;
    FrameView fv;
    int A;
    if (!locate<BATCH, PDG_WORK_ATOM>(sys0, plan0, n_frames, bt, (long)blockIdx.x * 8 + (threadIdx.x >> 5), fv, A)) return;
    const DeviceSystem &s = BATCH ? fv.s : sys0;
    const double *pg = ws + fv.ws + (BATCH ? fv.plan.pair_g : plan0.pair_g);
    double g[3] = { 0, 0, 0 };
    for (int B = lane; B < s.n_atoms; B += 32) {
        if (B == A) continue;
        int hi = A > B ? A : B, lo = A > B ? B : A;
        int p = hi * (hi - 1) / 2 + lo;
        double sg = (A > B) ? 1.0 : -1.0;   // pair term added to atom i, subtracted from atom j
        for (int x = 0; x < 3; x++) g[x] += sg * pg[(size_t)p * 3 + x];
    }
    for (int x = 0; x < 3; x++) g[x] = warp_sum(g[x]);
    if (lane < 3) grad[(fv.atom + A) * 3 + lane] = g[lane];
}

void launch_pair_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *xyz,
                           const double *density, double *ws, cudaStream_t st, bool fp32_terms)
{
    const Batch none = {};
    long warps = (long)n_frames * ((s.n_gen + 31) / 32);
    if (warps > 0) {
        if (fp32_terms)
            k_pair_gradients<false, float><<<(int)((warps + PG_WARPS - 1) / PG_WARPS), PG_WARPS * 32, 0, st>>>(s, p, n_frames, none, xyz, density, ws);
        else
            k_pair_gradients<false, double><<<(int)((warps + PG_WARPS - 1) / PG_WARPS), PG_WARPS * 32, 0, st>>>(s, p, n_frames, none, xyz, density, ws);
    }
    const long nss = (long)n_frames * s.n_ss;
    if (nss > 0) k_pair_gradients_ss<false><<<(int)((nss + 255) / 256), 256, 0, st>>>(s, p, n_frames, none, xyz, density, ws);
    const long nsps = (long)n_frames * s.n_sps;
    if (nsps > 0) {
        if (fp32_terms) k_pair_gradients_sps<false, float><<<(int)((nsps + 127) / 128), 128, 0, st>>>(s, p, n_frames, none, xyz, density, ws);
        else k_pair_gradients_sps<false, double><<<(int)((nsps + 127) / 128), 128, 0, st>>>(s, p, n_frames, none, xyz, density, ws);
    }
}

void launch_reduce_gradients(const DeviceSystem &s, const FramePlan &p, int n_frames, const double *ws, double *grad, cudaStream_t st)
{
    const Batch none = {};
    long warps = (long)n_frames * s.n_atoms;
    k_reduce_gradients<false><<<(int)((warps + 7) / 8), 256, 0, st>>>(s, p, n_frames, none, ws, grad);
}

void launch_batch_gradients(const Batch &b, const double *xyz, const double *density, double *ws, double *grad, cudaStream_t st,
                            bool fp32_terms)
{
    const DeviceSystem s0 = {};
    const FramePlan p0 = {};
    if (b.total[PDG_WORK_GEN] > 0) {
        if (fp32_terms)
            k_pair_gradients<true, float><<<(b.total[PDG_WORK_GEN] + PG_WARPS - 1) / PG_WARPS, PG_WARPS * 32, 0, st>>>(s0, p0, 0, b, xyz, density, ws);
        else
            k_pair_gradients<true, double><<<(b.total[PDG_WORK_GEN] + PG_WARPS - 1) / PG_WARPS, PG_WARPS * 32, 0, st>>>(s0, p0, 0, b, xyz, density, ws);
    }
    if (b.total[PDG_WORK_SS] > 0)
        k_pair_gradients_ss<true><<<(b.total[PDG_WORK_SS] + 255) / 256, 256, 0, st>>>(s0, p0, 0, b, xyz, density, ws);
    if (b.total[PDG_WORK_SPS] > 0)
    {
        if (fp32_terms) k_pair_gradients_sps<true, float><<<(b.total[PDG_WORK_SPS] + 127) / 128, 128, 0, st>>>(s0, p0, 0, b, xyz, density, ws);
        else k_pair_gradients_sps<true, double><<<(b.total[PDG_WORK_SPS] + 127) / 128, 128, 0, st>>>(s0, p0, 0, b, xyz, density, ws);
    }
    k_reduce_gradients<true><<<(b.total[PDG_WORK_ATOM] + 7) / 8, 256, 0, st>>>(s0, p0, 0, b, ws, grad);
}
