// multipole.cuh - local-frame two-centre integrals of the NDDO sp multipole model, GPU formulation.
//
// pDynamo evaluates each local-frame integral (MNDOIntegralUtilities_LocalFrame2CTEIsSP and
// _LocalFrame2COEIsSP, MNDOIntegralUtilities.c:1117-1440) as a fixed linear combination of terms
//     s_k(r) = 1 / sqrt( (r + o_k)^2 + a_k )
// whose offsets o_k and additive terms a_k depend only on the two elements (the charge separations dd,
// 2 qq and the additive terms po of MNDOParameters.c:762-875).  Here the (o_k, a_k) are tabulated once
// per ordered element pair; the lanes of a warp each evaluate a few s_k, and the same combination applied
// to ds_k/dr = -(r + o_k) s_k^3 gives the r-derivatives that pDynamo codes separately (:1353-1438).
#pragma once
#include "common.cuh"

#define MP_NTERMS 96
// term indices: 0 ss; 1-6 sp/s; 7-12 s/sp; 13-60 and 61-68 sp/sp (reference sqr13..sqr60, sqr64..sqr71);
// 69-76 electron(i)-core(j); 77-84 electron(j)-core(i).
#define MP_CORE_I 69
#define MP_CORE_J 77
#define MP_TERMS_USED 85

// Local distributions packed i(i+1)/2 + j over local orbitals s, p-sigma, p-pi+, p-pi-.
enum { L_SS = 0, L_PZS = 1, L_PZPZ = 2, L_PXS = 3, L_PXPZ = 4, L_PXPX = 5, L_PYS = 6, L_PYPZ = 7, L_PYPX = 8, L_PYPY = 9 };

// Host: fill the (o, a) table of an ordered element pair (ei holds the first atom's electrons).
// a < 0 marks a term that does not occur for this pair.
inline void multipole_terms(const double *ei, const double *ej, double *o, double *a)
{
    for (int k = 0; k < MP_NTERMS; k++) { o[k] = 0.0; a[k] = -1.0; }
    const double *pi = ei + PDG_E_PO, *pj = ej + PDG_E_PO;
    bool spi = ei[PDG_E_NORB] > 3.5, spj = ej[PDG_E_NORB] > 3.5;
    double da = ei[PDG_E_DD], qa = 2.0 * ei[PDG_E_QQ], db = ej[PDG_E_DD], qb = 2.0 * ej[PDG_E_QQ];
    double qa0 = ei[PDG_E_QQ], qb0 = ej[PDG_E_QQ];
    auto set = [&](int k, double off, double add) { o[k] = off; a[k] = add; };
    auto sq = [](double x) { return x * x; };
    set(0, 0.0, sq(pi[0] + pj[0]));
    if (spi) {
        double ade = sq(pi[1] + pj[0]), aqe = sq(pi[2] + pj[0]);
        set(1, da, ade); set(2, -da, ade); set(3, qa, aqe); set(4, -qa, aqe); set(5, 0.0, aqe); set(6, 0.0, aqe + qa * qa);
    }
    if (spj) {
        double aed = sq(pi[0] + pj[1]), aeq = sq(pi[0] + pj[2]);
        set(7, -db, aed); set(8, db, aed); set(9, -qb, aeq); set(10, qb, aeq); set(11, 0.0, aeq); set(12, 0.0, aeq + qb * qb);
    }
    if (spi && spj) {
        double axx = sq(pi[1] + pj[1]), adq = sq(pi[1] + pj[2]), aqd = sq(pi[2] + pj[1]), aqq = sq(pi[2] + pj[2]);
        set(13, 0.0, axx + sq(da - db)); set(14, 0.0, axx + sq(da + db));
        set(15, da - db, axx); set(16, -da + db, axx); set(17, -da - db, axx); set(18, da + db, axx);
        set(19, da, adq); set(20, da, adq + qb * qb); set(21, -da, adq); set(22, -da, adq + qb * qb);
        set(23, -db, aqd); set(24, -db, aqd + qa * qa); set(25, db, aqd); set(26, db, aqd + qa * qa);
        set(27, da - qb, adq); set(28, -da - qb, adq); set(29, da + qb, adq); set(30, -da + qb, adq);
        set(31, qa - db, aqd); set(32, qa + db, aqd); set(33, -qa - db, aqd); set(34, -qa + db, aqd);
        set(35, 0.0, aqq); set(36, 0.0, aqq + sq(qa - qb)); set(37, 0.0, aqq + sq(qa + qb));
        set(38, 0.0, aqq + qa * qa); set(39, 0.0, aqq + qb * qb); set(40, 0.0, aqq + qa * qa + qb * qb);
        set(41, -qb, aqq); set(42, -qb, aqq + qa * qa); set(43, qb, aqq); set(44, qb, aqq + qa * qa);
        set(45, qa, aqq); set(46, qa, aqq + qb * qb); set(47, -qa, aqq); set(48, -qa, aqq + qb * qb);
        set(49, qa - qb, aqq); set(50, qa + qb, aqq); set(51, -qa - qb, aqq); set(52, -qa + qb, aqq);
        set(53, -qb0, sq(da - qb0) + adq); set(54, qb0, sq(da - qb0) + adq);
        set(55, -qb0, sq(da + qb0) + adq); set(56, qb0, sq(da + qb0) + adq);
        set(57, qa0, sq(qa0 - db) + aqd); set(58, -qa0, sq(qa0 - db) + aqd);
        set(59, qa0, sq(qa0 + db) + aqd); set(60, -qa0, sq(qa0 + db) + aqd);
        double x = sq(qa0 - qb0), y = sq(qa0 + qb0);
        set(61, qa0 - qb0, x + aqq); set(62, qa0 - qb0, y + aqq);
        set(63, qa0 + qb0, x + aqq); set(64, qa0 + qb0, y + aqq);
        set(65, -qa0 - qb0, x + aqq); set(66, -qa0 - qb0, y + aqq);
        set(67, -qa0 + qb0, x + aqq); set(68, -qa0 + qb0, y + aqq);
    }
    // electron distribution on i, core of j (swapped = False)
    set(MP_CORE_I, 0.0, sq(pi[0] + pj[8]));
    if (spi) {
        double ade = sq(pi[1] + pj[8]), aqe = sq(pi[2] + pj[8]);
        set(MP_CORE_I + 1, da, ade); set(MP_CORE_I + 2, -da, ade); set(MP_CORE_I + 3, qa, aqe); set(MP_CORE_I + 4, -qa, aqe);
        set(MP_CORE_I + 5, 0.0, aqe); set(MP_CORE_I + 6, 0.0, aqe + qa * qa); set(MP_CORE_I + 7, 0.0, sq(pi[6] + pj[8]));
    }
    // electron distribution on j, core of i (swapped = True: charge separations change sign)
    set(MP_CORE_J, 0.0, sq(pj[0] + pi[8]));
    if (spj) {
        double ade = sq(pj[1] + pi[8]), aqe = sq(pj[2] + pi[8]);
        set(MP_CORE_J + 1, -db, ade); set(MP_CORE_J + 2, db, ade); set(MP_CORE_J + 3, -qb, aqe); set(MP_CORE_J + 4, qb, aqe);
        set(MP_CORE_J + 5, 0.0, aqe); set(MP_CORE_J + 6, 0.0, aqe + qb * qb); set(MP_CORE_J + 7, 0.0, sq(pj[6] + pi[8]));
    }
}

// Device: combine term values s (or their r-derivatives) into the local-frame TEI matrix L (10 x 10,
// row = distribution on i, column = distribution on j) and the two electron-core vectors (before the
// -Z scaling).  L, ci and cj must be zero on entry.  Formulas: MNDOIntegralUtilities.c:1130-1170,1198-1351.
__host__ __device__ inline void multipole_combine(const double *s, bool spi, bool spj, double *L, double *ci, double *cj)
{
    const double E1 = 0.5, E2 = 0.25, E3 = 0.125, E4 = 0.0625;
    double ri0 = s[0];
    double dze = 0, qzze = 0, qxxe = 0, edz = 0, eqzz = 0, eqxx = 0;
    L[L_SS * 10 + L_SS] = ri0;
    if (spi) {
        dze = -E1 * (s[1] - s[2]); qzze = E2 * (s[3] + s[4]) - E1 * s[5]; qxxe = E1 * (s[6] - s[5]);
        L[L_PZS * 10 + L_SS] = dze; L[L_PZPZ * 10 + L_SS] = ri0 + qzze; L[L_PXPX * 10 + L_SS] = ri0 + qxxe;
        L[L_PYPY * 10 + L_SS] = ri0 + qxxe;
    }
    if (spj) {
        edz = -E1 * (s[7] - s[8]); eqzz = E2 * (s[9] + s[10]) - E1 * s[11]; eqxx = E1 * (s[12] - s[11]);
        L[L_SS * 10 + L_PZS] = edz; L[L_SS * 10 + L_PZPZ] = ri0 + eqzz; L[L_SS * 10 + L_PXPX] = ri0 + eqxx;
        L[L_SS * 10 + L_PYPY] = ri0 + eqxx;
    }
    if (spi && spj) {
        const double *t = s;   // t[13..60] as in the reference, t[61..68] = reference sqr64..sqr71
        double dxdx = E1 * t[13] - E1 * t[14];
        double dzdz = E2 * t[15] + E2 * t[16] - E2 * t[17] - E2 * t[18];
        double dzqxx = E2 * t[19] - E2 * t[20] - E2 * t[21] + E2 * t[22];
        double qxxdz = E2 * t[23] - E2 * t[24] - E2 * t[25] + E2 * t[26];
        double dzqzz = -E3 * t[27] + E3 * t[28] - E3 * t[29] + E3 * t[30] - E2 * t[21] + E2 * t[19];
        double qzzdz = -E3 * t[31] + E3 * t[32] - E3 * t[33] + E3 * t[34] + E2 * t[23] - E2 * t[25];
        double qxxqxx = E3 * t[36] + E3 * t[37] - E2 * t[38] - E2 * t[39] + E2 * t[35];
        double qxxqyy = E2 * t[40] - E2 * t[38] - E2 * t[39] + E2 * t[35];
        double qxxqzz = E3 * t[42] + E3 * t[44] - E3 * t[41] - E3 * t[43] - E2 * t[38] + E2 * t[35];
        double qzzqxx = E3 * t[46] + E3 * t[48] - E3 * t[45] - E3 * t[47] - E2 * t[39] + E2 * t[35];
        double qzzqzz = E4 * t[49] + E4 * t[50] + E4 * t[51] + E4 * t[52] - E3 * t[47] - E3 * t[45] - E3 * t[41] - E3 * t[43] + E2 * t[35];
        double dxqxz = -E2 * t[53] + E2 * t[54] + E2 * t[55] - E2 * t[56];
        double qxzdx = -E2 * t[57] + E2 * t[58] + E2 * t[59] - E2 * t[60];
        double qxzqxz = E3 * t[61] - E3 * t[63] - E3 * t[65] + E3 * t[67] - E3 * t[62] + E3 * t[64] + E3 * t[66] - E3 * t[68];
        L[L_PZS * 10 + L_PZS] = dzdz;
        L[L_PXS * 10 + L_PXS] = dxdx;            L[L_PYS * 10 + L_PYS] = dxdx;
        L[L_PZPZ * 10 + L_PZS] = edz + qzzdz;
        L[L_PXPX * 10 + L_PZS] = edz + qxxdz;    L[L_PYPY * 10 + L_PZS] = edz + qxxdz;
        L[L_PXPZ * 10 + L_PXS] = qxzdx;          L[L_PYPZ * 10 + L_PYS] = qxzdx;
        L[L_PZS * 10 + L_PZPZ] = dze + dzqzz;
        L[L_PZS * 10 + L_PXPX] = dze + dzqxx;    L[L_PZS * 10 + L_PYPY] = dze + dzqxx;
        L[L_PXS * 10 + L_PXPZ] = dxqxz;          L[L_PYS * 10 + L_PYPZ] = dxqxz;
        L[L_PZPZ * 10 + L_PZPZ] = ri0 + eqzz + qzze + qzzqzz;
        L[L_PXPX * 10 + L_PZPZ] = ri0 + eqzz + qxxe + qxxqzz;  L[L_PYPY * 10 + L_PZPZ] = ri0 + eqzz + qxxe + qxxqzz;
        L[L_PZPZ * 10 + L_PXPX] = ri0 + eqxx + qzze + qzzqxx;  L[L_PZPZ * 10 + L_PYPY] = ri0 + eqxx + qzze + qzzqxx;
        L[L_PXPX * 10 + L_PXPX] = ri0 + eqxx + qxxe + qxxqxx;  L[L_PYPY * 10 + L_PYPY] = ri0 + eqxx + qxxe + qxxqxx;
        L[L_PXPZ * 10 + L_PXPZ] = qxzqxz;        L[L_PYPZ * 10 + L_PYPZ] = qxzqxz;
        L[L_PXPX * 10 + L_PYPY] = ri0 + eqxx + qxxe + qxxqyy;  L[L_PYPY * 10 + L_PXPX] = ri0 + eqxx + qxxe + qxxqyy;
        L[L_PYPX * 10 + L_PYPX] = 0.5 * (qxxqxx - qxxqyy);
    }
    const double *c = s + MP_CORE_I;
    ci[L_SS] = c[0];
    if (spi) {
        double d1 = -E1 * (c[1] - c[2]), qz = E2 * (c[3] + c[4]) - E1 * c[5], qx = E1 * (c[6] - c[5]);
        ci[L_PZS] = d1; ci[L_PZPZ] = c[7] + qz; ci[L_PXPX] = c[7] + qx; ci[L_PYPY] = c[7] + qx;
    }
    c = s + MP_CORE_J;
    cj[L_SS] = c[0];
    if (spj) {
        double d1 = -E1 * (c[1] - c[2]), qz = E2 * (c[3] + c[4]) - E1 * c[5], qx = E1 * (c[6] - c[5]);
        cj[L_PZS] = d1; cj[L_PZPZ] = c[7] + qz; cj[L_PXPX] = c[7] + qx; cj[L_PYPY] = c[7] + qx;
    }
}

// multipole_combine of an sp-sp pair is linear in the term values: as a sparse map, output o (0-99 L,
// 100-109 ci, 110-119 cj) = sum over at most MP_MAP_NNZ terms of weight * s[term].  Built once on the host
// (by applying multipole_combine to unit vectors) so that the lanes of a warp each evaluate a few outputs.
#define MP_MAP_NNZ 16
#define MP_MAP_MAX 120
struct MultipoleMap { int n; int out[MP_MAP_MAX], nnz[MP_MAP_MAX], term[MP_MAP_MAX * MP_MAP_NNZ]; double w[MP_MAP_MAX * MP_MAP_NNZ]; };

inline bool multipole_map_spsp(MultipoleMap &m)
{
    double M[MP_MAP_MAX][MP_TERMS_USED] = {};
    for (int k = 0; k < MP_TERMS_USED; k++) {
        double sv[MP_NTERMS] = {}, L[100] = {}, ci[10] = {}, cj[10] = {};
        sv[k] = 1.0;
        multipole_combine(sv, true, true, L, ci, cj);
        for (int o = 0; o < 100; o++) M[o][k] = L[o];
        for (int o = 0; o < 10; o++) { M[100 + o][k] = ci[o]; M[110 + o][k] = cj[o]; }
    }
    m.n = 0;
    for (int o = 0; o < MP_MAP_MAX; o++) {
        int nz = 0;
        for (int k = 0; k < MP_TERMS_USED; k++)
            if (M[o][k] != 0.0) {
                if (nz == MP_MAP_NNZ) return false;
                m.term[m.n * MP_MAP_NNZ + nz] = k; m.w[m.n * MP_MAP_NNZ + nz] = M[o][k]; nz++;
            }
        if (nz == 0) continue;
        m.out[m.n] = o; m.nnz[m.n] = nz; m.n++;
    }
    return true;
}

// Local-to-molecular rotation of the p shell and its derivatives with respect to the coordinates of
// atom j (MNDOIntegralUtilities_GetTransformationMatrices, MNDOIntegralUtilities.c:449-465 for s/p,
// axes swapped when |z/r| > 0.99999999).  T[a][m]: molecular orbital a (s, pz, px, py), local m
// (s, sigma, pi+, pi-).  Returns false when no rotation applies (identity, zero derivatives).
template <typename R> struct RotationT { R T[4][4]; R D[3][4][4]; bool active; };
using Rotation = RotationT<double>;

// The geometry-dependent scalars of the rotation (square root, divisions): direction cosines and, for
// gradients, their derivatives.  Computed once per pair (one thread per pair) and broadcast to the
// lanes that assemble T and D from them.
struct RotScalars { double ca, sa, cb, sb, caX, caY, saX, saY, cbX, cbY, cbZ, sbX, sbY, sbZ; int swapped, active; };

__device__ __forceinline__ void rot_scalars(double x, double y, double z, double r, int norb_max, bool derivs, RotScalars &q)
{
    q.active = (norb_max > 1) && (r * r > 2.0e-5);
    q.swapped = 0;
    q.ca = q.sa = q.cb = q.sb = 0.0;
    q.caX = q.caY = q.saX = q.saY = q.cbX = q.cbY = q.cbZ = q.sbX = q.sbY = q.sbZ = 0.0;
    if (!q.active) return;
    q.swapped = fabs(z / r) > 0.99999999;
    if (q.swapped) { double t = x; x = z; z = t; }
    const double b2 = x * x + y * y, b = sqrt(b2);
    q.sb = b / r; q.ca = x / b; q.sa = y / b; q.cb = z / r;
    if (!derivs) return;
    const double r3 = r * r * r;
    q.caX = y * y / (b2 * b); q.caY = -x * y / (b2 * b); q.saX = q.caY; q.saY = x * x / (b2 * b);
    q.cbX = -x * z / r3; q.cbY = -y * z / r3; q.cbZ = b2 / r3;
    q.sbX = x * z * z / (b * r3); q.sbY = y * z * z / (b * r3); q.sbZ = -b * z / r3;
}

__device__ __forceinline__ RotScalars rot_shfl(const RotScalars &q, int src, bool derivs)
{
    RotScalars o;
    const unsigned m = 0xffffffffu;
    o.active = __shfl_sync(m, q.active, src); o.swapped = __shfl_sync(m, q.swapped, src);
    o.ca = __shfl_sync(m, q.ca, src); o.sa = __shfl_sync(m, q.sa, src); o.cb = __shfl_sync(m, q.cb, src); o.sb = __shfl_sync(m, q.sb, src);
    if (derivs) {
        o.caX = __shfl_sync(m, q.caX, src); o.caY = __shfl_sync(m, q.caY, src); o.saX = __shfl_sync(m, q.saX, src);
        o.saY = __shfl_sync(m, q.saY, src); o.cbX = __shfl_sync(m, q.cbX, src); o.cbY = __shfl_sync(m, q.cbY, src);
        o.cbZ = __shfl_sync(m, q.cbZ, src); o.sbX = __shfl_sync(m, q.sbX, src); o.sbY = __shfl_sync(m, q.sbY, src);
        o.sbZ = __shfl_sync(m, q.sbZ, src);
    } else {
        o.caX = o.caY = o.saX = o.saY = o.cbX = o.cbY = o.cbZ = o.sbX = o.sbY = o.sbZ = 0.0;
    }
    return o;
}

// Local-to-molecular rotation of the p shell and its derivatives with respect to the coordinates of
// atom j (MNDOIntegralUtilities_GetTransformationMatrices, MNDOIntegralUtilities.c:449-465 for s/p,
// axes swapped when |z/r| > 0.99999999).  T[a][m]: molecular orbital a (s, pz, px, py), local m
// (s, sigma, pi+, pi-).  Inactive: identity, zero derivatives.
// (R = float: the same assembly from the scalars rounded to FP32, for the mixed method's gradient terms.)
template <typename Real>
__device__ __forceinline__ void rot_assemble(const RotScalars &q, bool derivs, RotationT<Real> &R)
{
    for (int a = 0; a < 4; a++) for (int m = 0; m < 4; m++) {
        R.T[a][m] = (a == m) ? Real(1) : Real(0);
        if (derivs) { R.D[0][a][m] = Real(0); R.D[1][a][m] = Real(0); R.D[2][a][m] = Real(0); }
    }
    R.active = q.active;
    if (!q.active) return;
    const int PZ = 1, PX = 2, PY = 3;
    const Real ca = (Real)q.ca, sa = (Real)q.sa, cb = (Real)q.cb, sb = (Real)q.sb;
    Real T[4][4] = {{1, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    T[PX][1] = ca * sb; T[PX][2] = ca * cb; T[PX][3] = -sa;
    T[PY][1] = sa * sb; T[PY][2] = sa * cb; T[PY][3] = ca;
    T[PZ][1] = cb;      T[PZ][2] = -sb;
    if (q.swapped) for (int c = 0; c < 4; c++) { Real t = T[PX][c]; T[PX][c] = T[PZ][c]; T[PZ][c] = t; }
    for (int a = 0; a < 4; a++) for (int m = 0; m < 4; m++) R.T[a][m] = T[a][m];
    if (!derivs) return;
    const Real caX = (Real)q.caX, caY = (Real)q.caY, saX = (Real)q.saX, saY = (Real)q.saY, cbX = (Real)q.cbX, cbY = (Real)q.cbY;
    const Real cbZ = (Real)q.cbZ, sbX = (Real)q.sbX, sbY = (Real)q.sbY, sbZ = (Real)q.sbZ;
    Real D[3][4][4] = {};
    D[0][PX][1] = caX * sb + ca * sbX; D[0][PX][2] = caX * cb + ca * cbX; D[0][PX][3] = -saX;
    D[0][PY][1] = saX * sb + sa * sbX; D[0][PY][2] = saX * cb + sa * cbX; D[0][PY][3] = caX;
    D[0][PZ][1] = cbX; D[0][PZ][2] = -sbX;
    D[1][PX][1] = caY * sb + ca * sbY; D[1][PX][2] = caY * cb + ca * cbY; D[1][PX][3] = -saY;
    D[1][PY][1] = saY * sb + sa * sbY; D[1][PY][2] = saY * cb + sa * cbY; D[1][PY][3] = caY;
    D[1][PZ][1] = cbY; D[1][PZ][2] = -sbY;
    D[2][PX][1] = ca * sbZ; D[2][PX][2] = ca * cbZ;
    D[2][PY][1] = sa * sbZ; D[2][PY][2] = sa * cbZ;
    D[2][PZ][1] = cbZ; D[2][PZ][2] = -sbZ;
    if (q.swapped) {
        for (int k = 0; k < 3; k++) for (int c = 0; c < 4; c++) { Real t = D[k][PX][c]; D[k][PX][c] = D[k][PZ][c]; D[k][PZ][c] = t; }
        for (int a = 0; a < 4; a++) for (int c = 0; c < 4; c++) { Real t = D[0][a][c]; D[0][a][c] = D[2][a][c]; D[2][a][c] = t; }
    }
    for (int k = 0; k < 3; k++) for (int a = 0; a < 4; a++) for (int m = 0; m < 4; m++) R.D[k][a][m] = D[k][a][m];
}

// Distribution-pair transform element C[ab][mn] (and its derivative) built from T on demand
// (MNDOIntegralUtilities.c:786-840).
__constant__ const int8_t MP_DA[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
__constant__ const int8_t MP_DB[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};

template <typename Real>
__device__ __forceinline__ Real ctrans(const Real (*T)[4], int ab, int mn)
{
    int a = MP_DA[ab], b = MP_DB[ab], m = MP_DA[mn], n = MP_DB[mn];
    if (m == n) return T[a][m] * T[b][m];
    return T[a][m] * T[b][n] + T[a][n] * T[b][m];
}
template <typename Real>
__device__ __forceinline__ Real ctrans_d(const Real (*T)[4], const Real (*D)[4], int ab, int mn)
{
    int a = MP_DA[ab], b = MP_DB[ab], m = MP_DA[mn], n = MP_DB[mn];
    if (m == n) return D[a][m] * T[b][m] + T[a][m] * D[b][m];
    return D[a][m] * T[b][n] + T[a][m] * D[b][n] + D[a][n] * T[b][m] + T[a][n] * D[b][m];
}
