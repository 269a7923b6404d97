// overlap.cuh - STO-6G overlap of two sp shells and its derivative in closed form.
//
// For primitives a (on atom i) and b (on atom j), g = a + b, AB = R_j - R_i, the s/p overlap blocks of
// GaussianBasis_2Overlap (GaussianBasisCore.c:469, orbital order s, pz, px, py) are
//     ss = s0,  p_k s = (b/g) AB_k s0,  s p_k = -(a/g) AB_k s0,  p_k p_l = (-(ab/g^2) AB_k AB_l + delta_kl / 2g) s0,
// with s0 = c_a c_b (pi/g)^(3/2) exp(-(ab/g) |AB|^2).  So every element of a shell pair's block is AB
// times a few radial sums over the primitive pairs (F), and the derivative with respect to R_i
// (GaussianBasis_2OverlapD, :570) needs the same sums weighted by 2ab/g (D).  The primitive constants are
// tabulated per ordered element pair on the host; on the device one exp per primitive pair remains.
// Primitive pairs with (ab/g)|AB|^2 above 18 ln 10 are skipped, as the reference does (GaussianBasis.h:43).
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

#define OV_REC 4   // per primitive pair: ab/g, pre * w1, pre * w2, type
enum { OV_SS = 0, OV_PS = 1, OV_SP = 2, OV_PP = 3 };
#define PRIMITIVE_OVERLAP_TOLERANCE (2.30258509299405 * 18.0)

// Host: append the records of the ordered element pair (A holds atom i's basis, B atom j's).
inline void overlap_records(const double *A, const double *B, std::vector<double> &out)
{
    const int nsa = (int)A[PDG_E_NSHELL], nsb = (int)B[PDG_E_NSHELL];
    const int kinds[4][3] = { { OV_SS, 0, 0 }, { OV_PS, 1, 0 }, { OV_SP, 0, 1 }, { OV_PP, 1, 1 } };
    for (const auto &k : kinds) {
        const int ty = k[0], sa = k[1], sb = k[2];
        if (sa >= nsa || sb >= nsb) continue;
        const int npa = (int)A[sa ? PDG_E_NPRIM_P : PDG_E_NPRIM_S], npb = (int)B[sb ? PDG_E_NPRIM_P : PDG_E_NPRIM_S];
        for (int p = 0; p < npa; p++)
            for (int q = 0; q < npb; q++) {
                const double a = A[(sa ? PDG_E_EXP_P : PDG_E_EXP_S) + p], b = B[(sb ? PDG_E_EXP_P : PDG_E_EXP_S) + q], g = a + b;
                const double abg = a * b / g, tg = M_PI / g;
                const double pre = A[(sa ? PDG_E_CCBF_P : PDG_E_CCBF_S) + p] * B[(sb ? PDG_E_CCBF_P : PDG_E_CCBF_S) + q] * tg * sqrt(tg);
                const double w1 = ty == OV_SS ? 1.0 : ty == OV_PS ? b / g : ty == OV_SP ? a / g : abg / g;
                const double w2 = ty == OV_PP ? 0.5 / g : 0.0;
                out.push_back(abg); out.push_back(pre * w1); out.push_back(pre * w2); out.push_back((double)ty);
            }
    }
}

// Radial sums of one atom pair: F[0..4] = ss, ps, sp, pp(AB AB), pp(delta); D[0..4] their 2ab/g-weighted
// companions (derivs only).  Primitive pairs are spread over the lanes; `used` (bit k = sum k) selects the
// sums the pair's shells need, and only those are warp-reduced.
__device__ __forceinline__ double ov_exp(double x) { return exp(x); }
__device__ __forceinline__ float ov_exp(float x) { return __expf(x); }
__device__ __forceinline__ float warp_sum_r(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_r(double v) { return warp_sum(v); }

// (Real = float: the records rounded to FP32 and the FP32 exponential, for the mixed method's gradients.)
template <typename Real>
__device__ __forceinline__ void overlap_sums(const Real *__restrict__ rec, int nrec, Real R2, bool derivs, int used,
                                             Real *F, Real *D)
{
    const int lane = threadIdx.x & 31;
    Real f0 = 0, f1 = 0, f2 = 0, f3 = 0, f4 = 0, d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0;
    for (int t = lane; t < nrec; t += 32) {
        const Real *r = rec + OV_REC * t;
        const Real abg = r[0], fac = abg * R2;
        const Real e = fac > (Real)PRIMITIVE_OVERLAP_TOLERANCE ? Real(0) : ov_exp(-fac);
        const int ty = (int)r[3];
        const Real t1 = r[1] * e, t2 = r[2] * e;
        f0 += ty == OV_SS ? t1 : Real(0); f1 += ty == OV_PS ? t1 : Real(0); f2 += ty == OV_SP ? t1 : Real(0); f3 += ty == OV_PP ? t1 : Real(0);
        f4 += t2;
        if (derivs) {
            const Real a2 = abg + abg, u1 = a2 * t1;
            d0 += ty == OV_SS ? u1 : Real(0); d1 += ty == OV_PS ? u1 : Real(0); d2 += ty == OV_SP ? u1 : Real(0); d3 += ty == OV_PP ? u1 : Real(0);
            d4 = fma(a2, t2, d4);
        }
    }
    const Real fl[5] = { f0, f1, f2, f3, f4 }, dl[5] = { d0, d1, d2, d3, d4 };
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int bit = k < 4 ? k : 3;
        F[k] = (used >> bit & 1) ? warp_sum_r(fl[k]) : Real(0);
        D[k] = (derivs && (used >> bit & 1)) ? warp_sum_r(dl[k]) : Real(0);
    }
}

// Cartesian axis of orbital o (1 pz, 2 px, 3 py).
__device__ __forceinline__ int ov_axis(int o) { return o == 1 ? 2 : o - 2; }

// Overlap element S_ab (a on i, b on j) from the radial sums.
__device__ __forceinline__ double overlap_element(int a, int b, const double *AB, const double *F)
{
    if (a == 0 && b == 0) return F[0];
    if (b == 0) return AB[ov_axis(a)] * F[1];
    if (a == 0) return -AB[ov_axis(b)] * F[2];
    return -AB[ov_axis(a)] * AB[ov_axis(b)] * F[3] + (a == b ? F[4] : 0.0);
}

// sum_ab W_ab dS_ab / dR_i,k for a weight matrix W (W[a*4+b], a < noi, b < noj), from the radial sums.
template <typename Real>
__device__ __forceinline__ void overlap_gradient(const Real *W, int noi, int noj, const Real *AB, const Real *F,
                                                 const Real *D, Real *g)
{
    const int ox[3] = { 2, 3, 1 };   // orbital of axis k: x -> px, y -> py, z -> pz
    Real radial = W[0] * D[0];
    Real wps[3] = { 0, 0, 0 }, wsp[3] = { 0, 0, 0 }, u[3] = { 0, 0, 0 }, v[3] = { 0, 0, 0 };
    if (noi > 1) {
        Real s = 0;
        for (int k = 0; k < 3; k++) { wps[k] = W[ox[k] * 4]; s += wps[k] * AB[k]; }
        radial += s * D[1];
    }
    if (noj > 1) {
        Real s = 0;
        for (int k = 0; k < 3; k++) { wsp[k] = W[ox[k]]; s += wsp[k] * AB[k]; }
        radial -= s * D[2];
    }
    if (noi > 1 && noj > 1) {
        Real q = 0, tr = 0;
        for (int k = 0; k < 3; k++) {
            for (int l = 0; l < 3; l++) { const Real w = W[ox[k] * 4 + ox[l]]; u[k] += w * AB[l]; v[l] += w * AB[k]; }
            tr += W[ox[k] * 4 + ox[k]];
        }
        for (int k = 0; k < 3; k++) q += AB[k] * u[k];
        radial += -q * D[3] + tr * D[4];
    }
    for (int k = 0; k < 3; k++) g[k] = AB[k] * radial - wps[k] * F[1] + wsp[k] * F[2] + (u[k] + v[k]) * F[3];
}

// ---- Tabulated radial sums (the mixed method).  The five sums F_k(R) = sum_t w_kt exp(-(ab/g)_t R^2) of an ordered
// element pair are smooth in R, so they are tabulated once per system at nodes R_n = n h (h = 0.005 Bohr, out to the
// distance at which every primitive pair falls below the tolerance) with their exact derivatives, and evaluated by
// cubic Hermite interpolation: error <= h^4 max|F''''| / 384 (~1e-11 of the sums at bonding distances; the derivative
// ~1e-8), against 36-144 FP64 exponentials per pair.  Node layout: F_0..F_4, dF_0/dR..dF_4/dR (10 doubles).
#define OV_TAB_H 0.005
#define OV_TAB_NODE 10

// Host: append the table of records rec[0 .. nrec) (OV_REC each); returns the node count.
inline int overlap_table(const double *rec, int nrec, std::vector<double> &out)
{
    double abg_min = 1e300;
    for (int t = 0; t < nrec; t++) abg_min = std::min(abg_min, rec[OV_REC * t]);
    if (nrec == 0) abg_min = 1.0;
    const double rmax = std::sqrt(PRIMITIVE_OVERLAP_TOLERANCE / abg_min);
    const int n = (int)std::ceil(rmax / OV_TAB_H) + 2;
    for (int i = 0; i < n; i++) {
        const double R = i * OV_TAB_H, R2 = R * R;
        double F[5] = { 0, 0, 0, 0, 0 }, G[5] = { 0, 0, 0, 0, 0 };
        for (int t = 0; t < nrec; t++) {
            const double *q = rec + OV_REC * t;
            const double fac = q[0] * R2;
            if (fac > PRIMITIVE_OVERLAP_TOLERANCE) continue;
            const double e = std::exp(-fac), d = -2.0 * q[0] * R * e;
            const int ty = (int)q[3];
            F[ty] += q[1] * e;  G[ty] += q[1] * d;
            F[4] += q[2] * e;   G[4] += q[2] * d;
        }
        for (int k = 0; k < 5; k++) out.push_back(F[k]);
        for (int k = 0; k < 5; k++) out.push_back(G[k]);
    }
    return n;
}

// Device: F[0..4] and D[0..4] (D_k = sum 2 (ab/g) w e = -(dF_k/dR) / R; D may be null) of ordered element pair eo at
// distance R from the table; zero beyond it.
__device__ __forceinline__ void overlap_sums_table(const DeviceSystem &s, int eo, double R, double *F, double *D)
{
    const double u = R * s.ovl_tab_inv_h;
    const int i = (int)u, n = s.ovl_tab_n[eo];
    if (i >= n - 1) {
        for (int k = 0; k < 5; k++) { F[k] = 0.0; if (D) D[k] = 0.0; }
        return;
    }
    const double t = u - (double)i, t2 = t * t, t3 = t2 * t;
    const double h00 = 2.0 * t3 - 3.0 * t2 + 1.0, h10 = (t3 - 2.0 * t2 + t) * OV_TAB_H;
    const double h01 = 3.0 * t2 - 2.0 * t3, h11 = (t3 - t2) * OV_TAB_H;
    const double *a = s.ovl_tab + s.ovl_tab_off[eo] + (size_t)OV_TAB_NODE * i, *b = a + OV_TAB_NODE;
#pragma unroll
    for (int k = 0; k < 5; k++) F[k] = h00 * a[k] + h10 * a[5 + k] + h01 * b[k] + h11 * b[5 + k];
    if (D) {
        const double g00 = (6.0 * t2 - 6.0 * t) * s.ovl_tab_inv_h, g10 = 3.0 * t2 - 4.0 * t + 1.0;
        const double g01 = (6.0 * t - 6.0 * t2) * s.ovl_tab_inv_h, g11 = 3.0 * t2 - 2.0 * t;
        const double ir = 1.0 / R;
#pragma unroll
        for (int k = 0; k < 5; k++) D[k] = -(g00 * a[k] + g10 * a[5 + k] + g01 * b[k] + g11 * b[5 + k]) * ir;
    }
}
