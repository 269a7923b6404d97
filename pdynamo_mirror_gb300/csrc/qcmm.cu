// qcmm.cu - QC/MM point-charge electrostatics (FP64 pair terms, FP32 cutoff prefilter).
//
// Potentials phi_A = sum_m q_m f(r_Am) at the QC atoms and the gradients of E = sum_A q_A phi_A with the
// QC charges held fixed, for
//   model 0  NBModelFull: f = 1 / r over every pair (NBModelFull.c:604-690 potentials, :392-600 gradients);
//   model 1  NBModelABFS: f = cubic spline in r^2 of the switched Delta/Gaussian interaction, zero beyond the
//            outer cutoff (PairwiseInteractionABFS_QCMMPotentials, PairwiseInteraction.c:612;
//            _QCMMGradients, :542; spline evaluation CubicSpline_Evaluate, CubicSpline.c:88).
// The reference walks a cell-grid pair list (13.5 A) and skips pairs beyond the 12 A outer cutoff itself,
// so the result is the cutoff sum over all pairs: here every MM atom is tested (FP32 distance with a
// conservative margin), and only pairs inside the cutoff are evaluated in FP64.
// Coordinates are in Angstrom as the reference evaluates these terms; results are in atomic units.
#include "common.cuh"

struct Spline { int n; const double *x, *y, *h; double r2off, inc; };

// Interval search equivalent to CubicSpline_Evaluate's bisection (largest l with x_l <= v); the knots are
// squares of a uniform r grid, so the FP32 estimate is off by at most one and is corrected exactly.
__device__ __forceinline__ void spline_eval(const Spline &sp, double v, double *f, double *g)
{
    int n = sp.n;
    int l = (int)(sqrtf((float)v) / (float)sp.inc);
    l = max(0, min(l, n - 2));
    while (l > 0 && sp.x[l] > v) l--;
    while (l < n - 2 && sp.x[l + 1] <= v) l++;
    int u = l + 1;
    double d = sp.x[u] - sp.x[l], id = 1.0 / d;
    double s = (v - sp.x[l]) * id, t = (sp.x[u] - v) * id;
    double hl = sp.h[l] * d / 6.0, hu = sp.h[u] * d / 6.0, yl = sp.y[l], yu = sp.y[u];
    *f = t * yl + s * yu + d * (t * (t * t - 1.0) * hl + s * (s * s - 1.0) * hu);
    if (g) *g = (yu - yl) * id + (-(3.0 * t * t - 1.0) * hl + (3.0 * s * s - 1.0) * hu);
}

// pair term: value f (a.u. per unit charges) and df/d(r^2) (per A^2)
__device__ __forceinline__ bool pair_term(int model, const Spline &sp, double r2, double *f, double *g)
{
    if (model == 1) {
        if (r2 > sp.r2off) return false;
        spline_eval(sp, r2, f, g);
        return true;
    }
    double ir = rsqrt(r2);
    *f = ir * (1.0 / PDG_ANGSTROMS_TO_BOHRS);
    if (g) *g = -0.5 * ir * ir * ir * (1.0 / PDG_ANGSTROMS_TO_BOHRS);
    return true;
}

#define QB 256

__global__ void __launch_bounds__(QB) k_qcmm_potentials(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                        const double *__restrict__ mm, const double *__restrict__ q, double *__restrict__ phi)
{
    __shared__ double red[QB / 32];
    int f = blockIdx.x / n_qc, A = blockIdx.x % n_qc;
    const double *xa = qc + ((size_t)f * n_qc + A) * 3;
    const double *xm = mm + (size_t)f * n_mm * 3;
    double ax = xa[0], ay = xa[1], az = xa[2];
    float r2cut = (float)(sp.r2off * (1.0 + 1.0e-4)) + 1.0e-3f;
    double pot = 0.0;
    for (int m = threadIdx.x; m < n_mm; m += QB) {
        double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        if (model == 1) {
            float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            if (fx * fx + fy * fy + fz * fz > r2cut) continue;
        }
        double fv;
        if (pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, nullptr)) pot += q[m] * fv;
    }
    double t = block_sum(pot, red);
    if (threadIdx.x == 0) phi[(size_t)f * n_qc + A] = t;
}

// dE/dx_A = sum_m 2 q_A q_m f'(r^2) (x_A - x_m), converted from per-A to per-Bohr.
__global__ void __launch_bounds__(QB) k_qcmm_grad_qc(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q,
                                                     const double *__restrict__ qcq, double *__restrict__ gqc)
{
    __shared__ double red[QB / 32];
    int f = blockIdx.x / n_qc, A = blockIdx.x % n_qc;
    const double *xa = qc + ((size_t)f * n_qc + A) * 3;
    const double *xm = mm + (size_t)f * n_mm * 3;
    double ax = xa[0], ay = xa[1], az = xa[2], qa = qcq[(size_t)f * n_qc + A];
    float r2cut = (float)(sp.r2off * (1.0 + 1.0e-4)) + 1.0e-3f;
    double g[3] = { 0, 0, 0 };
    for (int m = threadIdx.x; m < n_mm; m += QB) {
        double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        if (model == 1) {
            float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            if (fx * fx + fy * fy + fz * fz > r2cut) continue;
        }
        double fv, gv;
        if (!pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, &gv)) continue;
        double s = 2.0 * qa * q[m] * gv / PDG_ANGSTROMS_TO_BOHRS;
        g[0] += s * dx; g[1] += s * dy; g[2] += s * dz;
    }
    for (int k = 0; k < 3; k++) {
        double t = block_sum(g[k], red);
        if (threadIdx.x == 0) gqc[((size_t)f * n_qc + A) * 3 + k] = t;
    }
}

__global__ void __launch_bounds__(QB) k_qcmm_grad_mm(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q,
                                                     const double *__restrict__ qcq, double *__restrict__ gmm)
{
    extern __shared__ double sq[];   // QC coordinates and charges of this frame
    int blocks_per_frame = (n_mm + QB - 1) / QB;
    int f = blockIdx.x / blocks_per_frame, m = (blockIdx.x % blocks_per_frame) * QB + threadIdx.x;
    for (int k = threadIdx.x; k < n_qc; k += QB) {
        sq[4 * k] = qc[((size_t)f * n_qc + k) * 3]; sq[4 * k + 1] = qc[((size_t)f * n_qc + k) * 3 + 1];
        sq[4 * k + 2] = qc[((size_t)f * n_qc + k) * 3 + 2]; sq[4 * k + 3] = qcq[(size_t)f * n_qc + k];
    }
    __syncthreads();
    if (m >= n_mm) return;
    const double *xm = mm + ((size_t)f * n_mm + m) * 3;
    double mx = xm[0], my = xm[1], mz = xm[2], qm = q[m];
    float r2cut = (float)(sp.r2off * (1.0 + 1.0e-4)) + 1.0e-3f;
    double g[3] = { 0, 0, 0 };
    for (int A = 0; A < n_qc; A++) {
        double dx = sq[4 * A] - mx, dy = sq[4 * A + 1] - my, dz = sq[4 * A + 2] - mz;
        if (model == 1) {
            float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            if (fx * fx + fy * fy + fz * fz > r2cut) continue;
        }
        double fv, gv;
        if (!pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, &gv)) continue;
        double s = 2.0 * sq[4 * A + 3] * qm * gv / PDG_ANGSTROMS_TO_BOHRS;
        g[0] -= s * dx; g[1] -= s * dy; g[2] -= s * dz;
    }
    double *o = gmm + ((size_t)f * n_mm + m) * 3;
    o[0] = g[0]; o[1] = g[1]; o[2] = g[2];
}

static Spline make_spline(int n, const double *knots, double cutoff)
{
    Spline s;
    s.n = n; s.x = knots; s.y = knots + n; s.h = knots + 2 * n;
    s.r2off = cutoff * cutoff; s.inc = (n > 1) ? cutoff / (double)(n - 1) : 1.0;
    return s;
}

int launch_qcmm_potentials(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                           const double *q, int n_knots, const double *knots, double cutoff, double *phi, cudaStream_t st)
{
    if (n_frames <= 0 || n_qc <= 0) return 0;
    Spline sp = make_spline(n_knots, knots, cutoff);
    k_qcmm_potentials<<<n_frames * n_qc, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, phi);
    return 0;
}

int launch_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                          const double *q, const double *qcq, int n_knots, const double *knots, double cutoff,
                          double *gqc, double *gmm, cudaStream_t st)
{
    if (n_frames <= 0 || n_qc <= 0) return 0;
    Spline sp = make_spline(n_knots, knots, cutoff);
    k_qcmm_grad_qc<<<n_frames * n_qc, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gqc);
    if (n_mm > 0) {
        int bpf = (n_mm + QB - 1) / QB;
        size_t sm = sizeof(double) * 4 * (size_t)n_qc;
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_qcmm_grad_mm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_qcmm_grad_mm<<<n_frames * bpf, QB, sm, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gmm);
    }
    return 0;
}
