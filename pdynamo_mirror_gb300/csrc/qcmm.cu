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

// GB300 runs FP64 at one warp instruction per ~64 cycles per sub-partition whatever the active lanes, so
// the FP32 cutoff test runs on FP32 copies of the MM coordinates staged in shared memory, and the pairs that
// pass are queued per warp and evaluated in FP64 thirty-two at a time: only ~6 % of the QC x MM pairs of a
// 12 A cutoff in a 50 A box are inside, and no warp runs the spline for one lane.  The queue keeps the scan
// order, so every sum is taken in a fixed order (deterministic).
#define QW 8              // QC atoms per block, one warp each
#define QB (QW * 32)
#define MCH 1024          // MM atoms staged per chunk

__device__ __forceinline__ float cutoff_r2(int model, const Spline &sp)
{
    return model == 1 ? (float)(sp.r2off * (1.0 + 1.0e-4)) + 1.0e-3f : __int_as_float(0x7f800000);
}

// Scan this frame's MM atoms for the warp's QC atom; call body(m) for every MM atom that passes the FP32
// test, on all 32 lanes at once (lane k handles queue entry k), then on the final partial batch.
template <typename Body>
__device__ __forceinline__ void scan_mm(int n_mm, const double *__restrict__ xm, float fax, float fay, float faz, float r2cut,
                                        bool live, float4 *sxm, int *queue, Body body)
{
    const int lane = threadIdx.x & 31;
    int qn = 0;
    for (int c0 = 0; c0 < n_mm; c0 += MCH) {
        const int cn = min(MCH, n_mm - c0);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += QB) {
            const double *p = xm + 3 * (size_t)(c0 + k);
            sxm[k] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.0f);
        }
        __syncthreads();
        if (!live) continue;
        for (int k0 = 0; k0 < cn; k0 += 32) {
            const int k = k0 + lane;
            bool in = false;
            if (k < cn) {
                const float4 p = sxm[k];
                const float dx = fax - p.x, dy = fay - p.y, dz = faz - p.z;
                in = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2cut;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (in) queue[qn + __popc(bal & ((1u << lane) - 1u))] = c0 + k;
            qn += __popc(bal);
            __syncwarp();
            if (qn >= 32) {
                body(queue[lane]);
                const int rest = qn - 32;
                const int carry = lane < rest ? queue[32 + lane] : 0;
                __syncwarp();
                if (lane < rest) queue[lane] = carry;
                __syncwarp();
                qn = rest;
            }
        }
    }
    if (live && lane < qn) body(queue[lane]);
}

__global__ void __launch_bounds__(QB) k_qcmm_potentials(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                        const double *__restrict__ mm, const double *__restrict__ q, double *__restrict__ phi)
{
    __shared__ float4 sxm[MCH];
    __shared__ int queue[QW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
    const double *xm = mm + (size_t)f * n_mm * 3;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (live) { const double *xa = qc + ((size_t)f * n_qc + A) * 3; ax = xa[0]; ay = xa[1]; az = xa[2]; }
    double pot = 0.0;
    scan_mm(n_mm, xm, (float)ax, (float)ay, (float)az, cutoff_r2(model, sp), live, sxm, queue[w], [&](int m) {
        const double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        double fv;
        if (pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, nullptr)) pot += q[m] * fv;
    });
    pot = warp_sum(pot);
    if (live && lane == 0) phi[(size_t)f * n_qc + A] = pot;
}

// dE/dx_A = sum_m 2 q_A q_m f'(r^2) (x_A - x_m), converted from per-A to per-Bohr.
__global__ void __launch_bounds__(QB) k_qcmm_grad_qc(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q,
                                                     const double *__restrict__ qcq, double *__restrict__ gqc)
{
    __shared__ float4 sxm[MCH];
    __shared__ int queue[QW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
    const double *xm = mm + (size_t)f * n_mm * 3;
    double ax = 0.0, ay = 0.0, az = 0.0, qa = 0.0;
    if (live) { const double *xa = qc + ((size_t)f * n_qc + A) * 3; ax = xa[0]; ay = xa[1]; az = xa[2]; qa = qcq[(size_t)f * n_qc + A]; }
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    scan_mm(n_mm, xm, (float)ax, (float)ay, (float)az, cutoff_r2(model, sp), live, sxm, queue[w], [&](int m) {
        const double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        double fv, gv;
        if (!pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, &gv)) return;
        const double s = 2.0 * qa * q[m] * gv / PDG_ANGSTROMS_TO_BOHRS;
        g0 += s * dx; g1 += s * dy; g2 += s * dz;
    });
    g0 = warp_sum(g0); g1 = warp_sum(g1); g2 = warp_sum(g2);
    if (live && lane == 0) { double *o = gqc + ((size_t)f * n_qc + A) * 3; o[0] = g0; o[1] = g1; o[2] = g2; }
}

// MM side: a block takes 256 MM atoms of one frame.  An FP32 pass (one thread per atom) marks the atoms within
// the cutoff of any QC atom, packs them (block prefix in atom order) and writes zero for the others; the warps
// then take the packed atoms one at a time (w, w + 8, ...): for its atom a warp tests the QC atoms 32 at a time
// in FP32, queues the ones inside the cutoff and evaluates the queue in FP64 thirty-two pairs at a time (as the
// QC side does), so that no FP64 pass runs for a few lanes; lane partial sums are reduced in a fixed order.
#define MB 256
__global__ void __launch_bounds__(MB) k_qcmm_grad_mm(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q,
                                                     const double *__restrict__ qcq, double *__restrict__ gmm)
{
    extern __shared__ double sq[];   // QC atoms: x, y, z, charge (doubles), then x, y, z (floats)
    __shared__ int queue[MB / 32][64], wcount[MB / 32], near_list[MB];
    float *sf = (float *)(sq + 4 * (size_t)n_qc);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int blocks_per_frame = (n_mm + MB - 1) / MB;
    const int f = blockIdx.x / blocks_per_frame, base = (blockIdx.x % blocks_per_frame) * MB;
    for (int k = threadIdx.x; k < n_qc; k += MB) {
        const double *x = qc + ((size_t)f * n_qc + k) * 3;
        sq[4 * k] = x[0]; sq[4 * k + 1] = x[1]; sq[4 * k + 2] = x[2]; sq[4 * k + 3] = qcq[(size_t)f * n_qc + k];
        sf[3 * k] = (float)x[0]; sf[3 * k + 1] = (float)x[1]; sf[3 * k + 2] = (float)x[2];
    }
    __syncthreads();
    const float r2cut = cutoff_r2(model, sp);
    bool near = false;
    if (base + (int)threadIdx.x < n_mm) {
        const int m = base + threadIdx.x;
        const double *xm = mm + ((size_t)f * n_mm + m) * 3;
        const float fx = (float)xm[0], fy = (float)xm[1], fz = (float)xm[2];
        for (int A = 0; A < n_qc && !near; A++) {
            const float dx = sf[3 * A] - fx, dy = sf[3 * A + 1] - fy, dz = sf[3 * A + 2] - fz;
            near = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2cut;
        }
        if (!near) { double *o = gmm + ((size_t)f * n_mm + m) * 3; o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; }
    }
    const unsigned nbal = __ballot_sync(0xffffffffu, near);
    if (lane == 0) wcount[w] = __popc(nbal);
    __syncthreads();
    int off = 0, total = 0;
    for (int k = 0; k < MB / 32; k++) { if (k < w) off += wcount[k]; total += wcount[k]; }
    if (near) near_list[off + __popc(nbal & ((1u << lane) - 1u))] = base + threadIdx.x;
    __syncthreads();
    int *qw = queue[w];
    for (int k = w; k < total; k += MB / 32) {
        const int m = near_list[k];
        const double *xm = mm + ((size_t)f * n_mm + m) * 3;
        const double mx = xm[0], my = xm[1], mz = xm[2], qm = q[m];
        const float fx = (float)mx, fy = (float)my, fz = (float)mz;
        double g0 = 0.0, g1 = 0.0, g2 = 0.0;
        auto body = [&](int A) {
            const double dx = sq[4 * A] - mx, dy = sq[4 * A + 1] - my, dz = sq[4 * A + 2] - mz;
            double fv, gv;
            if (!pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, &gv)) return;
            const double s = 2.0 * sq[4 * A + 3] * qm * gv / PDG_ANGSTROMS_TO_BOHRS;
            g0 -= s * dx; g1 -= s * dy; g2 -= s * dz;
        };
        int qn = 0;
        for (int A0 = 0; A0 < n_qc; A0 += 32) {
            const int A = A0 + lane;
            bool in = false;
            if (A < n_qc) {
                const float ex = sf[3 * A] - fx, ey = sf[3 * A + 1] - fy, ez = sf[3 * A + 2] - fz;
                in = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= r2cut;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (in) qw[qn + __popc(bal & ((1u << lane) - 1u))] = A;
            qn += __popc(bal);
            __syncwarp();
            if (qn >= 32) {
                body(qw[lane]);
                const int rest = qn - 32;
                const int carry = lane < rest ? qw[32 + lane] : 0;
                __syncwarp();
                if (lane < rest) qw[lane] = carry;
                __syncwarp();
                qn = rest;
            }
        }
        if (lane < qn) body(qw[lane]);
        __syncwarp();
        g0 = warp_sum(g0); g1 = warp_sum(g1); g2 = warp_sum(g2);
        if (lane == 0) { double *o = gmm + ((size_t)f * n_mm + m) * 3; o[0] = g0; o[1] = g1; o[2] = g2; }
    }
}

// ---------------------------------------------------------------------------------------------------
// FP32 pair terms for the gradients (the mixed method; model | PDG_QCMM_FP32_PAIRS).  A gradient pair term is
// up to ~0.1 Eh/Bohr at the closest contacts; in FP32 (coordinates, r^2 and the spline, with the knot value
// differences formed in FP64) each carries ~1e-7 relative, and the per-atom sums stay near 1e-7 Eh/Bohr, two
// orders inside the 1e-5 gate.  Lane partial sums are FP32, the sums over lanes FP64.
// Coordinates, charges and knots are staged in FP32 shared memory and the queues carry FP32 coordinates, so no
// FP64 instruction runs per pair.
#define KMAX32 1024
// knots x, second derivatives h, and the value differences y_{l+1} - y_l taken in FP64 before rounding (the
// differences of neighbouring FP32 values would lose ~1e-5 relative where 1/r is large)
struct Knots32 { float x[KMAX32], dy[KMAX32], h[KMAX32]; };

__device__ __forceinline__ void stage_knots32(const Spline &sp, Knots32 &k)
{
    for (int i = threadIdx.x; i < sp.n; i += blockDim.x) {
        k.x[i] = (float)sp.x[i]; k.h[i] = (float)sp.h[i];
        k.dy[i] = i + 1 < sp.n ? (float)(sp.y[i + 1] - sp.y[i]) : 0.0f;
    }
}

// df/d(r^2) in FP32 (per A^2, a.u. per unit charges); false beyond the cutoff
__device__ __forceinline__ bool pair_grad32(int model, const Spline &sp, const Knots32 &k, float r2, float &g)
{
    if (model == 1) {
        if (r2 > (float)sp.r2off) return false;
        const int n = sp.n;
        int l = (int)(sqrtf(r2) / (float)sp.inc);
        l = max(0, min(l, n - 2));
        while (l > 0 && k.x[l] > r2) l--;
        while (l < n - 2 && k.x[l + 1] <= r2) l++;
        const int u = l + 1;
        const float d = k.x[u] - k.x[l], id = 1.0f / d;
        const float s = (r2 - k.x[l]) * id, t = (k.x[u] - r2) * id;
        const float hl = k.h[l] * d * (1.0f / 6.0f), hu = k.h[u] * d * (1.0f / 6.0f);
        g = k.dy[l] * id + (-(3.0f * t * t - 1.0f) * hl + (3.0f * s * s - 1.0f) * hu);
        return true;
    }
    const float ir = rsqrtf(r2);
    g = -0.5f * ir * ir * ir * (float)(1.0 / PDG_ANGSTROMS_TO_BOHRS);
    return true;
}

__global__ void __launch_bounds__(QB) k_qcmm_grad_qc32(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                       const double *__restrict__ mm, const double *__restrict__ q,
                                                       const double *__restrict__ qcq, double *__restrict__ gqc)
{
    __shared__ float4 sxm[MCH];       // MM atoms of the chunk: x, y, z, charge
    __shared__ float4 queue[QW][64];
    __shared__ Knots32 kn;
    if (model == 1) stage_knots32(sp, kn);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
    const double *xm = mm + (size_t)f * n_mm * 3;
    float ax = 0.f, ay = 0.f, az = 0.f, qa = 0.f;
    if (live) { const double *xa = qc + ((size_t)f * n_qc + A) * 3; ax = (float)xa[0]; ay = (float)xa[1]; az = (float)xa[2]; qa = (float)qcq[(size_t)f * n_qc + A]; }
    const float r2cut = cutoff_r2(model, sp), sc = (float)(2.0 / PDG_ANGSTROMS_TO_BOHRS);
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
    float4 *qw = queue[w];
    auto body = [&](const float4 p) {
        const float dx = ax - p.x, dy = ay - p.y, dz = az - p.z;
        float gv;
        if (!pair_grad32(model, sp, kn, fmaf(dx, dx, fmaf(dy, dy, dz * dz)), gv)) return;
        const float s = sc * qa * p.w * gv;
        g0 = fmaf(s, dx, g0); g1 = fmaf(s, dy, g1); g2 = fmaf(s, dz, g2);
    };
    int qn = 0;
    for (int c0 = 0; c0 < n_mm; c0 += MCH) {
        const int cn = min(MCH, n_mm - c0);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += QB) {
            const double *p = xm + 3 * (size_t)(c0 + k);
            sxm[k] = make_float4((float)p[0], (float)p[1], (float)p[2], (float)q[c0 + k]);
        }
        __syncthreads();
        if (!live) continue;
        for (int k0 = 0; k0 < cn; k0 += 32) {
            const int k = k0 + lane;
            bool in = false;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < cn) {
                p = sxm[k];
                const float dx = ax - p.x, dy = ay - p.y, dz = az - p.z;
                in = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2cut;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (in) qw[qn + __popc(bal & ((1u << lane) - 1u))] = p;
            qn += __popc(bal);
            __syncwarp();
            if (qn >= 32) {
                body(qw[lane]);
                const int rest = qn - 32;
                const float4 carry = lane < rest ? qw[32 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
                __syncwarp();
                if (lane < rest) qw[lane] = carry;
                __syncwarp();
                qn = rest;
            }
        }
    }
    if (live && lane < qn) body(qw[lane]);
    const double d0 = warp_sum((double)g0), d1 = warp_sum((double)g1), d2 = warp_sum((double)g2);
    if (live && lane == 0) { double *o = gqc + ((size_t)f * n_qc + A) * 3; o[0] = d0; o[1] = d1; o[2] = d2; }
}

__global__ void __launch_bounds__(MB) k_qcmm_grad_mm32(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                       const double *__restrict__ mm, const double *__restrict__ q,
                                                       const double *__restrict__ qcq, double *__restrict__ gmm)
{
    extern __shared__ float4 sa[];    // QC atoms: x, y, z, charge
    __shared__ int queue[MB / 32][64], wcount[MB / 32], near_list[MB];
    __shared__ Knots32 kn;
    if (model == 1) stage_knots32(sp, kn);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int blocks_per_frame = (n_mm + MB - 1) / MB;
    const int f = blockIdx.x / blocks_per_frame, base = (blockIdx.x % blocks_per_frame) * MB;
    for (int k = threadIdx.x; k < n_qc; k += MB) {
        const double *x = qc + ((size_t)f * n_qc + k) * 3;
        sa[k] = make_float4((float)x[0], (float)x[1], (float)x[2], (float)qcq[(size_t)f * n_qc + k]);
    }
    __syncthreads();
    const float r2cut = cutoff_r2(model, sp), sc = (float)(2.0 / PDG_ANGSTROMS_TO_BOHRS);
    bool near = false;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    if (base + (int)threadIdx.x < n_mm) {
        const int m = base + threadIdx.x;
        const double *xm = mm + ((size_t)f * n_mm + m) * 3;
        fx = (float)xm[0]; fy = (float)xm[1]; fz = (float)xm[2];
        for (int A = 0; A < n_qc && !near; A++) {
            const float dx = sa[A].x - fx, dy = sa[A].y - fy, dz = sa[A].z - fz;
            near = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2cut;
        }
        if (!near) { double *o = gmm + ((size_t)f * n_mm + m) * 3; o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; }
    }
    const unsigned nbal = __ballot_sync(0xffffffffu, near);
    if (lane == 0) wcount[w] = __popc(nbal);
    __syncthreads();
    int off = 0, total = 0;
    for (int k = 0; k < MB / 32; k++) { if (k < w) off += wcount[k]; total += wcount[k]; }
    if (near) near_list[off + __popc(nbal & ((1u << lane) - 1u))] = base + threadIdx.x;
    __syncthreads();
    int *qw = queue[w];
    for (int k = w; k < total; k += MB / 32) {
        const int m = near_list[k];
        const double *xm = mm + ((size_t)f * n_mm + m) * 3;
        const float mx = (float)xm[0], my = (float)xm[1], mz = (float)xm[2], qm = (float)q[m];
        float g0 = 0.f, g1 = 0.f, g2 = 0.f;
        auto body = [&](int A) {
            const float4 a = sa[A];
            const float dx = a.x - mx, dy = a.y - my, dz = a.z - mz;
            float gv;
            if (!pair_grad32(model, sp, kn, fmaf(dx, dx, fmaf(dy, dy, dz * dz)), gv)) return;
            const float s = sc * a.w * qm * gv;
            g0 = fmaf(-s, dx, g0); g1 = fmaf(-s, dy, g1); g2 = fmaf(-s, dz, g2);
        };
        int qn = 0;
        for (int A0 = 0; A0 < n_qc; A0 += 32) {
            const int A = A0 + lane;
            bool in = false;
            if (A < n_qc) {
                const float4 a = sa[A];
                const float ex = a.x - mx, ey = a.y - my, ez = a.z - mz;
                in = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= r2cut;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (in) qw[qn + __popc(bal & ((1u << lane) - 1u))] = A;
            qn += __popc(bal);
            __syncwarp();
            if (qn >= 32) {
                body(qw[lane]);
                const int rest = qn - 32;
                const int carry = lane < rest ? qw[32 + lane] : 0;
                __syncwarp();
                if (lane < rest) qw[lane] = carry;
                __syncwarp();
                qn = rest;
            }
        }
        if (lane < qn) body(qw[lane]);
        __syncwarp();
        const double d0 = warp_sum((double)g0), d1 = warp_sum((double)g1), d2 = warp_sum((double)g2);
        if (lane == 0) { double *o = gmm + ((size_t)f * n_mm + m) * 3; o[0] = d0; o[1] = d1; o[2] = d2; }
    }
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
    const int groups = (n_qc + QW - 1) / QW;
    k_qcmm_potentials<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, phi);
    return 0;
}

int launch_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                          const double *q, const double *qcq, int n_knots, const double *knots, double cutoff,
                          double *gqc, double *gmm, cudaStream_t st)
{
    if (n_frames <= 0 || n_qc <= 0) return 0;
    const bool f32 = (model & PDG_QCMM_FP32_PAIRS) != 0 && n_knots <= KMAX32;
    model &= ~PDG_QCMM_FP32_PAIRS;
    Spline sp = make_spline(n_knots, knots, cutoff);
    if (f32) {
        const int groups = (n_qc + QW - 1) / QW;
        k_qcmm_grad_qc32<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gqc);
        if (n_mm > 0 && gmm) {
            const int bpf = (n_mm + MB - 1) / MB;
            const size_t sm = sizeof(float4) * (size_t)n_qc;
            if (sm > 8 * 1024) cudaFuncSetAttribute(k_qcmm_grad_mm32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_qcmm_grad_mm32<<<n_frames * bpf, MB, sm, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gmm);
        }
        return 0;
    }
    const int groups = (n_qc + QW - 1) / QW;
    k_qcmm_grad_qc<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gqc);
    if (n_mm > 0 && gmm) {
        const int bpf = (n_mm + MB - 1) / MB;
        const size_t sm = sizeof(double) * 4 * (size_t)n_qc + sizeof(float) * 3 * (size_t)n_qc;
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_qcmm_grad_mm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_qcmm_grad_mm<<<n_frames * bpf, MB, sm, st>>>(model, sp, n_qc, n_mm, qc, mm, q, qcq, gmm);
    }
    return 0;
}
