// qcmm.cu - QC/MM point-charge electrostatics (FP64 pair terms, FP32 cutoff prefilter).
//
// Potentials phi_A = sum_m q_m f(r_Am) at the QC atoms and the gradients of E = sum_A q_A phi_A with the
// QC charges held fixed, for
//   model 0  NBModelFull: f = 1 / r over every pair (NBModelFull.c:604-690 potentials, :392-600 gradients);
//   model 1  NBModelABFS: f = cubic spline in r^2 of the switched Delta/Gaussian interaction, zero beyond the
//            outer cutoff (PairwiseInteractionABFS_QCMMPotentials, PairwiseInteraction.c:612;
//            _QCMMGradients, :542; spline evaluation CubicSpline_Evaluate, CubicSpline.c:88).
// The reference walks a cell-grid pair list (13.5 A) and skips pairs beyond the 12 A outer cutoff itself,
// so the result is the cutoff sum over all pairs.  Here each call first builds, per frame, the near list: the MM
// atoms within the cutoff of at least one QC atom (FP32 distance with a conservative margin, after a test against
// the QC atoms' bounding box), compacted in MM index order with FP32 copies of their coordinates and charges.  The
// pair kernels scan that list instead of every MM atom (in the 50 A water box about a fifth of them), and only pairs
// inside the cutoff are evaluated; the near list keeps the MM index order, so every sum runs in the order of the
// full scan.  Coordinates are in Angstrom as the reference evaluates these terms; results are in atomic units.
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

__host__ __device__ __forceinline__ float cutoff_r2(int model, const Spline &sp)
{
    return model == 1 ? (float)(sp.r2off * (1.0 + 1.0e-4)) + 1.0e-3f : __builtin_huge_valf();
}
static inline float cutoff_r2_host(int model, const Spline &sp) { return cutoff_r2(model, sp); }

// ---------------------------------------------------------------------------------------------------
// Near list of each frame (workspace): count[f] entries at idx + f * stride (MM atom indices, increasing) and
// xq + f * stride (x, y, z, charge in FP32).  One CTA per frame: the QC atoms and their bounding box in shared
// memory; every MM atom is tested against the box (FP32), those within the cutoff of it against the QC atoms one
// by one until one is inside; a block-wide prefix of the warps' ballots places the near atoms in index order.
// gmm_zero (optional) receives zero gradients for the atoms that are not near (the MM-side gradient kernels
// write the near ones).
#define NL_THREADS 1024
struct NearList { int *count; int *idx; float4 *xq; size_t stride; };

__global__ void __launch_bounds__(NL_THREADS) k_qcmm_near(float r2cut, int n_qc, int n_mm, const double *__restrict__ qc,
                                                          const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                          double *__restrict__ gmm_zero)
{
    extern __shared__ float4 sa4[];   // QC atoms x, y, z
    __shared__ float wbox[NL_THREADS / 32][6], box[6];
    __shared__ int wc[NL_THREADS / 32], wo[NL_THREADS / 32 + 1];
    const int f = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    float lo[3] = { 3.4e38f, 3.4e38f, 3.4e38f }, hi[3] = { -3.4e38f, -3.4e38f, -3.4e38f };
    for (int k = tid; k < n_qc; k += NL_THREADS) {
        const double *x = qc + ((size_t)f * n_qc + k) * 3;
        const float4 a = make_float4((float)x[0], (float)x[1], (float)x[2], 0.0f);
        sa4[k] = a;
        lo[0] = fminf(lo[0], a.x); lo[1] = fminf(lo[1], a.y); lo[2] = fminf(lo[2], a.z);
        hi[0] = fmaxf(hi[0], a.x); hi[1] = fmaxf(hi[1], a.y); hi[2] = fmaxf(hi[2], a.z);
    }
    for (int c = 0; c < 3; c++)
        for (int o = 16; o > 0; o >>= 1) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
    if (lane == 0)
        for (int c = 0; c < 3; c++) { wbox[w][c] = lo[c]; wbox[w][3 + c] = hi[c]; }
    __syncthreads();
    if (tid < 6) {
        float v = wbox[0][tid];
        for (int k = 1; k < NL_THREADS / 32; k++) v = tid < 3 ? fminf(v, wbox[k][tid]) : fmaxf(v, wbox[k][tid]);
        box[tid] = v;
    }
    __syncthreads();
    const float bx0 = box[0], by0 = box[1], bz0 = box[2], bx1 = box[3], by1 = box[4], bz1 = box[5];
    int *idx = nl.idx + (size_t)f * nl.stride;
    float4 *xq = nl.xq + (size_t)f * nl.stride;
    int placed = 0;
    for (int m0 = 0; m0 < n_mm; m0 += NL_THREADS) {
        const int m = m0 + tid;
        bool near = false;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (m < n_mm) {
            const double *xm = mm + ((size_t)f * n_mm + m) * 3;
            fx = (float)xm[0]; fy = (float)xm[1]; fz = (float)xm[2];
            const float ex = fmaxf(0.f, fmaxf(bx0 - fx, fx - bx1)), ey = fmaxf(0.f, fmaxf(by0 - fy, fy - by1)),
                        ez = fmaxf(0.f, fmaxf(bz0 - fz, fz - bz1));
            if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= r2cut)
                for (int A = 0; A < n_qc && !near; A++) {
                    const float4 a = sa4[A];
                    const float dx = a.x - fx, dy = a.y - fy, dz = a.z - fz;
                    near = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= r2cut;
                }
            if (!near && gmm_zero) { double *o = gmm_zero + ((size_t)f * n_mm + m) * 3; o[0] = 0.0; o[1] = 0.0; o[2] = 0.0; }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, near);
        if (lane == 0) wc[w] = __popc(bal);
        __syncthreads();
        if (w == 0) {
            const int v = wc[lane];
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) { const int t = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= o) incl += t; }
            wo[lane] = incl - v;
            if (lane == 31) wo[32] = incl;
        }
        __syncthreads();
        if (near) {
            const int p = placed + wo[w] + __popc(bal & ((1u << lane) - 1u));
            idx[p] = m;
            xq[p] = make_float4(fx, fy, fz, (float)q[m]);
        }
        placed += wo[32];
        __syncthreads();
    }
    if (tid == 0) nl.count[f] = placed;
}

// Scan the frame's near list for the warp's QC atom; call body(k) (k the near-list entry) for every entry that
// passes the FP32 test, on all 32 lanes at once (lane k handles queue entry k), then on the final partial batch.
template <typename Body>
__device__ __forceinline__ void scan_near(int count, const float4 *__restrict__ xq, float fax, float fay, float faz, float r2cut,
                                          bool live, float4 *sxm, int *queue, Body body)
{
    const int lane = threadIdx.x & 31;
    int qn = 0;
    for (int c0 = 0; c0 < count; c0 += MCH) {
        const int cn = min(MCH, count - c0);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += QB) sxm[k] = xq[c0 + k];
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
                                                        const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                        double *__restrict__ phi)
{
    __shared__ float4 sxm[MCH];
    __shared__ int queue[QW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
    const double *xm = mm + (size_t)f * n_mm * 3;
    const int *idx = nl.idx + (size_t)f * nl.stride;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (live) { const double *xa = qc + ((size_t)f * n_qc + A) * 3; ax = xa[0]; ay = xa[1]; az = xa[2]; }
    double pot = 0.0;
    scan_near(nl.count[f], nl.xq + (size_t)f * nl.stride, (float)ax, (float)ay, (float)az, cutoff_r2(model, sp), live, sxm, queue[w], [&](int k) {
        const int m = idx[k];
        const double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        double fv;
        if (pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, nullptr)) pot += q[m] * fv;
    });
    pot = warp_sum(pot);
    if (live && lane == 0) phi[(size_t)f * n_qc + A] = pot;
}

// dE/dx_A = sum_m 2 q_A q_m f'(r^2) (x_A - x_m), converted from per-A to per-Bohr.
__global__ void __launch_bounds__(QB) k_qcmm_grad_qc(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                     const double *__restrict__ qcq, double *__restrict__ gqc)
{
    __shared__ float4 sxm[MCH];
    __shared__ int queue[QW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
    const double *xm = mm + (size_t)f * n_mm * 3;
    const int *idx = nl.idx + (size_t)f * nl.stride;
    double ax = 0.0, ay = 0.0, az = 0.0, qa = 0.0;
    if (live) { const double *xa = qc + ((size_t)f * n_qc + A) * 3; ax = xa[0]; ay = xa[1]; az = xa[2]; qa = qcq[(size_t)f * n_qc + A]; }
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    scan_near(nl.count[f], nl.xq + (size_t)f * nl.stride, (float)ax, (float)ay, (float)az, cutoff_r2(model, sp), live, sxm, queue[w], [&](int k) {
        const int m = idx[k];
        const double dx = ax - xm[3 * m], dy = ay - xm[3 * m + 1], dz = az - xm[3 * m + 2];
        double fv, gv;
        if (!pair_term(model, sp, dx * dx + dy * dy + dz * dz, &fv, &gv)) return;
        const double s = 2.0 * qa * q[m] * gv / PDG_ANGSTROMS_TO_BOHRS;
        g0 += s * dx; g1 += s * dy; g2 += s * dz;
    });
    g0 = warp_sum(g0); g1 = warp_sum(g1); g2 = warp_sum(g2);
    if (live && lane == 0) { double *o = gqc + ((size_t)f * n_qc + A) * 3; o[0] = g0; o[1] = g1; o[2] = g2; }
}

// MM side: a block takes 256 consecutive entries of one frame's near list (every other MM atom got a zero gradient
// from the near-list kernel); the warps take them one at a time (w, w + 8, ...): for its atom a warp tests the QC
// atoms 32 at a time in FP32, queues the ones inside the cutoff and evaluates the queue in FP64 thirty-two pairs at
// a time (as the QC side does), so that no FP64 pass runs for a few lanes; lane partial sums are reduced in a fixed
// order.  The grid covers n_mm entries per frame; blocks past the frame's near count return at once.
#define MB 256
__global__ void __launch_bounds__(MB) k_qcmm_grad_mm(int model, Spline sp, int n_qc, int n_mm, const double *__restrict__ qc,
                                                     const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                     const double *__restrict__ qcq, double *__restrict__ gmm)
{
    extern __shared__ double sq[];   // QC atoms: x, y, z, charge (doubles), then x, y, z (floats)
    __shared__ int queue[MB / 32][64];
    float *sf = (float *)(sq + 4 * (size_t)n_qc);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int blocks_per_frame = (n_mm + MB - 1) / MB;
    const int f = blockIdx.x / blocks_per_frame, base = (blockIdx.x % blocks_per_frame) * MB;
    const int count = nl.count[f];
    if (base >= count) return;
    for (int k = threadIdx.x; k < n_qc; k += MB) {
        const double *x = qc + ((size_t)f * n_qc + k) * 3;
        sq[4 * k] = x[0]; sq[4 * k + 1] = x[1]; sq[4 * k + 2] = x[2]; sq[4 * k + 3] = qcq[(size_t)f * n_qc + k];
        sf[3 * k] = (float)x[0]; sf[3 * k + 1] = (float)x[1]; sf[3 * k + 2] = (float)x[2];
    }
    __syncthreads();
    const float r2cut = cutoff_r2(model, sp);
    const int total = min(MB, count - base);
    const int *near_list = nl.idx + (size_t)f * nl.stride + base;
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
                                                       const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                       const double *__restrict__ qcq, double *__restrict__ gqc)
{
    __shared__ float4 sxm[MCH];       // MM atoms of the chunk: x, y, z, charge
    __shared__ float4 queue[QW][64];
    __shared__ Knots32 kn;
    if (model == 1) stage_knots32(sp, kn);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, groups = (n_qc + QW - 1) / QW;
    const int f = blockIdx.x / groups, A = (blockIdx.x % groups) * QW + w;
    const bool live = A < n_qc;
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
    const int count = nl.count[f];
    const float4 *xq = nl.xq + (size_t)f * nl.stride;
    for (int c0 = 0; c0 < count; c0 += MCH) {
        const int cn = min(MCH, count - c0);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += QB) sxm[k] = xq[c0 + k];
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
                                                       const double *__restrict__ mm, const double *__restrict__ q, NearList nl,
                                                       const double *__restrict__ qcq, double *__restrict__ gmm)
{
    extern __shared__ float4 sa[];    // QC atoms: x, y, z, charge
    __shared__ int queue[MB / 32][64];
    __shared__ Knots32 kn;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int blocks_per_frame = (n_mm + MB - 1) / MB;
    const int f = blockIdx.x / blocks_per_frame, base = (blockIdx.x % blocks_per_frame) * MB;
    const int count = nl.count[f];
    if (base >= count) return;
    if (model == 1) stage_knots32(sp, kn);
    for (int k = threadIdx.x; k < n_qc; k += MB) {
        const double *x = qc + ((size_t)f * n_qc + k) * 3;
        sa[k] = make_float4((float)x[0], (float)x[1], (float)x[2], (float)qcq[(size_t)f * n_qc + k]);
    }
    __syncthreads();
    const float r2cut = cutoff_r2(model, sp), sc = (float)(2.0 / PDG_ANGSTROMS_TO_BOHRS);
    const int total = min(MB, count - base);
    const int *near_list = nl.idx + (size_t)f * nl.stride + base;
    const float4 *xq = nl.xq + (size_t)f * nl.stride + base;
    int *qw = queue[w];
    for (int k = w; k < total; k += MB / 32) {
        const int m = near_list[k];
        const float4 pm = xq[k];
        const float mx = pm.x, my = pm.y, mz = pm.z, qm = pm.w;
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

size_t qcmm_workspace_bytes(int n_frames, int n_mm)
{
    const size_t F = n_frames > 0 ? (size_t)n_frames : 0, M = n_mm > 0 ? (size_t)n_mm : 1;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    return up(4 * F) + up(4 * F * M) + 16 * F * M;
}

static NearList near_list(void *ws, int n_frames, int n_mm)
{
    const size_t F = (size_t)n_frames, M = n_mm > 0 ? (size_t)n_mm : 1;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    char *b = (char *)ws;
    NearList nl;
    nl.count = (int *)b; nl.idx = (int *)(b + up(4 * F)); nl.xq = (float4 *)(b + up(4 * F) + up(4 * F * M)); nl.stride = M;
    return nl;
}

static void launch_near(int model, const Spline &sp, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                        const double *q, const NearList &nl, double *gmm_zero, cudaStream_t st)
{
    const size_t sm = sizeof(float4) * (size_t)n_qc;
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_qcmm_near, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_qcmm_near<<<n_frames, NL_THREADS, sm, st>>>(cutoff_r2_host(model, sp), n_qc, n_mm, qc, mm, q, nl, gmm_zero);
}

int launch_qcmm_potentials(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                           const double *q, int n_knots, const double *knots, double cutoff, double *phi, void *ws, cudaStream_t st)
{
    if (n_frames <= 0 || n_qc <= 0) return 0;
    Spline sp = make_spline(n_knots, knots, cutoff);
    const NearList nl = near_list(ws, n_frames, n_mm);
    launch_near(model, sp, n_frames, n_qc, n_mm, qc, mm, q, nl, nullptr, st);
    const int groups = (n_qc + QW - 1) / QW;
    k_qcmm_potentials<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, nl, phi);
    return 0;
}

int launch_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                          const double *q, const double *qcq, int n_knots, const double *knots, double cutoff,
                          double *gqc, double *gmm, void *ws, cudaStream_t st)
{
    if (n_frames <= 0 || n_qc <= 0) return 0;
    const bool f32 = (model & PDG_QCMM_FP32_PAIRS) != 0 && n_knots <= KMAX32;
    model &= ~PDG_QCMM_FP32_PAIRS;
    Spline sp = make_spline(n_knots, knots, cutoff);
    const NearList nl = near_list(ws, n_frames, n_mm);
    double *gmm_out = (n_mm > 0) ? gmm : nullptr;
    launch_near(model, sp, n_frames, n_qc, n_mm, qc, mm, q, nl, gmm_out, st);
    const int groups = (n_qc + QW - 1) / QW, bpf = (n_mm + MB - 1) / MB;
    if (f32) {
        k_qcmm_grad_qc32<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, nl, qcq, gqc);
        if (gmm_out) {
            const size_t sm = sizeof(float4) * (size_t)n_qc;
            if (sm > 8 * 1024) cudaFuncSetAttribute(k_qcmm_grad_mm32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_qcmm_grad_mm32<<<n_frames * bpf, MB, sm, st>>>(model, sp, n_qc, n_mm, qc, mm, q, nl, qcq, gmm);
        }
        return 0;
    }
    k_qcmm_grad_qc<<<n_frames * groups, QB, 0, st>>>(model, sp, n_qc, n_mm, qc, mm, q, nl, qcq, gqc);
    if (gmm_out) {
        const size_t sm = sizeof(double) * 4 * (size_t)n_qc + sizeof(float) * 3 * (size_t)n_qc;
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_qcmm_grad_mm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_qcmm_grad_mm<<<n_frames * bpf, MB, sm, st>>>(model, sp, n_qc, n_mm, qc, mm, q, nl, qcq, gmm);
    }
    return 0;
}
