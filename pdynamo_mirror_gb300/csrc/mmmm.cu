// MM/MM electrostatic and Lennard-Jones energies and QC/MM Lennard-Jones energies of NBModelABFS, with gradients,
// for many frames of one system.
//
// Reference: NBModelABFS_MMMMEnergy and NBModelABFS_QCMMEnergyLJ (pMolecule-1.9.0/extensions/csource/NBModelABFS.c:228,
// :306) evaluate PairwiseInteractionABFS_MMMMEnergy (PairwiseInteraction.c:292) in its default analytic form
// (PairwiseInteraction.c:29-45 sets useAnalyticForm) over pair lists made by the cell-grid pair-list generator
// (pCore-1.9.0/extensions/csource/PairListGenerator.c:414-530) under the selections of GenerateLists and
// GenerateLists14 (NBModelABFS.c:1050-1160): MM/MM pairs of active MM atoms, QC/MM LJ pairs of a QC atom that has
// LJ interactions with an MM atom, exclusions removed, at least one atom of a pair free, and the 1-4 list with its
// own LJ tables and electrostaticScale14.  The pair terms are PairwiseInteractionABFS_CheckDistances /
// _ElectrostaticTerm / _LennardJonesTerm (cinclude/PairwiseInteraction.h:72-120).
//
// Here the pair list is replaced by a cell grid rebuilt for every evaluation (the reference's list cutoff only
// bounds its search, and every pair inside the outer cutoff is evaluated either way):
//   k_mm_grid   one block per frame: bounding box, cells of at least half the outer cutoff (at most 32 per
//               dimension), atoms counted into cells, an exclusive scan, a scatter, and each cell's atoms sorted by
//               index so that every later sum runs in a fixed order; coordinates and charges copied in cell order.
//   k_mm_pairs  one warp per atom (full neighbour lists: each pair is seen from both atoms, half its energy
//               counted at each): the cells within two cells of the atom's cell in y and z, the five cells along x
//               read as one contiguous segment; FP64 pair terms; the atom's own gradient summed without atomics;
//               then the atom's 1-4 partners.  Per-block energies in fixed order.
//   k_mm_sum    per frame, the block energies in fixed order.
#include "common.cuh"

namespace {

struct MMGrid {
    double lo[3], inv_h[3];
    int nd[3], ncell;
};
static_assert(sizeof(MMGrid) == 64, "grid record");

__device__ __forceinline__ int mm_cell_1d(double x, double lo, double inv_h, int nd)
{
    const int c = (int)((x - lo) * inv_h);   // x >= lo: truncation is floor; NaN converts to 0
    return min(nd - 1, max(0, c));
}

// PairwiseInteraction.h:72-120 for one pair inside the outer cutoff: electrostatic energy (qij already scaled),
// LJ energy, and dF = dE/d(r^2).
__device__ __forceinline__ void mm_pair_terms(const MMFactors &F, double r2, double qij, double A, double B, bool el,
                                              double &fe, double &fl, double &dF)
{
    double s = 0.0, s2 = 0.0;
    if (!(r2 < F.r2Damp)) { s2 = 1.0 / r2; s = sqrt(s2); }
    fe = 0.0; dF = 0.0;
    if (el) {
        if (r2 > F.r2On) {
            fe = qij * (s * (F.a - r2 * (F.b + r2 * (F.c + F.d * r2))) + F.qShift2);
            dF -= qij * 0.5 * s * (F.a + r2 * (F.b + r2 * (3.0 * F.c + 5.0 * F.d * r2))) / r2;
        } else if (r2 > F.r2Damp) {
            fe = qij * (s + F.qShift1);
            dF -= qij * 0.5 * s / r2;
        } else {
            fe = qij * (F.qF0 - F.qAlpha * r2);
            dF -= qij * F.qAlpha;
        }
    }
    const double s6 = s2 * s2 * s2;
    if (r2 > F.r2On) {
        const double l1 = s6 - F.aF6, l2 = s / r2 - F.bF3;
        fl = A * F.aK12 * l1 * l1 - B * F.bK6 * l2 * l2;
        dF -= 3.0 * s6 * (2.0 * A * F.aK12 * l1 / r2 - B * F.bK6 * l2 / s);
    } else if (r2 > F.r2Damp) {
        fl = A * (s6 * s6 - F.aShift12) - B * (s6 - F.bShift6);
        dF -= 3.0 * s6 * (2.0 * A * s6 - B) / r2;
    } else {
        fl = A * (F.aF0 - F.aAlpha * r2) - B * (F.bF0 - F.bAlpha * r2);
        dF += -A * F.aAlpha + B * F.bAlpha;
    }
}

struct MMFrameWS {
    MMGrid *grid;
    int *count, *start, *cell_of, *order;
    double4 *sxyzq;
    double *part;
};

__device__ __forceinline__ MMFrameWS mm_frame_ws(char *ws, const MMLayout &L, int f)
{
    char *b = ws + (size_t)f * L.stride;
    MMFrameWS w;
    w.grid = (MMGrid *)(b + L.grid);
    w.count = (int *)(b + L.count);
    w.start = (int *)(b + L.start);
    w.cell_of = (int *)(b + L.cell_of);
    w.order = (int *)(b + L.order);
    w.sxyzq = (double4 *)(b + L.sxyzq);
    w.part = (double *)(b + L.part);
    return w;
}

__global__ void __launch_bounds__(256) k_mm_grid(MMDevice m, MMLayout L, const double *__restrict__ xyz, char *ws)
{
    const int f = blockIdx.x, tid = threadIdx.x, n = m.n_atoms;
    const double *X = xyz + (size_t)f * n * 3;
    MMFrameWS w = mm_frame_ws(ws, L, f);
    __shared__ double red[6][256];
    __shared__ MMGrid g;
    __shared__ int chunk[257];
    double lo[3] = { 1e300, 1e300, 1e300 }, hi[3] = { -1e300, -1e300, -1e300 };
    for (int i = tid; i < n; i += 256)
        for (int d = 0; d < 3; d++) { const double x = X[3 * i + d]; lo[d] = fmin(lo[d], x); hi[d] = fmax(hi[d], x); }
    for (int d = 0; d < 3; d++) { red[d][tid] = lo[d]; red[3 + d][tid] = hi[d]; }
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (tid < s)
            for (int d = 0; d < 3; d++) {
                red[d][tid] = fmin(red[d][tid], red[d][tid + s]);
                red[3 + d][tid] = fmax(red[3 + d][tid], red[3 + d][tid + s]);
            }
        __syncthreads();
    }
    if (tid == 0) {
        const double half = 0.5 * m.outer;
        int nc = 1;
        for (int d = 0; d < 3; d++) {
            const double ext = red[3 + d][0] - red[d][0];
            const double q = ext / half;
            int nd = (q >= 1.0 && q < 1.0e9) ? (int)q : 1;   // cells of at least half the outer cutoff
            nd = min(MM_MAX_CELLS_1D, max(1, nd));
            const double h = ext / (double)nd;
            g.lo[d] = red[d][0];
            g.inv_h[d] = (h > 0.0 && h < 1.0e300) ? 1.0 / h : 0.0;
            g.nd[d] = nd;
            nc *= nd;
        }
        g.ncell = nc;
        *w.grid = g;
    }
    __syncthreads();
    const int ncell = g.ncell;
    for (int c = tid; c < ncell; c += 256) w.count[c] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += 256) {
        const int cx = mm_cell_1d(X[3 * i], g.lo[0], g.inv_h[0], g.nd[0]);
        const int cy = mm_cell_1d(X[3 * i + 1], g.lo[1], g.inv_h[1], g.nd[1]);
        const int cz = mm_cell_1d(X[3 * i + 2], g.lo[2], g.inv_h[2], g.nd[2]);
        const int c = (cz * g.nd[1] + cy) * g.nd[0] + cx;
        w.cell_of[i] = c;
        atomicAdd(&w.count[c], 1);
    }
    __syncthreads();
    // exclusive scan: thread t owns cells [t * per, (t + 1) * per)
    const int per = (ncell + 255) / 256;
    {
        int s = 0;
        for (int c = tid * per; c < min(ncell, (tid + 1) * per); c++) s += w.count[c];
        chunk[tid + 1] = s;
    }
    __syncthreads();
    if (tid == 0) {
        chunk[0] = 0;
        for (int t = 1; t <= 256; t++) chunk[t] += chunk[t - 1];
    }
    __syncthreads();
    {
        int s = chunk[tid];
        for (int c = tid * per; c < min(ncell, (tid + 1) * per); c++) { const int k = w.count[c]; w.start[c] = s; s += k; w.count[c] = 0; }
        if (tid == 0) w.start[ncell] = n;
    }
    __syncthreads();
    for (int i = tid; i < n; i += 256) {
        const int c = w.cell_of[i];
        w.order[w.start[c] + atomicAdd(&w.count[c], 1)] = i;
    }
    __syncthreads();
    // each cell's atoms in index order (the scatter's order depends on the atomics)
    for (int c = tid; c < ncell; c += 256) {
        const int a = w.start[c], b = w.start[c + 1];
        for (int p = a + 1; p < b; p++) {
            const int v = w.order[p];
            int q = p - 1;
            while (q >= a && w.order[q] > v) { w.order[q + 1] = w.order[q]; q--; }
            w.order[q + 1] = v;
        }
    }
    __syncthreads();
    for (int p = tid; p < n; p += 256) {
        const int i = w.order[p];
        w.sxyzq[p] = make_double4(X[3 * i], X[3 * i + 1], X[3 * i + 2], m.charge[i]);
    }
}

__device__ __forceinline__ double mm_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) k_mm_pairs(MMDevice m, MMLayout L, const double *__restrict__ xyz, double *grad, char *ws)
{
    const int f = blockIdx.y, lane = threadIdx.x & 31, wp = threadIdx.x >> 5, n = m.n_atoms;
    const int i = blockIdx.x * 8 + wp;
    const double *X = xyz + (size_t)f * n * 3;
    const MMFrameWS w = mm_frame_ws(ws, L, f);
    __shared__ double es[8][MM_NCH];
    double e[MM_NCH] = { 0.0, 0.0, 0.0, 0.0, 0.0, 0.0 };
    double gx = 0.0, gy = 0.0, gz = 0.0;
    const int fi = i < n ? (int)m.flags[i] : 0;
    if (fi & (MM_FLAG_MM | MM_FLAG_QC_LJ)) {
        const MMGrid g = *w.grid;
        const double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2], qi = m.charge[i];
        const bool mm_i = fi & MM_FLAG_MM, fixed_i = fi & MM_FLAG_FIXED;
        const int ti = m.lj_type[i] * m.n_types;
        const int es0 = m.excl_start[i], es1 = m.excl_start[i + 1];
        const int cx = mm_cell_1d(xi, g.lo[0], g.inv_h[0], g.nd[0]);
        const int cy = mm_cell_1d(yi, g.lo[1], g.inv_h[1], g.nd[1]);
        const int cz = mm_cell_1d(zi, g.lo[2], g.inv_h[2], g.nd[2]);
        const int x0 = max(0, cx - 2), x1 = min(g.nd[0] - 1, cx + 2);
        for (int z = max(0, cz - 2); z <= min(g.nd[2] - 1, cz + 2); z++)
            for (int y = max(0, cy - 2); y <= min(g.nd[1] - 1, cy + 2); y++) {
                const int row = (z * g.nd[1] + y) * g.nd[0];
                const int p1 = w.start[row + x1 + 1];
                for (int p = w.start[row + x0] + lane; p < p1; p += 32) {
                    const int j = w.order[p];
                    if (j == i) continue;
                    const int fj = m.flags[j];
                    const bool mm_j = fj & MM_FLAG_MM;
                    const bool el = mm_i && mm_j;
                    if (!el && !((mm_i && (fj & MM_FLAG_QC_LJ)) || (!mm_i && mm_j))) continue;
                    if (fixed_i && (fj & MM_FLAG_FIXED)) continue;
                    bool excluded = false;
                    for (int k = es0; k < es1; k++) excluded |= (m.excl[k] == j);
                    if (excluded) continue;
                    const double4 pj = w.sxyzq[p];
                    const double dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 > m.fac.r2Off) continue;
                    const int tij = ti + m.lj_type[j];
                    double fe, fl, dF;
                    mm_pair_terms(m.fac, r2, el ? m.escale * qi * pj.w : 0.0, m.A[tij], m.B[tij], el, fe, fl, dF);
                    if (el) { e[0] += 0.5 * fe; e[1] += 0.5 * fl; }
                    else e[4] += 0.5 * fl;
                    const double t = 2.0 * dF;
                    gx = fma(t, dx, gx); gy = fma(t, dy, gy); gz = fma(t, dz, gz);
                }
            }
        // 1-4 partners (their own tables and electrostatic scale; not filtered by the exclusions)
        for (int k = m.p14_start[i] + lane; k < m.p14_start[i + 1]; k += 32) {
            const int j = m.p14[k];
            const int fj = m.flags[j];
            const bool mm_j = fj & MM_FLAG_MM;
            const bool el = mm_i && mm_j;
            if (!el && !((mm_i && (fj & MM_FLAG_QC_LJ)) || (!mm_i && mm_j))) continue;
            if (fixed_i && (fj & MM_FLAG_FIXED)) continue;
            const double dx = xi - X[3 * j], dy = yi - X[3 * j + 1], dz = zi - X[3 * j + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > m.fac.r2Off) continue;
            const int tij = ti + m.lj_type[j];
            double fe, fl, dF;
            mm_pair_terms(m.fac, r2, el ? m.escale14 * qi * m.charge[j] : 0.0, m.A14[tij], m.B14[tij], el, fe, fl, dF);
            if (el) { e[2] += 0.5 * fe; e[3] += 0.5 * fl; }
            else e[5] += 0.5 * fl;
            const double t = 2.0 * dF;
            gx = fma(t, dx, gx); gy = fma(t, dy, gy); gz = fma(t, dz, gz);
        }
    }
    __syncwarp();
    for (int c = 0; c < MM_NCH; c++) e[c] = mm_warp_sum(e[c]);
    gx = mm_warp_sum(gx); gy = mm_warp_sum(gy); gz = mm_warp_sum(gz);
    if (lane == 0) {
        if (grad != nullptr && i < n) {
            double *G = grad + ((size_t)f * n + i) * 3;
            G[0] = gx; G[1] = gy; G[2] = gz;
        }
        for (int c = 0; c < MM_NCH; c++) es[wp][c] = e[c];
    }
    __syncthreads();
    if (threadIdx.x < MM_NCH) {
        double s = 0.0;
        for (int q = 0; q < 8; q++) s += es[q][threadIdx.x];
        w.part[(size_t)blockIdx.x * MM_NCH + threadIdx.x] = s;
    }
}

__global__ void k_mm_sum(MMLayout L, int n_blocks, char *ws, double *energies)
{
    const int f = blockIdx.x, c = threadIdx.x;
    if (c >= MM_NCH) return;
    const double *part = (const double *)(ws + (size_t)f * L.stride + L.part);
    double s = 0.0;
    for (int b = 0; b < n_blocks; b++) s += part[(size_t)b * MM_NCH + c];
    energies[(size_t)f * MM_NCH + c] = s;
}

}  // namespace

MMLayout mm_layout(int n_atoms)
{
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    MMLayout L;
    const size_t n = (size_t)n_atoms, maxc = (size_t)MM_MAX_CELLS_1D * MM_MAX_CELLS_1D * MM_MAX_CELLS_1D;
    size_t o = 0;
    L.grid = o;    o += al(sizeof(MMGrid));
    L.count = o;   o += al(sizeof(int) * maxc);
    L.start = o;   o += al(sizeof(int) * (maxc + 1));
    L.cell_of = o; o += al(sizeof(int) * n);
    L.order = o;   o += al(sizeof(int) * n);
    L.sxyzq = o;   o += al(sizeof(double4) * n);
    L.n_blocks = (n_atoms + 7) / 8;
    L.part = o;    o += al(sizeof(double) * MM_NCH * (size_t)L.n_blocks);
    L.stride = o;
    return L;
}

void launch_mm_energy(const MMDevice &m, int n_frames, const double *xyz, double *energies, double *grad, char *ws, cudaStream_t st)
{
    const MMLayout L = mm_layout(m.n_atoms);
    k_mm_grid<<<n_frames, 256, 0, st>>>(m, L, xyz, ws);
    k_mm_pairs<<<dim3(L.n_blocks, n_frames), 256, 0, st>>>(m, L, xyz, grad, ws);
    k_mm_sum<<<n_frames, 32, 0, st>>>(L, L.n_blocks, ws, energies);
}
