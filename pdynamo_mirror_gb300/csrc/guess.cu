// guess.cu - learned SCF start density: a per-atom-pair MLP, with its own training and inference kernels.
//
// For every atom pair closer than GUESS_CUT the MLP maps 64 geometric features (distance, its radial basis,
// element one-hots, radial environment functions of both atoms, the QC/MM potential at both atoms) through
// two SiLU layers of width 256 to 16 outputs: the pair's density block in its local frame (z from atom i to
// atom j; entries ss, s-sigma, sigma-s, sigma-sigma, pi-pi) and one-centre contributions to both atoms in the
// same frame (ss, s-sigma, sigma-sigma, pi-pi each).  The blocks are rotated to the molecular frame with the
// orbital rotation of the integrals (multipole.cuh), so the guess turns with the molecule; one-centre blocks
// are the diagonal start density of the reference (N_e / N on every orbital) plus the contributions of all
// pairs of the atom, gathered in pair order; the trace is then corrected to N_e.  Weights are stored in BF16,
// every product accumulates in FP32.  Training: the same forward pass, the squared error of the assembled
// blocks against converged densities, backward passes and Adam.  No counterpart in the reference (its SCF
// starts from the diagonal guess, QCOnePDM.c:280, or from the previous density).
#include <cuda_bf16.h>

#include "common.cuh"
#include "multipole.cuh"

#define GUESS_IN 64
#define GUESS_H 256
#define GUESS_OUT 16
#define GUESS_CUT 3.5      // Angstrom
#define GUESS_ENV_CUT 4.5  // Angstrom

// ---------------------------------------------------------------------------------------------------
// Features
__global__ void k_guess_env(int n_frames, int n_atoms, const int *__restrict__ atom_elem, const double *__restrict__ xyz,
                            float *__restrict__ env)
{
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long)n_frames * n_atoms) return;
    const int f = (int)(g / n_atoms), A = (int)(g % n_atoms);
    const double *R = xyz + (size_t)f * 3 * n_atoms;
    float e[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (int C = 0; C < n_atoms; C++) {
        if (C == A) continue;
        const int ec = atom_elem[C];
        if (ec > 1) continue;
        const float dx = (float)(R[3 * C] - R[3 * A]), dy = (float)(R[3 * C + 1] - R[3 * A + 1]), dz = (float)(R[3 * C + 2] - R[3 * A + 2]);
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        if (r > (float)GUESS_ENV_CUT) continue;
        const float fc = 0.5f * (cospif(r / (float)GUESS_ENV_CUT) + 1.0f);
        for (int k = 0; k < 4; k++) { const float t = (r - (1.0f + 0.8f * k)) * 2.0f; e[ec * 4 + k] += __expf(-t * t) * fc; }
    }
    for (int k = 0; k < 8; k++) env[g * 8 + k] = e[k];
}

__device__ __forceinline__ bool guess_pair_in(const DeviceSystem &s, const double *R, int p)
{
    const int i = s.pair_i[p], j = s.pair_j[p];
    const double dx = R[3 * j] - R[3 * i], dy = R[3 * j + 1] - R[3 * i + 1], dz = R[3 * j + 2] - R[3 * i + 2];
    return dx * dx + dy * dy + dz * dz < GUESS_CUT * GUESS_CUT;
}

// Pairs inside the cutoff per frame (one block per frame).
__global__ void k_guess_count(DeviceSystem s, int n_frames, const double *__restrict__ xyz, int *__restrict__ count)
{
    __shared__ int red[32];
    const int f = blockIdx.x;
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    int c = 0;
    for (int p = threadIdx.x; p < s.n_pairs; p += blockDim.x) c += guess_pair_in(s, R, p);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        count[f] = t;
    }
}

// Exclusive scan of the per-frame counts (one block): offsets[f], offsets[n_frames] = total rows.
__global__ void k_guess_scan(int n_frames, const int *__restrict__ count, int *__restrict__ offsets)
{
    if (threadIdx.x == 0) {
        int t = 0;
        for (int f = 0; f < n_frames; f++) { offsets[f] = t; t += count[f]; }
        offsets[n_frames] = t;
    }
}

// Rows of the frame's pairs in pair order (block prefix, deterministic) with their features.
__global__ void k_guess_features(DeviceSystem s, int n_frames, const double *__restrict__ xyz, const double *__restrict__ phi,
                                 const float *__restrict__ env, const int *__restrict__ offsets, float *__restrict__ X,
                                 int *__restrict__ row_frame, int *__restrict__ row_pair)
{
    __shared__ int wsum[32];
    __shared__ int base;
    const int f = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    if (tid == 0) base = offsets[f];
    __syncthreads();
    for (int p0 = 0; p0 < s.n_pairs; p0 += blockDim.x) {
        const int p = p0 + tid;
        const bool in = p < s.n_pairs && guess_pair_in(s, R, p);
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        if (lane == 0) wsum[w] = __popc(bal);
        __syncthreads();
        int off = base;
        for (int k = 0; k < w; k++) off += wsum[k];
        off += __popc(bal & ((1u << lane) - 1u));
        if (in) {
            const int i = s.pair_i[p], j = s.pair_j[p];
            const double dx = R[3 * j] - R[3 * i], dy = R[3 * j + 1] - R[3 * i + 1], dz = R[3 * j + 2] - R[3 * i + 2];
            const float r = (float)sqrt(dx * dx + dy * dy + dz * dz);
            float *x = X + (size_t)off * GUESS_IN;
            for (int k = 0; k < GUESS_IN; k++) x[k] = 0.0f;
            x[0] = r; x[1] = 1.0f / r;
            for (int k = 0; k < 8; k++) { const float t = (r - (0.8f + 0.4f * k)) * 2.5f; x[2 + k] = __expf(-t * t); }
            const int ei = s.atom_elem[i], ej = s.atom_elem[j];
            if (ei < 4) x[10 + ei] = 1.0f;
            if (ej < 4) x[14 + ej] = 1.0f;
            const float *envi = env + ((size_t)f * s.n_atoms + i) * 8, *envj = env + ((size_t)f * s.n_atoms + j) * 8;
            for (int k = 0; k < 8; k++) { x[18 + k] = envi[k]; x[26 + k] = envj[k]; }
            if (phi) { x[34] = (float)phi[(size_t)f * s.n_atoms + i]; x[35] = (float)phi[(size_t)f * s.n_atoms + j]; }
            row_frame[off] = f; row_pair[off] = p;
        }
        __syncthreads();
        if (tid == 0) { int t = 0; for (int k = 0; k < nw; k++) t += wsum[k]; base += t; }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------------
// FP32 GEMM tiles: C[i][j] = sum_r a(i, r) b(r, j) over 64 x 64 outputs per block of 256 threads (4 x 4 per
// thread), reduction staged 16 deep in shared memory.  Rows beyond *rows (device) are skipped.
template <typename FA, typename FB, typename Epi>
__device__ __forceinline__ void gemm_tile(int i0, int j0, int Mi, int Nj, int Rr, FA a, FB b, Epi epi)
{
    __shared__ float As[16][68], Bs[16][68];
    const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
    float acc[4][4] = {};
    for (int r0 = 0; r0 < Rr; r0 += 16) {
        for (int t = tid; t < 16 * 64; t += 256) {
            const int rr = t / 64, c = t % 64;
            As[rr][c] = (i0 + c < Mi && r0 + rr < Rr) ? a(i0 + c, r0 + rr) : 0.0f;
            Bs[rr][c] = (j0 + c < Nj && r0 + rr < Rr) ? b(r0 + rr, j0 + c) : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int rr = 0; rr < 16; rr++) {
            float av[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) { av[q] = As[rr][ty * 4 + q]; bv[q] = Bs[rr][tx * 4 + q]; }
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = fmaf(av[x], bv[y], acc[x][y]);
        }
        __syncthreads();
    }
    for (int x = 0; x < 4; x++)
        for (int y = 0; y < 4; y++) {
            const int i = i0 + ty * 4 + x, j = j0 + tx * 4 + y;
            if (i < Mi && j < Nj) epi(i, j, acc[x][y]);
        }
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) { const float sg = 1.0f / (1.0f + __expf(-z)); return sg * (1.0f + z * (1.0f - sg)); }

// Z = X W^T + b, H = silu(Z) (act) or Z.  X [rows x K], W [N x K] BF16.
__global__ void __launch_bounds__(256) k_mlp_forward(const int *__restrict__ rows, int K, int N, const float *__restrict__ X,
                                                     const __nv_bfloat16 *__restrict__ W, const float *__restrict__ b,
                                                     float *__restrict__ Z, float *__restrict__ H, int act)
{
    const int M = *rows, i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    if (i0 >= M) return;
    gemm_tile(i0, j0, M, N, K, [&](int i, int r) { return X[(size_t)i * K + r]; },
              [&](int r, int j) { return __bfloat162float(W[(size_t)j * K + r]); },
              [&](int i, int j, float v) {
                  const float z = v + b[j];
                  if (Z) Z[(size_t)i * N + j] = z;
                  H[(size_t)i * N + j] = act ? silu(z) : z;
              });
}

// dZin = (dZ W) * silu'(Zin): dZ [rows x N], W [N x K], Zin [rows x K].
__global__ void __launch_bounds__(256) k_mlp_backward_data(const int *__restrict__ rows, int N, int K, const float *__restrict__ dZ,
                                                           const __nv_bfloat16 *__restrict__ W, const float *__restrict__ Zin,
                                                           float *__restrict__ dZin)
{
    const int M = *rows, i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    if (i0 >= M) return;
    gemm_tile(i0, j0, M, K, N, [&](int i, int r) { return dZ[(size_t)i * N + r]; },
              [&](int r, int j) { return __bfloat162float(W[(size_t)r * K + j]); },
              [&](int i, int j, float v) { dZin[(size_t)i * K + j] = v * dsilu(Zin[(size_t)i * K + j]); });
}

// Per row segment s: dWpart[s][n][k] = sum_{m in s} dZ[m][n] Hin[m][k] (and the bias gradient in column K).
__global__ void __launch_bounds__(256) k_mlp_backward_weights(const int *__restrict__ rows, int segments, int N, int K,
                                                              const float *__restrict__ dZ, const float *__restrict__ Hin,
                                                              float *__restrict__ part)
{
    const int M = *rows, s = blockIdx.z, seg = (M + segments - 1) / segments, m0 = s * seg, m1 = min(M, m0 + seg);
    const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;   // i over N (outputs), j over K + 1 (inputs, bias)
    float *out = part + (size_t)s * N * (K + 1);
    const int len = m1 > m0 ? m1 - m0 : 0;
    gemm_tile(i0, j0, N, K + 1, len, [&](int i, int r) { return dZ[(size_t)(m0 + r) * N + i]; },
              [&](int r, int j) { return j < K ? Hin[(size_t)(m0 + r) * K + j] : 1.0f; },
              [&](int i, int j, float v) { out[(size_t)i * (K + 1) + j] = v; });
}

// Adam over the weights (with the bias in column K) from the summed segment gradients (fixed order).
__global__ void k_mlp_adam(int N, int K, int segments, const float *__restrict__ part, float scale, float *__restrict__ Wm,
                           float *__restrict__ bm, float *__restrict__ m1, float *__restrict__ m2, __nv_bfloat16 *__restrict__ W,
                           float lr, float b1, float b2, float c1, float c2)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N * (K + 1)) return;
    float g = 0.0f;
    for (int s = 0; s < segments; s++) g += part[(size_t)s * N * (K + 1) + e];
    g *= scale;
    const float a = b1 * m1[e] + (1.0f - b1) * g, v = b2 * m2[e] + (1.0f - b2) * g * g;
    m1[e] = a; m2[e] = v;
    const float step = lr * (a * c1) / (sqrtf(v * c2) + 1e-8f);
    const int n = e / (K + 1), k = e % (K + 1);
    if (k < K) { Wm[(size_t)n * K + k] -= step; W[(size_t)n * K + k] = __float2bfloat16_rn(Wm[(size_t)n * K + k]); }
    else bm[n] -= step;
}

// ---------------------------------------------------------------------------------------------------
// Assembly: predicted density of every frame (one block per frame).
__device__ __forceinline__ void guess_rotation(const DeviceSystem &s, const double *R, int p, double T[4][4])
{
    const int i = s.pair_i[p], j = s.pair_j[p];
    const double x = R[3 * j] - R[3 * i], y = R[3 * j + 1] - R[3 * i + 1], z = R[3 * j + 2] - R[3 * i + 2];
    const double r = sqrt(x * x + y * y + z * z);
    RotScalars q;
    rot_scalars(x * PDG_ANGSTROMS_TO_BOHRS, y * PDG_ANGSTROMS_TO_BOHRS, z * PDG_ANGSTROMS_TO_BOHRS, r * PDG_ANGSTROMS_TO_BOHRS,
                max(s.atom_norb[i], s.atom_norb[j]), false, q);
    Rotation rot;
    rot_assemble(q, false, rot);
    for (int a = 0; a < 4; a++) for (int m = 0; m < 4; m++) T[a][m] = rot.T[a][m];
}

// Local 4 x 4 blocks from the outputs: off-diagonal L, one-centre contributions Mi, Mj.
__device__ __forceinline__ void guess_local(const float *y, double L[4][4], double Mi[4][4], double Mj[4][4])
{
    for (int a = 0; a < 4; a++) for (int b = 0; b < 4; b++) { L[a][b] = 0.0; Mi[a][b] = 0.0; Mj[a][b] = 0.0; }
    L[0][0] = y[0]; L[0][1] = y[1]; L[1][0] = y[2]; L[1][1] = y[3]; L[2][2] = y[4]; L[3][3] = y[4];
    Mi[0][0] = y[5]; Mi[0][1] = Mi[1][0] = y[6]; Mi[1][1] = y[7]; Mi[2][2] = Mi[3][3] = y[8];
    Mj[0][0] = y[9]; Mj[0][1] = Mj[1][0] = y[10]; Mj[1][1] = y[11]; Mj[2][2] = Mj[3][3] = y[12];
}

__device__ __forceinline__ double rot_elem(const double T[4][4], const double L[4][4], int a, int b)
{
    double t = 0.0;
    for (int m = 0; m < 4; m++) for (int n = 0; n < 4; n++) t += T[a][m] * L[m][n] * T[b][n];
    return t;
}

__global__ void __launch_bounds__(256) k_guess_assemble(DeviceSystem s, int n_frames, const double *__restrict__ xyz,
                                                        const int *__restrict__ offsets, const int *__restrict__ row_pair,
                                                        const float *__restrict__ Y, double *__restrict__ P)
{
    __shared__ double red[32];
    const int f = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    const int N = s.n_basis, r0 = offsets[f], r1 = offsets[f + 1];
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    double *Pf = P + (size_t)f * N * N;
    const double g0 = (double)s.n_electrons / (double)N;
    for (size_t e = tid; e < (size_t)N * N; e += blockDim.x) Pf[e] = ((e / N) == (e % N)) ? g0 : 0.0;
    __syncthreads();
    // off-diagonal blocks: one row (pair) per thread
    for (int r = r0 + tid; r < r1; r += blockDim.x) {
        const int p = row_pair[r], i = s.pair_i[p], j = s.pair_j[p];
        double T[4][4], L[4][4], Mi[4][4], Mj[4][4];
        guess_rotation(s, R, p, T);
        guess_local(Y + (size_t)r * GUESS_OUT, L, Mi, Mj);
        const int noi = s.atom_norb[i], noj = s.atom_norb[j], is = s.atom_start[i], js = s.atom_start[j];
        for (int a = 0; a < noi; a++)
            for (int b = 0; b < noj; b++) {
                const double v = rot_elem(T, L, a, b);
                Pf[(size_t)(is + a) * N + js + b] = v;
                Pf[(size_t)(js + b) * N + is + a] = v;
            }
    }
    __syncthreads();
    // one-centre blocks: a warp per atom gathers the contributions of its pairs in row order
    for (int A = w; A < s.n_atoms; A += nw) {
        const int no = s.atom_norb[A], as = s.atom_start[A];
        double acc[16];
        for (int k = 0; k < 16; k++) acc[k] = 0.0;
        for (int r = r0 + lane; r < r1; r += 32) {
            const int p = row_pair[r], i = s.pair_i[p], j = s.pair_j[p];
            if (i != A && j != A) continue;
            double T[4][4], L[4][4], Mi[4][4], Mj[4][4];
            guess_rotation(s, R, p, T);
            guess_local(Y + (size_t)r * GUESS_OUT, L, Mi, Mj);
            for (int a = 0; a < no; a++)
                for (int b = 0; b < no; b++) acc[a * 4 + b] += rot_elem(T, i == A ? Mi : Mj, a, b);
        }
        for (int k = 0; k < 16; k++) acc[k] = warp_sum(acc[k]);
        if (lane < no * no) { const int a = lane / no, b = lane % no; Pf[(size_t)(as + a) * N + as + b] += acc[a * 4 + b]; }
    }
    __syncthreads();
    // electron count: spread the trace defect over the diagonal
    double t = 0.0;
    for (int k = tid; k < N; k += blockDim.x) t += Pf[(size_t)k * N + k];
    t = block_sum(t, red);
    const double d = ((double)s.n_electrons - t) / (double)N;
    for (int k = tid; k < N; k += blockDim.x) Pf[(size_t)k * N + k] += d;
}

// Training: squared error of the assembled blocks against the target densities; gradient with respect to the
// 16 outputs of every row (rotated back to the local frame), and the loss per frame.
__global__ void __launch_bounds__(256) k_guess_loss(DeviceSystem s, int n_frames, const double *__restrict__ xyz,
                                                    const int *__restrict__ offsets, const int *__restrict__ row_pair,
                                                    const double *__restrict__ P, const double *__restrict__ Ptarget,
                                                    float *__restrict__ dY, double *__restrict__ loss)
{
    __shared__ double red[32];
    const int f = blockIdx.x, tid = threadIdx.x, N = s.n_basis, r0 = offsets[f], r1 = offsets[f + 1];
    const double *R = xyz + (size_t)f * 3 * s.n_atoms;
    const double *Pf = P + (size_t)f * N * N, *Tf = Ptarget + (size_t)f * N * N;
    double l = 0.0;
    for (int r = r0 + tid; r < r1; r += blockDim.x) {
        const int p = row_pair[r], i = s.pair_i[p], j = s.pair_j[p];
        const int noi = s.atom_norb[i], noj = s.atom_norb[j], is = s.atom_start[i], js = s.atom_start[j];
        double T[4][4];
        guess_rotation(s, R, p, T);
        double G[4][4] = {}, Gi[4][4] = {}, Gj[4][4] = {};
        for (int a = 0; a < noi; a++)
            for (int b = 0; b < noj; b++) {
                const double gv = Pf[(size_t)(is + a) * N + js + b] - Tf[(size_t)(is + a) * N + js + b];
                G[a][b] = 2.0 * gv;   // the block appears twice in P
                l += 2.0 * 0.5 * gv * gv;
            }
        for (int a = 0; a < noi; a++) for (int b = 0; b < noi; b++) Gi[a][b] = Pf[(size_t)(is + a) * N + is + b] - Tf[(size_t)(is + a) * N + is + b];
        for (int a = 0; a < noj; a++) for (int b = 0; b < noj; b++) Gj[a][b] = Pf[(size_t)(js + a) * N + js + b] - Tf[(size_t)(js + a) * N + js + b];
        // local-frame gradients: T^T G T
        double Lg[4][4], Ig[4][4], Jg[4][4];
        for (int m = 0; m < 4; m++)
            for (int n = 0; n < 4; n++) {
                double a1 = 0.0, a2 = 0.0, a3 = 0.0;
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) {
                        const double tt = T[a][m] * T[b][n];
                        a1 += tt * G[a][b]; a2 += tt * Gi[a][b]; a3 += tt * Gj[a][b];
                    }
                Lg[m][n] = a1; Ig[m][n] = a2; Jg[m][n] = a3;
            }
        float *d = dY + (size_t)r * GUESS_OUT;
        d[0] = (float)Lg[0][0]; d[1] = (float)Lg[0][1]; d[2] = (float)Lg[1][0]; d[3] = (float)Lg[1][1]; d[4] = (float)(Lg[2][2] + Lg[3][3]);
        d[5] = (float)Ig[0][0]; d[6] = (float)(Ig[0][1] + Ig[1][0]); d[7] = (float)Ig[1][1]; d[8] = (float)(Ig[2][2] + Ig[3][3]);
        d[9] = (float)Jg[0][0]; d[10] = (float)(Jg[0][1] + Jg[1][0]); d[11] = (float)Jg[1][1]; d[12] = (float)(Jg[2][2] + Jg[3][3]);
        d[13] = d[14] = d[15] = 0.0f;
    }
    // one-centre blocks enter the loss once per atom
    for (int A = tid; A < s.n_atoms; A += blockDim.x) {
        const int no = s.atom_norb[A], as = s.atom_start[A];
        for (int a = 0; a < no; a++)
            for (int b = 0; b < no; b++) {
                const double gv = Pf[(size_t)(as + a) * N + as + b] - Tf[(size_t)(as + a) * N + as + b];
                l += 0.5 * gv * gv;
            }
    }
    l = block_sum(l, red);
    if (tid == 0) loss[f] = l;
}

// ---------------------------------------------------------------------------------------------------
// Launchers (row counts stay on the device; grids are sized by the upper bound n_frames * n_pairs)
void launch_guess_features(const DeviceSystem &s, int n_frames, const double *xyz, const double *phi, float *env, int *count,
                           int *offsets, float *X, int *row_frame, int *row_pair, cudaStream_t st)
{
    const long na = (long)n_frames * s.n_atoms;
    k_guess_env<<<(int)((na + 255) / 256), 256, 0, st>>>(n_frames, s.n_atoms, s.atom_elem, xyz, env);
    k_guess_count<<<n_frames, 256, 0, st>>>(s, n_frames, xyz, count);
    k_guess_scan<<<1, 32, 0, st>>>(n_frames, count, offsets);
    k_guess_features<<<n_frames, 256, 0, st>>>(s, n_frames, xyz, phi, env, offsets, X, row_frame, row_pair);
}

void launch_mlp_forward(int max_rows, const int *rows, int K, int N, const float *X, const void *W, const float *b, float *Z, float *H,
                        int act, cudaStream_t st)
{
    dim3 g((max_rows + 63) / 64, (N + 63) / 64);
    k_mlp_forward<<<g, 256, 0, st>>>(rows, K, N, X, (const __nv_bfloat16 *)W, b, Z, H, act);
}

void launch_mlp_backward(int max_rows, const int *rows, int N, int K, const float *dZ, const void *W, const float *Zin, const float *Hin,
                         float *dZin, int segments, float *part, cudaStream_t st)
{
    if (dZin) {
        dim3 g((max_rows + 63) / 64, (K + 63) / 64);
        k_mlp_backward_data<<<g, 256, 0, st>>>(rows, N, K, dZ, (const __nv_bfloat16 *)W, Zin, dZin);
    }
    dim3 gw((N + 63) / 64, (K + 1 + 63) / 64, segments);
    k_mlp_backward_weights<<<gw, 256, 0, st>>>(rows, segments, N, K, dZ, Hin, part);
}

void launch_mlp_adam(int N, int K, int segments, const float *part, float scale, float *Wm, float *bm, float *m1, float *m2, void *W,
                     float lr, float b1, float b2, float c1, float c2, cudaStream_t st)
{
    const int n = N * (K + 1);
    k_mlp_adam<<<(n + 255) / 256, 256, 0, st>>>(N, K, segments, part, scale, Wm, bm, m1, m2, (__nv_bfloat16 *)W, lr, b1, b2, c1, c2);
}

void launch_guess_assemble(const DeviceSystem &s, int n_frames, const double *xyz, const int *offsets, const int *row_pair,
                           const float *Y, double *P, cudaStream_t st)
{
    k_guess_assemble<<<n_frames, 256, 0, st>>>(s, n_frames, xyz, offsets, row_pair, Y, P);
}

void launch_guess_loss(const DeviceSystem &s, int n_frames, const double *xyz, const int *offsets, const int *row_pair, const double *P,
                       const double *Ptarget, float *dY, double *loss, cudaStream_t st)
{
    k_guess_loss<<<n_frames, 256, 0, st>>>(s, n_frames, xyz, offsets, row_pair, P, Ptarget, dY, loss);
}
