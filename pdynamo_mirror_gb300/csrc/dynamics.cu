// dynamics.cu - Langevin velocity Verlet dynamics of the QC atoms of many independent replicas, and the linear
// combination of densities that starts each step's SCF.
//
// The integrator restates pDynamo's LangevinVelocityVerletIntegrator.Iteration
// (pCore-1.9.0/pCore/LangevinVelocityVerletIntegrator.py:126-155): with mass-weighted variables x_w = sqrt(m) x,
//   x_w += facR1 v_w + facR2 a_w ;  v_w = facV1 v_w + facV2 a_w ;
//   w1 ~ N(0,1): x_w += sdR w1, v_w += sdV1 w1 ;  w2 ~ N(0,1): v_w += sdV2 w2 ;
//   a_w = -100 g / sqrt(m) at the new point (SystemGeometryObjectiveFunction.py:62-66, kJ/mol -> amu A^2 ps^-2) ;
//   v_w += facV3 a_w.
// Here the same update is applied to unweighted Cartesian coordinates (Angstrom), velocities (A/ps) and
// accelerations (A/ps^2): dividing every line by sqrt(m) gives x += facR1 v + facR2 a, v = facV1 v + facV2 a,
// x += sdR w1 / sqrt(m), v += (sdV1 w1 + sdV2 w2) / sqrt(m), a = -100 g / m.  Only free atoms move; fixed atoms
// (System.DefineFixedAtoms) keep their coordinates, as the objective function's freeAtoms selection does
// (SystemGeometryObjectiveFunction.py:138-152).  With fixed atoms the reference removes no rotation or
// translation (:213-222).  Without them its LangevinDynamics_SystemGeometry removes both
// (MolecularDynamics.py:27-32): orthonormal mass-weighted rotation and translation vectors V, made once from the
// starting coordinates (Coordinates3_RotationTranslationVectors), are projected out of the assigned velocities,
// of both deviate vectors (RandomForces, LangevinVelocityVerletIntegrator.py:147-157) and of the gradients
// (GradientsGet, :177-183).  k_linear_project does that projection for any array whose weighted form is
// x_w = s x: x_w -= V (V^T x_w), with s = sqrt(m) for velocities, 1 for the deviates, 1 / sqrt(m) for gradients.
//
// Normal deviates come from a counter-based generator, so a replica's stream depends only on (seed, replica,
// element, step) and not on launch shape: Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011) gives four 32-bit words per (counter, key); two 53-bit uniforms are
// formed from them and the Box-Muller transform turns them into the pair (w1, w2).  The reference draws its
// deviates from its own generator (RandomDeviateGenerator.NormalDeviateGenerator); trajectories are therefore
// compared with it for given deviates, which pdg_langevin_positions can return.
#include "common.cuh"

namespace {

constexpr uint32_t PHILOX_M0 = 0xD2511F53u, PHILOX_M1 = 0xCD9E8D57u;
constexpr uint32_t PHILOX_W0 = 0x9E3779B9u, PHILOX_W1 = 0xBB67AE85u;

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = PHILOX_M0 * c[0], hi0 = __umulhi(PHILOX_M0, c[0]);
        const uint32_t lo1 = PHILOX_M1 * c[2], hi1 = __umulhi(PHILOX_M1, c[2]);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
}

// Two standard normal deviates for counter (element, stream, step) under key seed.
__device__ __forceinline__ void normal_pair(uint64_t element, uint32_t step, uint32_t stream, uint64_t seed, double &w1, double &w2)
{
    uint32_t c[4] = { (uint32_t)element, (uint32_t)(element >> 32), step, stream };
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    // 53-bit uniforms in [0, 1): the top 26 and 27 bits of two words each
    const double u1 = (double)(((uint64_t)(c[0] >> 6) << 27) | (c[1] >> 5)) * 0x1.0p-53;
    const double u2 = (double)(((uint64_t)(c[2] >> 6) << 27) | (c[3] >> 5)) * 0x1.0p-53;
    const double rad = sqrt(-2.0 * log(1.0 - u1));   // 1 - u1 in (0, 1]
    double s, co;
    sincospi(2.0 * u2, &s, &co);
    w1 = rad * co;
    w2 = rad * s;
}

// First half of a step: positions, half velocities and random forces; thread per free (replica, atom, axis).
__global__ void k_langevin_positions(int n_replicas, int n_atoms, int n_free, const int *__restrict__ free_atom,
                                     const double *__restrict__ inv_sqrt_mass, double *__restrict__ xyz,
                                     double *__restrict__ vel, const double *__restrict__ acc, LangevinFactors f,
                                     uint64_t seed, uint32_t step, double *__restrict__ deviates)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)n_replicas * n_free * 3;
    if (g >= n) return;
    const int k = (int)(g % 3);
    const long long rf = g / 3;
    const int fa = (int)(rf % n_free), r = (int)(rf / n_free);
    const double s = inv_sqrt_mass[fa];
    double *x = xyz + ((size_t)r * n_atoms + free_atom[fa]) * 3 + k;
    double v = vel[g];
    const double a = acc[g];
    double xv = *x + f.facR1 * v + f.facR2 * a;
    v = f.facV1 * v + f.facV2 * a;
    double w1 = 0.0, w2 = 0.0;
    if (f.random == 1) {
        normal_pair((uint64_t)g, step, 0u, seed, w1, w2);
    } else if (f.random == 2) {                 // given (e.g. projected) deviates
        w1 = deviates[2 * g];
        w2 = deviates[2 * g + 1];
    }
    if (f.random) {
        xv += f.sdR * s * w1;
        v += (f.sdV1 * w1 + f.sdV2 * w2) * s;
    }
    *x = xv;
    vel[g] = v;
    if (deviates && f.random != 2) { deviates[2 * g] = w1; deviates[2 * g + 1] = w2; }
}

// Linear constraints (see the header): one block per replica.  Element (fa, k, c) of replica r sits at
// arr[((r n_rows + row(fa)) 3 + k) width + c] with row(fa) = rows[fa] (fa when rows is NULL); each of the width
// components is a vector of its own.  vec: n_replicas x n_vectors x n_free x 3, orthonormal; scale: s per free atom
// (NULL: 1).  Dot products in a fixed order: per thread over its strided elements, then lanes, then warps.
constexpr int LP_T = 256, LP_MAXV = 6, LP_MAXW = 2;
__global__ void __launch_bounds__(LP_T) k_linear_project(int n_free, int n_rows, const int *__restrict__ rows, int nv,
                                                         const double *__restrict__ vec, const double *__restrict__ scale, int width,
                                                         double *__restrict__ arr)
{
    __shared__ double part[LP_T / 32][LP_MAXV * LP_MAXW];
    __shared__ double dots[LP_MAXV * LP_MAXW];
    const int r = blockIdx.x;
    const int ne = 3 * n_free;
    const double *V = vec + (size_t)r * nv * ne;
    double acc[LP_MAXV * LP_MAXW];
#pragma unroll
    for (int i = 0; i < LP_MAXV * LP_MAXW; i++) acc[i] = 0.0;
    for (int e = threadIdx.x; e < ne; e += LP_T) {
        const int fa = e / 3, k = e - 3 * fa;
        const double s = scale ? scale[fa] : 1.0;
        const double *x = arr + (((size_t)r * n_rows + (rows ? rows[fa] : fa)) * 3 + k) * width;
#pragma unroll
        for (int c = 0; c < LP_MAXW; c++) {
            if (c < width) {
                const double xw = s * x[c];
#pragma unroll
                for (int v = 0; v < LP_MAXV; v++)
                    if (v < nv) acc[v * LP_MAXW + c] += V[(size_t)v * ne + e] * xw;
            }
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < LP_MAXV * LP_MAXW; i++) {
        double t = acc[i];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) part[w][i] = t;
    }
    __syncthreads();
    if (threadIdx.x < LP_MAXV * LP_MAXW) {
        double t = 0.0;
        for (int q = 0; q < LP_T / 32; q++) t += part[q][threadIdx.x];
        dots[threadIdx.x] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ne; e += LP_T) {
        const int fa = e / 3, k = e - 3 * fa;
        const double s = scale ? scale[fa] : 1.0;
        double *x = arr + (((size_t)r * n_rows + (rows ? rows[fa] : fa)) * 3 + k) * width;
#pragma unroll
        for (int c = 0; c < LP_MAXW; c++) {
            if (c < width) {
                double p = 0.0;
#pragma unroll
                for (int v = 0; v < LP_MAXV; v++)
                    if (v < nv) p += dots[v * LP_MAXW + c] * V[(size_t)v * ne + e];
                x[c] -= p / s;
            }
        }
    }
}

// Second half: accelerations from the gradients at the new point and the velocity completion, one block per
// replica; the replica's sum of m v^2 (amu A^2 ps^-2) in fixed order.  grad_a / grad_b: n_replicas x n_rows x 3
// (grad_b may be NULL), scaled by grad_scale to kJ/mol/A; free atom fa reads row grad_row[fa].
__global__ void k_langevin_velocities(int n_free, int n_rows, const int *__restrict__ grad_row, const double *__restrict__ mass,
                                      const double *__restrict__ grad_a, const double *__restrict__ grad_b, double grad_scale,
                                      double facV3, double *__restrict__ vel, double *__restrict__ acc, double *__restrict__ mv2)
{
    __shared__ double red[32];
    const int r = blockIdx.x;
    const size_t base = (size_t)r * n_free * 3;
    const size_t gbase = (size_t)r * n_rows * 3;
    double sum = 0.0;
    for (int e = threadIdx.x; e < n_free * 3; e += blockDim.x) {
        const int fa = e / 3, k = e % 3;
        const size_t gi = gbase + (size_t)grad_row[fa] * 3 + k;
        double g = grad_a[gi];
        if (grad_b) g += grad_b[gi];
        const double m = mass[fa];
        const double a = -100.0 * grad_scale * g / m;
        const double v = vel[base + e] + facV3 * a;
        acc[base + e] = a;
        vel[base + e] = v;
        sum += m * v * v;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0 && mv2) mv2[r] = t;
    }
}

// out = sum_k c_k D_k over n doubles (two per thread).
__global__ void k_density_combine(long long n, DensityTerms t, double *__restrict__ out)
{
    const long long i = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    if (i + 1 < n) {
        double2 acc = make_double2(0.0, 0.0);
        for (int k = 0; k < t.count; k++) {
            const double2 d = *reinterpret_cast<const double2 *>(t.d[k] + i);
            acc.x += t.c[k] * d.x;
            acc.y += t.c[k] * d.y;
        }
        *reinterpret_cast<double2 *>(out + i) = acc;
    } else {
        double acc = 0.0;
        for (int k = 0; k < t.count; k++) acc += t.c[k] * t.d[k][i];
        out[i] = acc;
    }
}

__global__ void k_normal_deviates(long long n_pairs, uint64_t seed, uint32_t step, uint32_t stream, double *__restrict__ out)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_pairs) return;
    double w1, w2;
    normal_pair((uint64_t)g, step, stream, seed, w1, w2);
    out[2 * g] = w1;
    out[2 * g + 1] = w2;
}

}  // namespace

void launch_langevin_positions(int n_replicas, int n_atoms, int n_free, const int *free_atom, const double *inv_sqrt_mass, double *xyz,
                               double *vel, const double *acc, const LangevinFactors &f, uint64_t seed, uint32_t step,
                               double *deviates, cudaStream_t st)
{
    const long long n = (long long)n_replicas * n_free * 3;
    const int threads = 256;
    k_langevin_positions<<<(unsigned)((n + threads - 1) / threads), threads, 0, st>>>(n_replicas, n_atoms, n_free, free_atom, inv_sqrt_mass,
                                                                                      xyz, vel, acc, f, seed, step, deviates);
}

void launch_langevin_velocities(int n_replicas, int n_free, int n_rows, const int *grad_row, const double *mass, const double *grad_a,
                                const double *grad_b, double grad_scale, double facV3, double *vel, double *acc, double *mv2,
                                cudaStream_t st)
{
    k_langevin_velocities<<<n_replicas, 256, 0, st>>>(n_free, n_rows, grad_row, mass, grad_a, grad_b, grad_scale, facV3, vel, acc, mv2);
}

void launch_density_combine(long long n, const DensityTerms &t, double *out, cudaStream_t st)
{
    const long long pairs = (n + 1) / 2;
    const int threads = 256;
    k_density_combine<<<(unsigned)((pairs + threads - 1) / threads), threads, 0, st>>>(n, t, out);
}

void launch_normal_deviates(long long n_pairs, uint64_t seed, uint32_t step, uint32_t stream, double *out, cudaStream_t st)
{
    const int threads = 256;
    k_normal_deviates<<<(unsigned)((n_pairs + threads - 1) / threads), threads, 0, st>>>(n_pairs, seed, step, stream, out);
}

void launch_linear_project(int n_replicas, int n_free, int n_rows, const int *rows, int n_vectors, const double *vectors,
                           const double *scale, int width, double *arr, cudaStream_t st)
{
    k_linear_project<<<n_replicas, LP_T, 0, st>>>(n_free, n_rows, rows, n_vectors, vectors, scale, width, arr);
}
