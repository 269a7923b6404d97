// tc.cu - check of the tcgen05 split-BF16 product on this device (pdg_tc_selftest, include/pdg.h).
//
// C = X X for a symmetric n x n FP32 matrix (n <= 144) with k split-BF16 partial products accumulated in
// FP32 tensor memory: k = 1 hi.hi; k = 3 adds hi.mid + mid.hi; k = 6 adds mid.mid + hi.lo + lo.hi.  Rows
// 0..127 come from one M = 128 tcgen05 tile; rows 128..n-1 are the transposed columns of that tile (X X is
// symmetric) except the trailing 16 x 16 corner, which FP32 cores compute directly.  This is the product the
// purification density step runs every iteration.
//
// kprod = 0 checks the bounded completion wait itself: the kernel initialises the barrier, issues no tcgen05
// operation at all (no tensor-memory allocation, no product, no commit), waits wait_limit polls on the barrier
// that nothing will ever arrive on, and reports status 1.  That is the path every tensor-core wait of the SCF
// takes when a completion never comes: it gives up and reports, it does not hang.
#include "tc.cuh"

#define TC_THREADS 256
#define TC_WAIT_LIMIT (1 << 22)

__global__ void __launch_bounds__(TC_THREADS) k_tc_selftest(int n, int kprod, int wait_limit, const float *__restrict__ X,
                                                            float *__restrict__ C, int *__restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ uint32_t taddr_s;
    __shared__ __align__(8) uint64_t bar_s;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (kprod == 0) {
        if (tid == 0) {
            const uint32_t bar = tc_smem_addr(&bar_s);
            mbar_init(bar, 1);
            *status = mbar_wait(bar, 0, wait_limit) ? 0 : 1;
        }
        return;
    }
    const int Kp = (n + 15) & ~15, R = Kp > TC_M ? Kp : TC_M;
    const size_t part = (size_t)R * Kp * 2;
    unsigned char *ph = tsm, *pm = tsm + part, *pl = tsm + 2 * part;
    const uint32_t bar = tc_smem_addr(&bar_s);
    if (w == 0) tc_alloc(tc_smem_addr(&taddr_s), 256);
    if (tid == 0) mbar_init(bar, 1);
    for (int e = tid; e < R * Kp; e += TC_THREADS) {
        const int r = e / Kp, c = e % Kp;
        const float x = (r < n && c < n) ? X[(size_t)r * n + c] : 0.0f;
        __nv_bfloat16 h, m, l;
        bf16_split3(x, h, m, l);
        const uint32_t o = tc_offset(r, c, Kp);
        *(__nv_bfloat16 *)(ph + o) = h; *(__nv_bfloat16 *)(pm + o) = m; *(__nv_bfloat16 *)(pl + o) = l;
    }
    tc_fence_proxy();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;
    if (tid == 0) {
        const uint32_t H = tc_smem_addr(ph), M = tc_smem_addr(pm), L = tc_smem_addr(pl);
        const uint32_t pa[6] = { H, H, M, M, H, L }, pb[6] = { H, M, H, M, L, H };
        for (int q = 0; q < kprod; q++) tc_product(taddr, pa[q], 0, pb[q], Kp, Kp, q > 0);
        tc_commit(bar);
    }
    const bool ok = mbar_wait(bar, 0, wait_limit);
    tc_fence_after();
    // accumulator rows 0..127: lane quarter w % 4; warps 0-3 and 4-7 split the column chunks
    const int nch = Kp / 16, half = (nch + 1) / 2, c0 = w < 4 ? 0 : half, c1 = w < 4 ? half : nch;
    const int r = 32 * (w & 3) + lane;
    for (int ch = c0; ch < c1; ch++) {
        float v[16];
        tc_ld16(taddr + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(ch * 16), v);
        for (int j = 0; j < 16; j++) {
            const int c = ch * 16 + j;
            if (r < n && c < n) {
                C[(size_t)r * n + c] = v[j];
                if (c >= TC_M) C[(size_t)c * n + r] = v[j];
            }
        }
    }
    for (int e = tid; e < (n - TC_M) * (n - TC_M) && n > TC_M; e += TC_THREADS) {
        const int rr = TC_M + e / (n - TC_M), cc = TC_M + e % (n - TC_M);
        float t = 0.0f;
        for (int k = 0; k < n; k++) t = fmaf(X[(size_t)rr * n + k], X[(size_t)k * n + cc], t);
        C[(size_t)rr * n + cc] = t;
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) tc_dealloc(taddr, 256);
    if (tid == 0) *status = ok ? 0 : 1;
}

int launch_tc_selftest(int n, int kprod, int wait_limit, const float *x, float *c, int *status, cudaStream_t st)
{
    const int Kp = (n + 15) & ~15, R = Kp > TC_M ? Kp : TC_M;
    const size_t sm = kprod == 0 ? 0 : (size_t)3 * R * Kp * 2;
    cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_tc_selftest<<<1, TC_THREADS, sm, st>>>(n, kprod, wait_limit > 0 ? wait_limit : TC_WAIT_LIMIT, x, c, status);
    return 0;
}
