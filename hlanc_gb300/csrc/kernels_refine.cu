// kernels_refine.cu -- the FP64 Rayleigh-Ritz refinement of a mixed-precision
// solve.
//
// The FP32-SpMV phase of HLANC_PREC_FP32_REFINE ends with k Ritz vectors Y
// (n x k, FP64 storage, orthonormal to FP64 rounding) whose Krylov space was
// built with an operator rounded to FP32.  The refinement projects the FP64
// operator on span(Y):  W = A Y (k FP64 SpMVs), G = Y^T W (k x k), G = Z Theta
// Z^T on the host, Y' = Y Z, and the FP64 residuals ||A y'_i - theta_i y'_i||
// decide whether the pairs are accepted (the same Ritz post-processing the
// reference does with its converged basis, HLanc.hpp:1765-1843, with true
// residuals in place of its Ritz estimates, H:1693-1695).
//
//   k_gram        per-CTA partial sums of Y^T W over 64-row slabs staged in
//                 shared memory (k <= 64), in fixed slots
//   k_gram_final  the slots summed in a fixed order (deterministic)
//   k_rotate      Y' = Y Z (thread per row, Z in shared memory)
#include "internal.cuh"

namespace hlanc {

constexpr int GR_ROWS = 32;     // rows per slab (two slabs of 32 x 65 doubles: 33 KB shared)
constexpr int GR_KMAX = 64;

__global__ void __launch_bounds__(256) k_gram(const double *__restrict__ Y, const double *__restrict__ W, int n,
                                              int ld, int k, double *__restrict__ part) {
    __shared__ double ys[GR_ROWS][GR_KMAX + 1], ws[GR_ROWS][GR_KMAX + 1];
    const int tid = threadIdx.x;
    const int npair = k * k;
    double acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.0;
    for (int r0 = blockIdx.x * GR_ROWS; r0 < n; r0 += gridDim.x * GR_ROWS) {
        __syncthreads();
        for (int idx = tid; idx < GR_ROWS * k; idx += 256) {
            const int c = idx / GR_ROWS, r = idx % GR_ROWS;
            const bool ok = r0 + r < n;
            ys[r][c] = ok ? Y[(size_t)c * ld + r0 + r] : 0.0;
            ws[r][c] = ok ? W[(size_t)c * ld + r0 + r] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int p = tid + q * 256;
            if (p >= npair) break;
            const int i = p / k, j = p % k;
            double a = acc[q];
            for (int r = 0; r < GR_ROWS; ++r) a = fma(ys[r][i], ws[r][j], a);
            acc[q] = a;
        }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const int p = tid + q * 256;
        if (p < npair) part[(size_t)blockIdx.x * npair + p] = acc[q];
    }
}

__global__ void k_gram_final(const double *__restrict__ part, int nblk, int npair, double *__restrict__ G) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int b = 0; b < nblk; ++b) a += part[(size_t)b * npair + p];
        G[p] = a;
    }
}

__global__ void __launch_bounds__(256) k_rotate(const double *__restrict__ Y, int n, int ld, int k,
                                                const double *__restrict__ Z, double *__restrict__ out) {
    __shared__ double zs[GR_KMAX * GR_KMAX];
    for (int i = threadIdx.x; i < k * k; i += 256) zs[i] = Z[i];
    __syncthreads();
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256) {
        for (int p0 = 0; p0 < k; p0 += 16) {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) acc[q] = 0.0;
            for (int l = 0; l < k; ++l) {
                const double y = Y[(size_t)l * ld + r];
#pragma unroll
                for (int q = 0; q < 16; ++q)
                    if (p0 + q < k) acc[q] = fma(y, zs[l + (p0 + q) * k], acc[q]);
            }
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (p0 + q < k) out[(size_t)(p0 + q) * ld + r] = acc[q];
        }
    }
}

int gram_blocks(int n) {
    int nb = (n + GR_ROWS - 1) / GR_ROWS;
    return nb < 304 ? (nb < 1 ? 1 : nb) : 304;
}

// G (k x k, column-major, device) = Y^T W; part holds gram_blocks(n) * k * k doubles.
void launch_gram(const double *Y, const double *W, int n, int ld, int k, double *part, double *G, cudaStream_t s) {
    const int nb = gram_blocks(n);
    k_gram<<<nb, 256, 0, s>>>(Y, W, n, ld, k, part);
    k_gram_final<<<(k * k + 255) / 256, 256, 0, s>>>(part, nb, k * k, G);
    launch_counter() += 2;
}

void launch_rotate(const double *Y, int n, int ld, int k, const double *Z, double *out, cudaStream_t s) {
    int nb = (n + 255) / 256;
    if (nb > 608) nb = 608;
    k_rotate<<<nb, 256, 0, s>>>(Y, n, ld, k, Z, out);
    launch_counter() += 1;
}

}  // namespace hlanc
