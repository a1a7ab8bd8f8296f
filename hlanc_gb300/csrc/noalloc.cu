// noalloc.cu -- residual verifier that allocates no memory.
//
// hlanc_residuals_device (engine.cu) allocates its partial-sum buffers on
// every call.  Some callers cannot allocate device memory at that point: a
// serving process whose HBM pool is already fully claimed by its own
// allocator, or a monitoring loop that checks Ritz pairs between solves and
// must not pay (or wait on) a cudaMalloc/cudaFree.  This file gives them one
// entry point with the same result whose scratch lives in a file-scope
// __device__ array of fixed size: HLANC_NOALLOC_MAX_PAIRS pairs.
//
// Every GPU that loads the library keeps this array (about 513 KB) until the
// process exits.  All calls share it, and it keeps the last call's contents:
// every slot a call reads is written earlier in the same call, so nothing has
// to start at zero, but calls that overlap on the GPU (from several host
// threads or streams) race on the array and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (there it is a
// host-side stand-in), so the first call on each device looks the address up
// with cudaGetSymbolAddress, with that device current, and caches it with the
// device's current context; a call that finds a different context (the old
// one was destroyed, e.g. by cudaDeviceReset, and the module loaded afresh)
// looks it up again.  Make the first call on a device, and the first after
// such a reset, outside any stream capture.
#include <cuda.h>            // CUcontext only; the driver call is found through the runtime
#include <cuda_runtime.h>

#include <mutex>

#include "internal.cuh"

namespace {

// cuCtxGetCurrent, looked up once through the runtime (no link against the
// driver library); null if unavailable, in which case every call looks the
// scratch address up again.
typedef CUresult (*ctx_get_fn)(CUcontext *);
ctx_get_fn ctx_get() {
    static const ctx_get_fn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return (ctx_get_fn)p;
    }();
    return fn;
}

constexpr int NA_BLOCKS = 256;                       // CTAs per pair
constexpr int NA_MAX = HLANC_NOALLOC_MAX_PAIRS;      // pairs per call
constexpr int NA_PART = NA_MAX * NA_BLOCKS * 4;      // per-CTA partials
constexpr int NA_TOTAL = NA_PART + 2 * NA_MAX;       // + resid / rdiff results

static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
double *g_na_ptr[NA_MAX_DEVICES] = {nullptr};
CUcontext g_na_ctx[NA_MAX_DEVICES] = {nullptr};

// Per CTA of pair i: sum of squares of A v - lambda v, max |A v - lambda v|,
// max |A v|, max |lambda v| over its rows (the quantities of verify_eigs).
__global__ void __launch_bounds__(256) k_na_resid_part(const int *__restrict__ rp, const int *__restrict__ ci,
                                                       const double *__restrict__ val, int n,
                                                       const double *__restrict__ values,
                                                       const double *__restrict__ V, int ldv,
                                                       double *__restrict__ scratch) {
    const int i = blockIdx.y;
    const double lam = values[i];
    const double *v = V + (size_t)i * ldv;
    double ss = 0.0, md = 0.0, ma = 0.0, mb = 0.0;
    for (int r = blockIdx.x * 256 + threadIdx.x; r < n; r += gridDim.x * 256) {
        double acc = 0.0;
        for (int q = rp[r]; q < rp[r + 1]; ++q) acc = fma(val[q], v[ci[q]], acc);
        const double lv = lam * v[r];
        const double d = acc - lv;
        ss = fma(d, d, ss);
        md = fmax(md, fabs(d));
        ma = fmax(ma, fabs(acc));
        mb = fmax(mb, fabs(lv));
    }
    __shared__ double sh[4][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
        ma = fmax(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mb = fmax(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    if (lane == 0) { sh[0][warp] = ss; sh[1][warp] = md; sh[2][warp] = ma; sh[3][warp] = mb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0, d = 0;
        for (int w = 0; w < 8; ++w) { a += sh[0][w]; b = fmax(b, sh[1][w]); c = fmax(c, sh[2][w]); d = fmax(d, sh[3][w]); }
        double *o = scratch + ((size_t)i * gridDim.x + blockIdx.x) * 4;
        o[0] = a; o[1] = b; o[2] = c; o[3] = d;
    }
}

// resid[i] = sqrt(sum), rdiff[i] = max|d| / max(max|Av|, max|lambda v|).
__global__ void k_na_resid_final(int nblk, int k, double *__restrict__ scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    double a = 0, b = 0, c = 0, d = 0;
    for (int q = 0; q < nblk; ++q) {
        const double *o = scratch + ((size_t)i * nblk + q) * 4;
        a += o[0]; b = fmax(b, o[1]); c = fmax(c, o[2]); d = fmax(d, o[3]);
    }
    const double mx = fmax(c, d);
    scratch[NA_PART + i] = sqrt(a);
    scratch[NA_PART + NA_MAX + i] = mx > 0.0 ? b / mx : b;
}

// Device address of the scratch array on `dev`, which must be current:
// looked up once per device and context.
int scratch_for(int dev, double **out) {
    if (dev < 0 || dev >= NA_MAX_DEVICES) return HLANC_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_na_mu);
    CUcontext ctx = nullptr;
    const ctx_get_fn get = ctx_get();
    if (get && get(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    if (!g_na_ptr[dev] || !ctx || ctx != g_na_ctx[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return HLANC_ERR_CUDA;
        CUcontext now = nullptr;       // the lookup may have created the primary context
        if (get && get(&now) != CUDA_SUCCESS) now = nullptr;
        g_na_ptr[dev] = static_cast<double *>(p);
        g_na_ctx[dev] = now;
    }
    *out = g_na_ptr[dev];
    return HLANC_OK;
}

}  // namespace

extern "C" int hlanc_residuals_device_noalloc(hlanc_csr_t csr, int k, const double *values_d,
                                              const double *vectors_d, int ldv_d, double *resid_h,
                                              double *rdiff_h) {
    hlanc::CsrView c;
    if (!csr || k <= 0 || !values_d || !vectors_d) return HLANC_ERR_INVALID;
    if (hlanc::csr_view_of(csr, &c) != HLANC_OK || ldv_d < c.nrows || c.ncols > c.nrows) return HLANC_ERR_INVALID;
    if (k > NA_MAX) return HLANC_ERR_UNSUPPORTED;   // more pairs than the fixed scratch holds
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c.dev) cudaSetDevice(c.dev);
    double *scratch = nullptr;
    int rc = scratch_for(c.dev, &scratch);
    if (rc) {
        if (prev != c.dev) cudaSetDevice(prev);
        return rc;
    }
    int nblk = (c.nrows + 255) / 256;
    if (nblk > NA_BLOCKS) nblk = NA_BLOCKS;
    if (nblk < 1) nblk = 1;
    k_na_resid_part<<<dim3(nblk, k), 256, 0, c.stream>>>(c.rp_d, c.ci_d, c.val_d, c.nrows, values_d, vectors_d,
                                                         ldv_d, scratch);
    k_na_resid_final<<<(k + 127) / 128, 128, 0, c.stream>>>(nblk, k, scratch);
    hlanc::launch_counter() += 2;
    cudaError_t e = cudaGetLastError();
    // each output is optional, as in hlanc_residuals_device
    if (e == cudaSuccess && resid_h)
        e = cudaMemcpyAsync(resid_h, scratch + NA_PART, sizeof(double) * k, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess && rdiff_h)
        e = cudaMemcpyAsync(rdiff_h, scratch + NA_PART + NA_MAX, sizeof(double) * k, cudaMemcpyDeviceToHost,
                            c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (prev != c.dev) cudaSetDevice(prev);
    return e == cudaSuccess ? HLANC_OK : HLANC_ERR_CUDA;
}
