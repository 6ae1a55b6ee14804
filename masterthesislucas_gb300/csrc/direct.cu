// O(N^2) direct sums on the GPU: the counterpart of NBodySolverNaive
// (src/nbodysolvers/cpu/nBodySolverNaive.h:53-112, FP64 "truth" of the
// reference) and of the reference's GPU naive kernel cudaTsneNaiveStepRep
// (src/nbodysolvers/gpu/nBodySolverGpuNaive.cu:50-81).
//
// Each block takes 256 sink rows and one slice of the sources; sources are
// staged through shared memory.  Per-(row, slice) partials are summed in a
// fixed order by a second kernel, so results are deterministic.  In FP64 this
// is the oracle the force error of every tree result is measured against
// (median over sampled sinks of |F - F_direct| / |F_direct|).
#include <mutex>

#include "kernels.cuh"
#include "state.cuh"

namespace tc {
namespace {

constexpr int DT = 256;

template <typename real, typename K>
__global__ void __launch_bounds__(DT) k_direct(K ker, const double2* __restrict__ pos, int64_t n,
                                               const int64_t* __restrict__ rows, int64_t m, int64_t slice,
                                               double* __restrict__ part)
{
    __shared__ real sx[DT], sy[DT];
    const int64_t r = (int64_t)blockIdx.x * DT + threadIdx.x;
    const bool act = r < m;
    const int64_t i = act ? (rows ? rows[r] : r) : 0;
    const double2 pi = pos[i];
    const real xi = (real)pi.x, yi = (real)pi.y;
    real gx = 0, gy = 0, z = 0;
    const int64_t j0 = (int64_t)blockIdx.y * slice;
    const int64_t j1 = j0 + slice < n ? j0 + slice : n;
    for (int64_t t0 = j0; t0 < j1; t0 += DT) {
        const int64_t j = t0 + threadIdx.x;
        if (j < j1) {
            double2 q = pos[j];
            sx[threadIdx.x] = (real)q.x;
            sy[threadIdx.x] = (real)q.y;
        }
        __syncthreads();
        const int cnt = (int)((j1 - t0) < DT ? (j1 - t0) : DT);
        if (act) {
            for (int k = 0; k < cnt; k++) {
                if (t0 + k == i) continue;
                const real Rx = xi - sx[k], Ry = yi - sy[k];
                real D1, t;
                ker.near(Rx * Rx + Ry * Ry, D1, t);
                gx += D1 * Rx;
                gy += D1 * Ry;
                z += t;
            }
        }
        __syncthreads();
    }
    if (act) {
        double* o = part + ((int64_t)blockIdx.y * m + r) * 3;
        o[0] = (double)gx;
        o[1] = (double)gy;
        o[2] = (double)z;
    }
}

__global__ void k_direct_reduce(const double* __restrict__ part, int64_t m, int nslice, double* __restrict__ grad,
                                double* __restrict__ zrow)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        double gx = 0, gy = 0, z = 0;
        for (int s = 0; s < nslice; s++) {
            const double* o = part + ((int64_t)s * m + r) * 3;
            gx += o[0];
            gy += o[1];
            z += o[2];
        }
        grad[2 * r] = gx;
        grad[2 * r + 1] = gy;
        zrow[r] = z;
    }
}

__global__ void k_sum_rows(const double* __restrict__ z, int64_t m, double* __restrict__ out)
{
    __shared__ double ws[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s += z[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *out = v;
    }
}

template <typename real, typename K>
int direct_t(K ker, const double* d_pos, int64_t n, const int64_t* d_rows, int64_t m, double* d_grad, double* d_total,
             cudaStream_t s)
{
    const int64_t rb = (m + DT - 1) / DT;
    // enough slices to fill the GPU several times over
    int64_t nslice = (sm_count() * 8 + rb - 1) / rb;
    if (nslice < 1) nslice = 1;
    int64_t slice = (n + nslice - 1) / nslice;
    slice = ((slice + DT - 1) / DT) * DT;
    nslice = (n + slice - 1) / slice;
    if (nslice > 65535) return TC_ERR_INVALID;
    void* part = nullptr;
    void* zrow = nullptr;
    TC_CUDA_TRY(cudaMallocAsync(&part, (size_t)(nslice * m * 3) * 8, s));
    TC_CUDA_TRY(cudaMallocAsync(&zrow, (size_t)m * 8, s));
    dim3 grid((unsigned)rb, (unsigned)nslice);
    k_direct<real, K><<<grid, DT, 0, s>>>(ker, (const double2*)d_pos, n, d_rows, m, slice, (double*)part);
    k_direct_reduce<<<grid_for(m, 256), 256, 0, s>>>((const double*)part, m, (int)nslice, d_grad, (double*)zrow);
    if (d_total) k_sum_rows<<<1, 1024, 0, s>>>((const double*)zrow, m, d_total);
    TC_CUDA_TRY(cudaFreeAsync(part, s));
    TC_CUDA_TRY(cudaFreeAsync(zrow, s));
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace
}  // namespace tc

using namespace tc;

extern "C" int tc_direct_device(int kernel, double softening, int precision, const double* d_pos, int64_t n,
                                const int64_t* d_rows, int64_t m, double* d_grad_rows, double* d_total, void* stream)
{
    // without a row list the sinks are points 0..m-1, so m may not exceed n
    if (!d_pos || !d_grad_rows || n <= 0 || m <= 0 || (kernel != TC_KERNEL_TSNE && kernel != TC_KERNEL_GRAVITY) ||
        (precision != TC_PREC_FP32 && precision != TC_PREC_FP64) || (!d_rows && m > n)) {
        tc_set_error("tc_direct_device: invalid arguments");
        return TC_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const double e2 = softening * softening;
    if (precision == TC_PREC_FP64) {
        if (kernel == TC_KERNEL_GRAVITY)
            return direct_t<double>(KGrav<double>{e2}, d_pos, n, d_rows, m, d_grad_rows, d_total, s);
        return direct_t<double>(KTsne<double>{}, d_pos, n, d_rows, m, d_grad_rows, d_total, s);
    }
    if (kernel == TC_KERNEL_GRAVITY)
        return direct_t<float>(KGrav<float>{(float)e2}, d_pos, n, d_rows, m, d_grad_rows, d_total, s);
    return direct_t<float>(KTsne<float>{}, d_pos, n, d_rows, m, d_grad_rows, d_total, s);
}

extern "C" int tc_direct(int kernel, double softening, int precision, const double* pos, int64_t n,
                         const int64_t* rows, int64_t m, double* grad_rows, double* total)
{
    if (!pos || !grad_rows || n <= 0) {
        tc_set_error("tc_direct: invalid arguments");
        return TC_ERR_INVALID;
    }
    if (!rows) m = n;
    cudaStream_t s;
    TC_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    void *dp = nullptr, *dr = nullptr, *dg = nullptr, *dt = nullptr;
    int rc = TC_OK;
    cudaError_t e = cudaMallocAsync(&dp, (size_t)n * 16, s);
    if (e == cudaSuccess && rows) e = cudaMallocAsync(&dr, (size_t)m * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dg, (size_t)m * 16, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dt, 8, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp, pos, (size_t)n * 16, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && rows) e = cudaMemcpyAsync(dr, rows, (size_t)m * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        rc = tc_direct_device(kernel, softening, precision, (const double*)dp, n, (const int64_t*)dr, m, (double*)dg,
                              (double*)dt, s);
        if (rc == TC_OK) e = cudaMemcpyAsync(grad_rows, dg, (size_t)m * 16, cudaMemcpyDeviceToHost, s);
        if (rc == TC_OK && e == cudaSuccess && total) e = cudaMemcpyAsync(total, dt, 8, cudaMemcpyDeviceToHost, s);
    }
    if (dp) cudaFreeAsync(dp, s);
    if (dr) cudaFreeAsync(dr, s);
    if (dg) cudaFreeAsync(dg, s);
    if (dt) cudaFreeAsync(dt, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc != TC_OK) return rc;
    if (e != cudaSuccess) return tc_cuda_fail(e, "tc_direct");
    if (e2 != cudaSuccess) return tc_cuda_fail(e2, "tc_direct sync");
    return TC_OK;
}

// ----------------------------------------------------------------------------
// Allocation-free variant of tc_direct_device.
//
// Some callers cannot call cudaMalloc: code running while a CUDA graph is being
// captured on the stream they hand us, allocators that forbid stray device
// allocations (for example a host framework that owns and pools all device
// memory), or real-time loops where an allocation may block on the driver.
// This entry point therefore allocates nothing: its per-slice partial sums
// live in one file-scope device array of TC_DIRECT_NOALLOC_SCRATCH doubles
// (4 MiB), which every GPU that loads this library holds until the process
// exits.  The caller still provides positions, rows and outputs.
//
// The array is shared by every call on a device and keeps the previous call's
// contents; each call overwrites every entry it later reads, so nothing needs
// clearing.  Calls that overlap on the GPU (two streams, or two host threads)
// race on the array and give wrong results: serialise them.
namespace tc {
namespace {

constexpr int64_t kNoAllocScratch = TC_DIRECT_NOALLOC_SCRATCH;
static __device__ __align__(256) double g_direct_scratch[kNoAllocScratch];

// device address of g_direct_scratch per device ordinal, looked up once per
// device with that device current (the host-side symbol is only a stand-in)
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

int scratch_for_current_device(double** out)
{
    int dev = 0;
    TC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        tc_set_error("tc_direct_device_noalloc: device ordinal %d out of range", dev);
        return TC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_direct_scratch);
        if (e != cudaSuccess) return tc_cuda_fail(e, "cudaGetSymbolAddress(g_direct_scratch)");
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return TC_OK;
}

template <typename real, typename K>
int direct_noalloc_t(K ker, const double* d_pos, int64_t n, const int64_t* d_rows, int64_t m, double* d_grad,
                     double* d_total, double* scratch, cudaStream_t s)
{
    const int64_t rb = (m + DT - 1) / DT;
    // as many source slices as fill the GPU and fit beside the m row sums
    int64_t fit = (kNoAllocScratch - m) / (3 * m);
    int64_t nslice = (sm_count() * 8 + rb - 1) / rb;
    if (nslice > fit) nslice = fit;
    if (nslice < 1) nslice = 1;
    int64_t slice = (n + nslice - 1) / nslice;
    slice = ((slice + DT - 1) / DT) * DT;
    nslice = (n + slice - 1) / slice;
    if (nslice * m * 3 + m > kNoAllocScratch || nslice > 65535) {
        tc_set_error("tc_direct_device_noalloc: %lld rows x %lld points need more than the %lld-double scratch",
                     (long long)m, (long long)n, (long long)kNoAllocScratch);
        return TC_ERR_INVALID;
    }
    double* part = scratch;
    double* zrow = scratch + nslice * m * 3;
    dim3 grid((unsigned)rb, (unsigned)nslice);
    k_direct<real, K><<<grid, DT, 0, s>>>(ker, (const double2*)d_pos, n, d_rows, m, slice, part);
    k_direct_reduce<<<grid_for(m, 256), 256, 0, s>>>(part, m, (int)nslice, d_grad, zrow);
    if (d_total) k_sum_rows<<<1, 1024, 0, s>>>(zrow, m, d_total);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace
}  // namespace tc

extern "C" int tc_direct_device_noalloc(int kernel, double softening, int precision, const double* d_pos, int64_t n,
                                        const int64_t* d_rows, int64_t m, double* d_grad_rows, double* d_total,
                                        void* stream)
{
    if (!d_pos || !d_grad_rows || n <= 0 || m <= 0 || (kernel != TC_KERNEL_TSNE && kernel != TC_KERNEL_GRAVITY) ||
        (precision != TC_PREC_FP32 && precision != TC_PREC_FP64) || (!d_rows && m > n)) {
        tc_set_error("tc_direct_device_noalloc: invalid arguments");
        return TC_ERR_INVALID;
    }
    // at least one source slice of 3 partials per row plus the row sums
    if (4 * m > tc::kNoAllocScratch) {
        tc_set_error("tc_direct_device_noalloc: m = %lld rows exceeds the maximum of %lld", (long long)m,
                     (long long)(tc::kNoAllocScratch / 4));
        return TC_ERR_INVALID;
    }
    double* scratch = nullptr;
    int rc = tc::scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const double e2 = softening * softening;
    if (precision == TC_PREC_FP64) {
        if (kernel == TC_KERNEL_GRAVITY)
            return direct_noalloc_t<double>(KGrav<double>{e2}, d_pos, n, d_rows, m, d_grad_rows, d_total, scratch, s);
        return direct_noalloc_t<double>(KTsne<double>{}, d_pos, n, d_rows, m, d_grad_rows, d_total, scratch, s);
    }
    if (kernel == TC_KERNEL_GRAVITY)
        return direct_noalloc_t<float>(KGrav<float>{(float)e2}, d_pos, n, d_rows, m, d_grad_rows, d_total, scratch, s);
    return direct_noalloc_t<float>(KTsne<float>{}, d_pos, n, d_rows, m, d_grad_rows, d_total, scratch, s);
}
