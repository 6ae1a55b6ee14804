// Particle-mesh (FFT-accelerated interpolation) t-SNE repulsion:
// NBodySolverPM::solveNbody (src/nbodysolvers/cpu/nBodySolverPM.h:274-305) and
// computeFftGradient (:763-1039) with precompute_2d (:686-760) and
// n_body_fft_2d (:413-682), the published FIt-SNE scheme, in FP64 as in the
// reference.
//   1. min/max of all coordinates in one pass with the reference's `else if`:
//      a value that raises the running maximum is never taken for the minimum
//      (a value is such a "record" iff it exceeds every earlier one), found
//      here by a max-scan over the interleaved coordinates.
//   2. nb x nb boxes of side (max - min)/nb on the square [min, max]^2, p
//      Lagrange nodes per box and dimension; every point's p + p basis values.
//   3. The charges (1, x, y, x^2 + y^2) spread to the nodes: points sorted by
//      box (stable, so each node sums its points in input order like the
//      reference), one warp per box, one lane per (node, charge) accumulator,
//      the box's points staged through shared memory 32 at a time.
//   4. Convolution with (1 + r^2)^-2 on the uniform node grid: zero-padded
//      real FFTs (cuFFT D2Z / Z2D, batched over the four charges) of the
//      smallest 2,3,5,7-smooth size >= 2n1 (the reference's 2n1 can hold a
//      large prime factor; the extracted block is the same linear
//      convolution), the reference's complex product, the unnormalised inverse
//      divided by the size squared.
//   5. Potentials interpolated back; gradient x phi1 - phi2, y phi1 - phi3;
//      Z = sum (1 + |y|^2) phi1 - 2 y.phi_(2,3) + phi4 - N (FP64, fixed order).
// cuFFT is loaded at the first call (dlopen), so the rest of the library does
// not depend on it.
#include <cufft.h>
#include <dlfcn.h>

#include <cmath>
#include <map>
#include <memory>
#include <mutex>

#include "state.cuh"

namespace tc {
namespace {

constexpr int kPmMaxInterp = 8;
constexpr int kPmItems = 8;  // values per thread in the min/max passes
constexpr int kPmThreads = 256;
constexpr int kPmChunk = kPmItems * kPmThreads;

// ------------------------------------------------------------------ cuFFT, loaded at run time
struct CufftApi {
    bool tried = false, ok = false;
    decltype(&cufftPlanMany) plan_many = nullptr;
    decltype(&cufftExecD2Z) exec_d2z = nullptr;
    decltype(&cufftExecZ2D) exec_z2d = nullptr;
    decltype(&cufftSetStream) set_stream = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
};

CufftApi& cufft()
{
    static CufftApi api;
    static std::mutex m;
    std::lock_guard<std::mutex> g(m);
    if (!api.tried) {
        api.tried = true;
        void* h = dlopen("libcufft.so.12", RTLD_NOW | RTLD_GLOBAL);
        if (!h) h = dlopen("libcufft.so", RTLD_NOW | RTLD_GLOBAL);
        if (h) {
            api.plan_many = (decltype(api.plan_many))dlsym(h, "cufftPlanMany");
            api.exec_d2z = (decltype(api.exec_d2z))dlsym(h, "cufftExecD2Z");
            api.exec_z2d = (decltype(api.exec_z2d))dlsym(h, "cufftExecZ2D");
            api.set_stream = (decltype(api.set_stream))dlsym(h, "cufftSetStream");
            api.destroy = (decltype(api.destroy))dlsym(h, "cufftDestroy");
            api.ok = api.plan_many && api.exec_d2z && api.exec_z2d && api.set_stream && api.destroy;
        }
    }
    return api;
}

// ------------------------------------------------------------------ min/max with the reference's quirk
__device__ inline double block_max_d(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    v = (int)threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : -INFINITY;
    if (threadIdx.x < 32)
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v, o);
            v = u > v ? u : v;
        }
    return v;  // valid in thread 0
}

// per chunk of kPmChunk values: the largest (comparisons as the reference's `v > max`)
__global__ void __launch_bounds__(kPmThreads) k_pm_chunk_max(const double* __restrict__ v, int64_t m,
                                                             double* __restrict__ cmax)
{
    __shared__ double sh[kPmThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kPmChunk + (int64_t)threadIdx.x * kPmItems;
    double mx = -INFINITY;
    for (int r = 0; r < kPmItems; r++)
        if (base + r < m && v[base + r] > mx) mx = v[base + r];
    mx = block_max_d(mx, sh);
    if (threadIdx.x == 0) cmax[blockIdx.x] = mx;
}

// exclusive prefix maximum of the chunk maxima: one block of kPmScanThreads
// threads walks the chunks in tiles, each tile a warp-shuffle scan plus a
// scan of the warp totals, carrying the running maximum between tiles (max is
// exact, so the result does not depend on the grouping)
constexpr int kPmScanThreads = 1024;

__device__ inline double dmax_cmp(double a, double b) { return b > a ? b : a; }

__global__ void __launch_bounds__(kPmScanThreads) k_pm_chunk_premax(double* __restrict__ c, int64_t nc)
{
    __shared__ double wtot[kPmScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double carry = -INFINITY;
    for (int64_t base = 0; base < nc; base += kPmScanThreads) {
        const int64_t i = base + threadIdx.x;
        const double v = i < nc ? c[i] : -INFINITY;
        double inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc = dmax_cmp(inc, u);
        }
        if (lane == 31) wtot[w] = inc;
        __syncthreads();
        if (w == 0) {
            double t = wtot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t = dmax_cmp(t, u);
            }
            wtot[lane] = t;  // inclusive maximum over warps 0..lane
        }
        __syncthreads();
        double before = carry;
        if (w > 0) before = dmax_cmp(before, wtot[w - 1]);
        const double prev = __shfl_up_sync(0xffffffffu, inc, 1);
        if (lane > 0) before = dmax_cmp(before, prev);
        if (i < nc) c[i] = before;
        carry = dmax_cmp(carry, wtot[kPmScanThreads / 32 - 1]);
        __syncthreads();
    }
}

// per chunk: the smallest value that is not a record (v > every earlier value)
__global__ void __launch_bounds__(kPmThreads) k_pm_chunk_min(const double* __restrict__ v, int64_t m,
                                                             const double* __restrict__ cpre,
                                                             double* __restrict__ cmin)
{
    __shared__ double sh[kPmThreads / 32];
    __shared__ double tmax[kPmThreads];
    const int64_t base = (int64_t)blockIdx.x * kPmChunk + (int64_t)threadIdx.x * kPmItems;
    double mx = -INFINITY;
    for (int r = 0; r < kPmItems; r++)
        if (base + r < m && v[base + r] > mx) mx = v[base + r];
    tmax[threadIdx.x] = mx;
    __syncthreads();
    // exclusive max over the earlier threads of the chunk, then the earlier chunks
    double run = cpre[blockIdx.x];
    for (int t = 0; t < (int)threadIdx.x; t++)
        if (tmax[t] > run) run = tmax[t];
    double mn = INFINITY;
    for (int r = 0; r < kPmItems; r++) {
        if (base + r >= m) break;
        const double x = v[base + r];
        if (x > run) run = x;           // a record: the reference's `if (v > max)` branch
        else if (x < mn) mn = x;        // its `else if (v < min)` branch
    }
    __syncthreads();
    // block minimum (comparison form, so NaN never enters)
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, mn, o);
        if (u < mn) mn = u;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = INFINITY;
        for (int w = 0; w < kPmThreads / 32; w++)
            if (sh[w] < b) b = sh[w];
        cmin[blockIdx.x] = b;
    }
}

// the smallest non-record value and the largest chunk maximum, one block of
// kPmScanThreads threads (comparison form, so NaN never enters)
__global__ void __launch_bounds__(kPmScanThreads) k_pm_minmax_final(const double* __restrict__ cmin,
                                                                    const double* __restrict__ cmax_raw, int64_t nc,
                                                                    double* __restrict__ mm)
{
    __shared__ double smn[kPmScanThreads / 32], smx[kPmScanThreads / 32];
    double mn = INFINITY, mx = -INFINITY;
    for (int64_t i = threadIdx.x; i < nc; i += kPmScanThreads) {
        if (cmin[i] < mn) mn = cmin[i];
        if (cmax_raw[i] > mx) mx = cmax_raw[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
        if (a < mn) mn = a;
        if (b > mx) mx = b;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        smn[w] = mn;
        smx[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kPmScanThreads / 32; k++) {
            if (smn[k] < mn) mn = smn[k];
            if (smx[k] > mx) mx = smx[k];
        }
        mm[0] = mn;
        mm[1] = mx;
    }
}

// ------------------------------------------------------------------ points and grid
struct PmGrid {
    int p, nb, n1, nf;
    double mn, bw;
    double sp[kPmMaxInterp], den[kPmMaxInterp];
};

__device__ inline void pm_lagrange(const PmGrid& g, double t, double* w)
{
    for (int j = 0; j < g.p; j++) {
        double num = 1.0;
        for (int k = 0; k < g.p; k++)
            if (j != k) num *= t - g.sp[k];
        w[j] = num / g.den[j];
    }
}

// box key (y box * nb + x box) and the p + p Lagrange values of every point
__global__ void k_pm_points(const double2* __restrict__ pos, int64_t n, PmGrid g, uint32_t* __restrict__ key,
                            double* __restrict__ wx, double* __restrict__ wy)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 q = pos[i];
        int ix = (int)((q.x - g.mn) / g.bw), iy = (int)((q.y - g.mn) / g.bw);
        ix = ix >= g.nb ? g.nb - 1 : (ix < 0 ? 0 : ix);
        iy = iy >= g.nb ? g.nb - 1 : (iy < 0 ? 0 : iy);
        key[i] = (uint32_t)iy * (uint32_t)g.nb + (uint32_t)ix;
        const double x0 = ix * g.bw + g.mn, y0 = iy * g.bw + g.mn;
        pm_lagrange(g, (q.x - x0) / g.bw, wx + i * g.p);
        pm_lagrange(g, (q.y - y0) / g.bw, wy + i * g.p);
    }
}

// first and one-past-last sorted index of every non-empty box
__global__ void k_pm_box_ranges(const uint32_t* __restrict__ skey, int64_t n, uint32_t* __restrict__ bstart,
                                uint32_t* __restrict__ bend)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t b = skey[k];
        if (k == 0 || skey[k - 1] != b) bstart[b] = (uint32_t)k;
        if (k == n - 1 || skey[k + 1] != b) bend[b] = (uint32_t)(k + 1);
    }
}

// one warp per box: accumulator u = ((a p) + b) 4 + d (x node a, y node b,
// charge d) sums its box's points in input order and lands on node row
// bx p + a, column by p + b of charge d's zero-padded FFT input.  The box's
// points are staged 32 at a time in shared memory (one lane each), so the
// accumulators' sequential sums read no dependent global loads.
constexpr int kPmSpreadWarps = 4;
constexpr int kPmAccPerLane = kPmMaxInterp * kPmMaxInterp * 4 / 32;

__global__ void __launch_bounds__(32 * kPmSpreadWarps)
    k_pm_spread(const double2* __restrict__ pos, const uint32_t* __restrict__ perm,
                const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bend,
                const double* __restrict__ wx, const double* __restrict__ wy, PmGrid g, double* __restrict__ fin)
{
    __shared__ double s_q[kPmSpreadWarps][32][4];
    __shared__ double s_wx[kPmSpreadWarps][32][kPmMaxInterp];
    __shared__ double s_wy[kPmSpreadWarps][32][kPmMaxInterp];
    const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
    const int64_t nbox = (int64_t)g.nb * g.nb;
    const int nacc = g.p * g.p * 4;
    const size_t plane = (size_t)g.nf * g.nf;
    const int64_t wstride = (int64_t)gridDim.x * kPmSpreadWarps;
    for (int64_t box = blockIdx.x * (int64_t)kPmSpreadWarps + wv; box < nbox; box += wstride) {
        const uint32_t k0 = bstart[box], k1 = bend[box];
        if (k1 <= k0) continue;
        const int bx = (int)(box % g.nb), by = (int)(box / g.nb);
        double acc[kPmAccPerLane];
#pragma unroll
        for (int t = 0; t < kPmAccPerLane; t++) acc[t] = 0.0;
        for (uint32_t c0 = k0; c0 < k1; c0 += 32) {
            const uint32_t m = min(32u, k1 - c0);
            if ((uint32_t)lane < m) {
                const uint32_t i = perm[c0 + lane];
                const double2 q = pos[i];
                s_q[wv][lane][0] = 1.0;
                s_q[wv][lane][1] = q.x;
                s_q[wv][lane][2] = q.y;
                s_q[wv][lane][3] = q.x * q.x + q.y * q.y;
                for (int a = 0; a < g.p; a++) {
                    s_wx[wv][lane][a] = wx[(size_t)i * g.p + a];
                    s_wy[wv][lane][a] = wy[(size_t)i * g.p + a];
                }
            }
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kPmAccPerLane; t++) {
                const int u = lane + 32 * t;
                if (u < nacc) {
                    const int d = u & 3, ab = u >> 2, a = ab / g.p, b = ab % g.p;
                    double s = acc[t];
                    for (uint32_t j = 0; j < m; j++) s += s_wy[wv][j][b] * s_wx[wv][j][a] * s_q[wv][j][d];
                    acc[t] = s;
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int t = 0; t < kPmAccPerLane; t++) {
            const int u = lane + 32 * t;
            if (u < nacc) {
                const int d = u & 3, ab = u >> 2, a = ab / g.p, b = ab % g.p;
                fin[d * plane + (size_t)(bx * g.p + a) * g.nf + (size_t)(by * g.p + b)] = acc[t];
            }
        }
    }
}

// (1 + r^2)^-2 between node 0 and node (i, j), mirrored into the circulant
// generator exactly as precompute_2d places it
__global__ void k_pm_kernel_tilde(const double* __restrict__ xt, int n1, int nf, double* __restrict__ kt)
{
    const int64_t total = (int64_t)n1 * n1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / n1), j = (int)(t % n1);
        const double dy = xt[0] - xt[i], dx = xt[0] - xt[j];
        const double u = 1.0 + dy * dy + dx * dx;
        const double v = 1.0 / (u * u);
        kt[(size_t)(n1 + i) * nf + (n1 + j)] = v;
        kt[(size_t)(n1 - i) * nf + (n1 + j)] = v;
        kt[(size_t)(n1 + i) * nf + (n1 - j)] = v;
        kt[(size_t)(n1 - i) * nf + (n1 - j)] = v;
    }
}

// the Hadamard product of every charge's spectrum with the kernel's
__global__ void k_pm_multiply(cufftDoubleComplex* __restrict__ fw, const cufftDoubleComplex* __restrict__ kf,
                              int64_t nspec, int nbatch)
{
    const int64_t total = nspec * nbatch;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const cufftDoubleComplex w = fw[t], k = kf[t % nspec];
        fw[t] = make_cuDoubleComplex(w.x * k.x - w.y * k.y, w.x * k.y + w.y * k.x);
    }
}

// potentials at every point (input order): gradient and the point's Z term
__global__ void k_pm_gather(const double2* __restrict__ pos, int64_t n, const uint32_t* __restrict__ key,
                            const double* __restrict__ wx, const double* __restrict__ wy,
                            const double* __restrict__ fout, PmGrid g, double* __restrict__ grad,
                            double* __restrict__ zterm)
{
    const size_t plane = (size_t)g.nf * g.nf;
    const double norm = (double)((int64_t)g.nf * g.nf);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t b = key[i];
        const int bx = (int)(b % (uint32_t)g.nb), by = (int)(b / (uint32_t)g.nb);
        double phi[4] = {0.0, 0.0, 0.0, 0.0};
        for (int a = 0; a < g.p; a++)
            for (int c = 0; c < g.p; c++) {
                const size_t node = (size_t)(g.n1 + bx * g.p + a) * g.nf + (size_t)(g.n1 + by * g.p + c);
                const double w = wx[(size_t)i * g.p + a] * wy[(size_t)i * g.p + c];
#pragma unroll
                for (int d = 0; d < 4; d++) phi[d] += w * (fout[d * plane + node] / norm);
            }
        const double2 q = pos[i];
        grad[2 * i] = q.x * phi[0] - phi[1];
        grad[2 * i + 1] = q.y * phi[0] - phi[2];
        zterm[i] = (1 + q.x * q.x + q.y * q.y) * phi[0] - 2 * (q.x * phi[1] + q.y * phi[2]) + phi[3];
    }
}

__global__ void k_pm_total(double* __restrict__ total, double n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *total = *total - n;
}

// ------------------------------------------------------------------ per-device workspace
struct PmWork {
    std::mutex mu;
    Buf vals_max, vals_min, mm, key, skey, perm, alt_k, alt_v, sort_tmp, wx, wy, bstart, bend, xt, kt, kf, fin, fw,
        fout, zterm, sumtmp, host_pos, host_out;
    std::map<int, cufftHandle> d2z1, d2z4, z2d4;  // plans by FFT size
    cudaEvent_t done = nullptr;
    bool recorded = false;
};

PmWork& pm_work(int dev)
{
    static std::mutex m;
    static std::map<int, std::unique_ptr<PmWork>> w;
    std::lock_guard<std::mutex> g(m);
    auto& p = w[dev];
    if (!p) p.reset(new PmWork());
    return *p;
}

struct PmRelease {
    PmWork& w;
    cudaStream_t s;
    ~PmRelease()
    {
        if (w.done && cudaEventRecord(w.done, s) == cudaSuccess) w.recorded = true;
    }
};

int smooth_size(int n)
{
    for (int m = n;; m++) {
        int r = m;
        for (int f : {2, 3, 5, 7})
            while (r % f == 0) r /= f;
        if (r == 1) return m;
    }
}

int pm_plan(CufftApi& api, std::map<int, cufftHandle>& cache, int nf, cufftType type, int batch, cufftHandle* out)
{
    auto it = cache.find(nf);
    if (it != cache.end()) {
        *out = it->second;
        return TC_OK;
    }
    cufftHandle h = 0;
    int dims[2] = {nf, nf};
    const cufftResult r = api.plan_many(&h, 2, dims, nullptr, 1, 0, nullptr, 1, 0, type, batch);
    if (r != CUFFT_SUCCESS) {
        tc_set_error("particle mesh: cufftPlanMany failed (%d) for %d x %d", (int)r, nf, nf);
        return TC_ERR_CUDA;
    }
    cache[nf] = h;
    *out = h;
    return TC_OK;
}

}  // namespace

int pm_solve_device(int n_interp, double cell_size, int min_intervals, const double* d_pos, int64_t n, double* d_grad,
                    double* d_total, cudaStream_t s)
{
    if (n <= 0 || n > (int64_t)UINT32_MAX / 2 || !d_pos || !d_grad || !d_total || n_interp < 1 ||
        n_interp > kPmMaxInterp || !(cell_size > 0.0) || min_intervals < 1) {
        tc_set_error("particle mesh: invalid arguments (1 <= n_interp <= %d, cell_size > 0, min_intervals >= 1)",
                     kPmMaxInterp);
        return TC_ERR_INVALID;
    }
    CufftApi& api = cufft();
    if (!api.ok) {
        tc_set_error("particle mesh: libcufft could not be loaded");
        return TC_ERR_CUDA;
    }
    int dev = 0;
    TC_CUDA_TRY(cudaGetDevice(&dev));
    PmWork& w = pm_work(dev);
    std::lock_guard<std::mutex> lock(w.mu);
    if (!w.done) TC_CUDA_TRY(cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming));
    if (w.recorded) TC_CUDA_TRY(cudaStreamWaitEvent(s, w.done, 0));
    PmRelease release_on_exit{w, s};
    int rc;
    // 1. min / max over the interleaved coordinates
    const int64_t m = 2 * n, nc = (m + kPmChunk - 1) / kPmChunk;
    if ((rc = ensure(w.vals_max, nc * 16 + 64)) || (rc = ensure(w.vals_min, nc * 8 + 64)) ||
        (rc = ensure(w.mm, 64)) || (rc = ensure(w.host_out, 64)))
        return rc;
    double* cmax = P<double>(w.vals_max);  // [0, nc): prefix maxima, [nc, 2nc): raw chunk maxima
    k_pm_chunk_max<<<(unsigned)nc, kPmThreads, 0, s>>>(d_pos, m, cmax + nc);
    TC_CUDA_TRY(cudaMemcpyAsync(cmax, cmax + nc, nc * 8, cudaMemcpyDeviceToDevice, s));
    k_pm_chunk_premax<<<1, kPmScanThreads, 0, s>>>(cmax, nc);
    k_pm_chunk_min<<<(unsigned)nc, kPmThreads, 0, s>>>(d_pos, m, cmax, P<double>(w.vals_min));
    k_pm_minmax_final<<<1, kPmScanThreads, 0, s>>>(P<double>(w.vals_min), cmax + nc, nc, P<double>(w.mm));
    double mm[2];
    TC_CUDA_TRY(cudaMemcpyAsync(mm, w.mm.p, 16, cudaMemcpyDeviceToHost, s));
    TC_CUDA_TRY(cudaStreamSynchronize(s));
    // 2. the grid, on the host in the reference's arithmetic
    PmGrid g{};
    g.p = n_interp;
    g.mn = mm[0];
    const double span = mm[1] - mm[0];
    if (!std::isfinite(span) || !(span >= 0.0)) {
        tc_set_error("particle mesh: non-finite coordinates (min %g, max %g)", mm[0], mm[1]);
        return TC_ERR_INVALID;
    }
    const double nbd = span / cell_size;
    if (nbd > 8192.0) {
        tc_set_error("particle mesh: %g boxes per dimension (extent %g / cell size %g) exceed 8192", nbd, span,
                     cell_size);
        return TC_ERR_INVALID;
    }
    g.nb = (int)nbd;
    if (g.nb < min_intervals) g.nb = min_intervals;
    g.bw = span / (double)g.nb;
    const double hs = 1.0 / (double)g.p;
    g.sp[0] = hs / 2;
    for (int i = 1; i < g.p; i++) g.sp[i] = g.sp[i - 1] + hs;
    for (int i = 0; i < g.p; i++) {
        g.den[i] = 1.0;
        for (int j = 0; j < g.p; j++)
            if (i != j) g.den[i] *= g.sp[i] - g.sp[j];
    }
    g.n1 = g.p * g.nb;
    // any transform size >= 2 n1 holds the same linear convolution on the extracted
    // [n1, 2 n1) block (the kernel generator is laid out around n1 either way); the
    // smallest size >= 2 n1 with factors 2, 3, 5, 7 avoids slow prime-length FFTs
    g.nf = smooth_size(2 * g.n1);
    const size_t plane = (size_t)g.nf * g.nf, nspec = (size_t)g.nf * (g.nf / 2 + 1);
    if (plane * 8 * 10 > ((size_t)48 << 30)) {
        tc_set_error("particle mesh: FFT grid %d x %d too large", g.nf, g.nf);
        return TC_ERR_INVALID;
    }
    std::vector<double> xt(g.n1);
    const double hw = hs * g.bw;
    xt[0] = g.mn + hw / 2;
    for (int i = 1; i < g.n1; i++) xt[i] = xt[i - 1] + hw;
    const int64_t nbox = (int64_t)g.nb * g.nb;
    if ((rc = ensure(w.key, n * 4)) || (rc = ensure(w.skey, n * 4)) || (rc = ensure(w.perm, n * 4)) ||
        (rc = ensure(w.alt_k, n * 4)) || (rc = ensure(w.alt_v, n * 4)) ||
        (rc = ensure(w.sort_tmp, radix_tmp_words(n) * 4)) || (rc = ensure(w.wx, n * g.p * 8)) ||
        (rc = ensure(w.wy, n * g.p * 8)) || (rc = ensure(w.bstart, nbox * 4)) || (rc = ensure(w.bend, nbox * 4)) ||
        (rc = ensure(w.xt, g.n1 * 8)) || (rc = ensure(w.kt, plane * 8)) || (rc = ensure(w.kf, nspec * 16)) ||
        (rc = ensure(w.fin, 4 * plane * 8)) || (rc = ensure(w.fw, 4 * nspec * 16)) ||
        (rc = ensure(w.fout, 4 * plane * 8)) || (rc = ensure(w.zterm, n * 8)) ||
        (rc = ensure(w.sumtmp, sum_tmp_doubles() * 8)))
        return rc;
    TC_CUDA_TRY(cudaMemcpyAsync(w.xt.p, xt.data(), g.n1 * 8, cudaMemcpyHostToDevice, s));
    // 3. points: boxes and weights; sort by box; spread the charges
    const double2* pos2 = (const double2*)d_pos;
    k_pm_points<<<grid_for(n, 256), 256, 0, s>>>(pos2, n, g, P<uint32_t>(w.key), P<double>(w.wx), P<double>(w.wy));
    TC_CUDA_TRY(cudaMemcpyAsync(w.skey.p, w.key.p, n * 4, cudaMemcpyDeviceToDevice, s));
    int launches = 0;
    if ((rc = radix_sort_u32(P<uint32_t>(w.skey), P<uint32_t>(w.perm), P<uint32_t>(w.alt_k), P<uint32_t>(w.alt_v), n,
                             P<uint32_t>(w.sort_tmp), s, &launches)))
        return rc;
    TC_CUDA_TRY(cudaMemsetAsync(w.bstart.p, 0, nbox * 4, s));
    TC_CUDA_TRY(cudaMemsetAsync(w.bend.p, 0, nbox * 4, s));
    k_pm_box_ranges<<<grid_for(n, 256), 256, 0, s>>>(P<uint32_t>(w.skey), n, P<uint32_t>(w.bstart),
                                                    P<uint32_t>(w.bend));
    TC_CUDA_TRY(cudaMemsetAsync(w.fin.p, 0, 4 * plane * 8, s));
    k_pm_spread<<<grid_for(nbox, kPmSpreadWarps), 32 * kPmSpreadWarps, 0, s>>>(pos2, P<uint32_t>(w.perm), P<uint32_t>(w.bstart),
                                                        P<uint32_t>(w.bend), P<double>(w.wx), P<double>(w.wy), g,
                                                        P<double>(w.fin));
    // 4. the kernel's spectrum and the four convolutions
    TC_CUDA_TRY(cudaMemsetAsync(w.kt.p, 0, plane * 8, s));
    k_pm_kernel_tilde<<<grid_for((int64_t)g.n1 * g.n1, 256), 256, 0, s>>>(P<double>(w.xt), g.n1, g.nf,
                                                                         P<double>(w.kt));
    cufftHandle p1, p4, q4;
    if ((rc = pm_plan(api, w.d2z1, g.nf, CUFFT_D2Z, 1, &p1)) || (rc = pm_plan(api, w.d2z4, g.nf, CUFFT_D2Z, 4, &p4)) ||
        (rc = pm_plan(api, w.z2d4, g.nf, CUFFT_Z2D, 4, &q4)))
        return rc;
    if (api.set_stream(p1, s) != CUFFT_SUCCESS || api.set_stream(p4, s) != CUFFT_SUCCESS ||
        api.set_stream(q4, s) != CUFFT_SUCCESS ||
        api.exec_d2z(p1, P<cufftDoubleReal>(w.kt), P<cufftDoubleComplex>(w.kf)) != CUFFT_SUCCESS ||
        api.exec_d2z(p4, P<cufftDoubleReal>(w.fin), P<cufftDoubleComplex>(w.fw)) != CUFFT_SUCCESS) {
        tc_set_error("particle mesh: forward FFT failed");
        return TC_ERR_CUDA;
    }
    k_pm_multiply<<<grid_for((int64_t)nspec * 4, 256), 256, 0, s>>>(P<cufftDoubleComplex>(w.fw),
                                                                    P<cufftDoubleComplex>(w.kf), (int64_t)nspec, 4);
    if (api.exec_z2d(q4, P<cufftDoubleComplex>(w.fw), P<cufftDoubleReal>(w.fout)) != CUFFT_SUCCESS) {
        tc_set_error("particle mesh: inverse FFT failed");
        return TC_ERR_CUDA;
    }
    // 5. potentials, gradient, Z
    k_pm_gather<<<grid_for(n, 256), 256, 0, s>>>(pos2, n, P<uint32_t>(w.key), P<double>(w.wx), P<double>(w.wy),
                                                P<double>(w.fout), g, d_grad, P<double>(w.zterm));
    if ((rc = sum_f64(P<double>(w.zterm), n, nullptr, nullptr, d_total, 0, P<double>(w.sumtmp), s))) return rc;
    k_pm_total<<<1, 32, 0, s>>>(d_total, (double)n);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace tc

extern "C" int tc_pm_solve_device(int n_interp, double cell_size, int min_intervals, const double* d_pos_xy,
                                  int64_t n, double* d_grad_xy, double* d_total, void* stream)
{
    return tc::pm_solve_device(n_interp, cell_size, min_intervals, d_pos_xy, n, d_grad_xy, d_total,
                               (cudaStream_t)stream);
}

extern "C" int tc_pm_solve(int n_interp, double cell_size, int min_intervals, const double* pos_xy, int64_t n,
                           double* grad_xy, double* total)
{
    using namespace tc;
    if (!pos_xy || !grad_xy || !total || n <= 0) {
        tc_set_error("tc_pm_solve: invalid arguments");
        return TC_ERR_INVALID;
    }
    double *dp = nullptr, *dg = nullptr, *dt = nullptr;
    cudaStream_t s = nullptr;
    int rc = TC_OK;
    auto fail = [&](cudaError_t e, const char* what) { rc = tc_cuda_fail(e, what); };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return tc_cuda_fail(e, "stream");
    if ((e = cudaMallocAsync((void**)&dp, n * 16, s)) != cudaSuccess || (e = cudaMallocAsync((void**)&dg, n * 16, s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&dt, 8, s)) != cudaSuccess)
        fail(e, "cudaMallocAsync");
    if (rc == TC_OK && (e = cudaMemcpyAsync(dp, pos_xy, n * 16, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        fail(e, "H2D");
    if (rc == TC_OK) rc = pm_solve_device(n_interp, cell_size, min_intervals, dp, n, dg, dt, s);
    if (rc == TC_OK && (e = cudaMemcpyAsync(grad_xy, dg, n * 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        fail(e, "D2H");
    if (rc == TC_OK && (e = cudaMemcpyAsync(total, dt, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) fail(e, "D2H");
    if (dp) cudaFreeAsync(dp, s);
    if (dg) cudaFreeAsync(dg, s);
    if (dt) cudaFreeAsync(dt, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc == TC_OK && se != cudaSuccess) rc = tc_cuda_fail(se, "cudaStreamSynchronize");
    return rc;
}
