// The t-SNE affinity matrix P on the GPU: exact k nearest neighbours, the
// per-point Gaussian bandwidth calibrated to a perplexity, and the symmetric
// CSR matrix (P + P^T) / (2N).
//
// The reference builds P offline with openTSNE (MnistLoader.ipynb cell 14:
// PerplexityBasedNN with k = 3 * perplexity, symmetrize=True, written with
// mmwrite) and reads it into CSR in TSNE::setupEfficientPmatrix
// (src/nBodyInstances/tsne.h:462-520: rows sorted, columns sorted within a
// row).  openTSNE is not available, so this file restates the published
// algorithm; every operation is defined so that the CPU restatement in the
// oracle (orc_knn, orc_perplexity, orc_symmetrize) gives the same bits:
// * distances: d_ij = sum_t (x_it - x_jt)^2 in FP32, t = 0..dim-1 in order,
//   each step one fused multiply-add; neighbours ordered by (d, j), self
//   excluded;
// * bandwidths: per row a bisection on beta (start 1, doubling until
//   bracketed) of H = log(s) + beta * sum_j d'_j w_j / s with
//   w_j = exp(-beta d'_j), d'_j = d_j - d_min, s = sum_j w_j (FP64, j in
//   order), stopping when |H - log(perplexity)| < tol; p_j = w_j / s;
// * exp and log in FP64 written here from the mathematics (a two-constant
//   reduction by ln 2 with a degree-13 Taylor polynomial; the atanh series of
//   log m on [sqrt(1/2), sqrt(2))), so no vendor math routine is involved;
// * symmetrisation: each stored p_ij contributes p_ij / (2N) to (i, j) and to
//   (j, i); the (at most two) contributions to an entry are added.
// This file is compiled without FMA contraction: the fused operations above
// are the explicit fma / fmaf calls.
#include "common.cuh"

namespace tc {
namespace {

// ------------------------------------------------------------------ exp, log
constexpr double kLn2Hi = 0x1.62e42fee00000p-1;   // ln 2 to 32 significant bits
constexpr double kLn2Lo = 0x1.a39ef35793c76p-33;  // ln 2 - kLn2Hi
constexpr double kInvLn2 = 0x1.71547652b82fep+0;
constexpr double kSqrt2 = 1.4142135623730951;

__device__ inline double scale2(double v, int k)
{
    // v * 2^k for k >= -1100 (exact until the result is subnormal)
    if (k < -1000) {
        v *= 0x1p-600;
        k += 600;
    }
    return v * __longlong_as_double((long long)(k + 1023) << 52);
}

__device__ inline double aff_exp(double x)
{
    if (!(x > -745.0)) return 0.0;  // below the smallest subnormal (and NaN)
    if (x > 709.0) return INFINITY;
    const double kf = floor(x * kInvLn2 + 0.5);
    const int k = (int)kf;
    double r = fma(-kf, kLn2Hi, x);
    r = fma(-kf, kLn2Lo, r);
    // e^r = sum_n r^n / n!, n <= 13, |r| <= ln(2) / 2
    double q = 0x1.6124613a86d09p-33;
    q = fma(q, r, 0x1.1eed8eff8d898p-29);
    q = fma(q, r, 0x1.ae64567f544e4p-26);
    q = fma(q, r, 0x1.27e4fb7789f5cp-22);
    q = fma(q, r, 0x1.71de3a556c734p-19);
    q = fma(q, r, 0x1.a01a01a01a01ap-16);
    q = fma(q, r, 0x1.a01a01a01a01ap-13);
    q = fma(q, r, 0x1.6c16c16c16c17p-10);
    q = fma(q, r, 0x1.1111111111111p-7);
    q = fma(q, r, 0x1.5555555555555p-5);
    q = fma(q, r, 0x1.5555555555555p-3);
    q = fma(q, r, 0.5);
    q = fma(q, r, 1.0);
    q = fma(q, r, 1.0);
    return scale2(q, k);
}

// natural log of a positive normal double
__device__ inline double aff_log(double x)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int e = (int)((b >> 52) & 0x7FF) - 1023;
    b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    double m = __longlong_as_double((long long)b);  // x = m 2^e, m in [1, 2)
    if (m > kSqrt2) {
        m *= 0.5;
        e += 1;
    }
    // log m = 2 atanh(z), z = (m - 1) / (m + 1), |z| <= 0.1716
    const double z = (m - 1.0) / (m + 1.0);
    const double z2 = z * z;
    double q = 0.037037037037037035;  // 1/27
    q = fma(q, z2, 0.04);
    q = fma(q, z2, 0.043478260869565216);
    q = fma(q, z2, 0.047619047619047616);
    q = fma(q, z2, 0.05263157894736842);
    q = fma(q, z2, 0.058823529411764705);
    q = fma(q, z2, 0.06666666666666667);
    q = fma(q, z2, 0.07692307692307693);
    q = fma(q, z2, 0.09090909090909091);
    q = fma(q, z2, 0.1111111111111111);
    q = fma(q, z2, 0.14285714285714285);
    q = fma(q, z2, 0.2);
    q = fma(q, z2, 0.3333333333333333);
    const double lm = 2.0 * fma(z * z2, q, z);
    const double ed = (double)e;
    return fma(ed, kLn2Hi, fma(ed, kLn2Lo, lm));
}

// ------------------------------------------------------------------ kNN
// A block takes kQ query rows and walks every candidate tile of kQ points:
// each thread accumulates a 4 x 4 block of squared distances over the
// dimensions in order (one fmaf per dimension, as the definition), the tile's
// distances go to shared memory, and each warp folds its rows' candidates into
// their sorted top-k lists (kept in shared memory, ordered by (d, j)).
constexpr int kQ = 64;        // query rows and candidates per tile
constexpr int kDC = 32;       // dimensions per staged chunk
constexpr int kKnnT = 256;    // threads
constexpr int kMaxK = 128;    // longest neighbour list

__device__ __forceinline__ bool before(float da, int ja, float db, int jb)
{
    return da < db || (da == db && ja < jb);
}

__global__ void __launch_bounds__(kKnnT) k_knn(const float* __restrict__ x, int64_t n, int dim, int k,
                                               float* __restrict__ out_d, int32_t* __restrict__ out_i)
{
    __shared__ float sq[kDC][kQ + 1];
    __shared__ float sc[kDC][kQ + 1];
    __shared__ float tile[kQ][kQ + 1];
    extern __shared__ uint8_t dyn[];
    float* ld = reinterpret_cast<float*>(dyn);                   // [kQ][k] distances
    int32_t* li = reinterpret_cast<int32_t*>(ld + kQ * k);      // [kQ][k] indices
    __shared__ int lcount[kQ];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t q0 = (int64_t)blockIdx.x * kQ;
    const int tr = (tid / 16) * 4, tc = (tid % 16) * 4;  // this thread's 4 x 4 block
    if (tid < kQ) lcount[tid] = 0;
    for (int64_t c0 = 0; c0 < n; c0 += kQ) {
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] = 0.f;
        for (int t0 = 0; t0 < dim; t0 += kDC) {
            __syncthreads();
            for (int e = tid; e < kQ * kDC; e += kKnnT) {
                const int r = e / kDC, t = e % kDC;
                const int64_t qi = q0 + r, ci = c0 + r;
                sq[t][r] = (qi < n && t0 + t < dim) ? x[qi * dim + t0 + t] : 0.f;
                sc[t][r] = (ci < n && t0 + t < dim) ? x[ci * dim + t0 + t] : 0.f;
            }
            __syncthreads();
            const int tn = dim - t0 < kDC ? dim - t0 : kDC;
            for (int t = 0; t < tn; t++) {
                float qv[4], cv[4];
#pragma unroll
                for (int a = 0; a < 4; a++) qv[a] = sq[t][tr + a];
#pragma unroll
                for (int b = 0; b < 4; b++) cv[b] = sc[t][tc + b];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const float df = qv[a] - cv[b];
                        acc[a][b] = fmaf(df, df, acc[a][b]);
                    }
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) tile[tr + a][tc + b] = acc[a][b];
        __syncthreads();
        // fold the tile into the lists: warp w owns rows w, w + 8, ...
        for (int r = warp; r < kQ; r += kKnnT / 32) {
            const int64_t qi = q0 + r;
            if (qi >= n) break;
            float* rd = ld + r * k;
            int32_t* ri = li + r * k;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int cc = lane + 32 * h;
                const int64_t cj = c0 + cc;
                const float d = tile[r][cc];
                int cnt = lcount[r];
                bool want = cj < n && cj != qi && (cnt < k || before(d, (int)cj, rd[k - 1], ri[k - 1]));
                uint32_t m = __ballot_sync(0xffffffffu, want);
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1u;
                    const float dv = __shfl_sync(0xffffffffu, d, src);
                    const int jv = (int)(c0 + src + 32 * h);
                    cnt = lcount[r];
                    if (cnt == k && !before(dv, jv, rd[k - 1], ri[k - 1])) continue;
                    // position: entries before (dv, jv)
                    int pos = 0;
                    for (int e = lane; e < cnt; e += 32) pos += before(rd[e], ri[e], dv, jv) ? 1 : 0;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) pos += __shfl_xor_sync(0xffffffffu, pos, o);
                    const int last = cnt < k ? cnt : k - 1;  // shift [pos, last) up by one
                    float sd[kMaxK / 32];
                    int si[kMaxK / 32];
#pragma unroll
                    for (int u = 0; u < kMaxK / 32; u++) {
                        const int e = lane + 32 * u;
                        sd[u] = (e > pos && e <= last) ? rd[e - 1] : 0.f;
                        si[u] = (e > pos && e <= last) ? ri[e - 1] : 0;
                    }
                    __syncwarp();
#pragma unroll
                    for (int u = 0; u < kMaxK / 32; u++) {
                        const int e = lane + 32 * u;
                        if (e > pos && e <= last) {
                            rd[e] = sd[u];
                            ri[e] = si[u];
                        }
                    }
                    if (lane == 0) {
                        rd[pos] = dv;
                        ri[pos] = jv;
                        if (cnt < k) lcount[r] = cnt + 1;
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < kQ * k; e += kKnnT) {
        const int r = e / k, c = e % k;
        const int64_t qi = q0 + r;
        if (qi < n) {
            out_d[qi * k + c] = ld[e];
            out_i[qi * k + c] = li[e];
        }
    }
}

// ------------------------------------------------------------------ bandwidths
__global__ void k_perplexity(const float* __restrict__ dist, int64_t n, int k, double perplexity, int max_iter,
                             double tol, double* __restrict__ p)
{
    const double log_perp = aff_log(perplexity);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* d = dist + i * k;
        const double dmin = (double)d[0];
        double beta = 1.0, lo = 0.0, hi = INFINITY;
        for (int it = 0; it < max_iter; it++) {
            double s = 0.0, sd = 0.0;
            for (int j = 0; j < k; j++) {
                const double dj = (double)d[j] - dmin;
                const double w = aff_exp(-dj * beta);
                s += w;
                sd = fma(dj, w, sd);
            }
            const double h = aff_log(s) + beta * sd / s;
            const double diff = h - log_perp;
            if (fabs(diff) < tol) break;
            if (diff > 0.0) {
                lo = beta;
                beta = isinf(hi) ? beta * 2.0 : (lo + hi) * 0.5;
            } else {
                hi = beta;
                beta = (lo + hi) * 0.5;
            }
        }
        double s = 0.0;
        for (int j = 0; j < k; j++) s += aff_exp(-((double)d[j] - dmin) * beta);
        for (int j = 0; j < k; j++) p[i * k + j] = aff_exp(-((double)d[j] - dmin) * beta) / s;
    }
}

// ------------------------------------------------------------------ symmetrisation
// entry e < nk: (i, j) with value p_ij / (2N); entry nk + e: its transpose (j, i)
__global__ void k_sym_entries(const int32_t* __restrict__ idx, const double* __restrict__ p, int64_t n, int k,
                              double c, uint32_t* __restrict__ col_key, uint32_t* __restrict__ row,
                              double* __restrict__ v)
{
    const int64_t nk = n * k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(e / k), j = (uint32_t)idx[e];
        const double w = p[e] * c;
        col_key[e] = j;
        row[e] = i;
        v[e] = w;
        col_key[nk + e] = i;
        row[nk + e] = j;
        v[nk + e] = w;
    }
}

__global__ void k_gather_u32(const uint32_t* __restrict__ in, const uint32_t* __restrict__ perm, int64_t m,
                             uint32_t* __restrict__ out)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = in[perm[e]];
}

// sorted position q holds entry ord[q] = perm1[perm2[q]] (rows sorted, columns
// within a row); flag the first entry of each (row, col)
__global__ void k_sym_flags(const uint32_t* __restrict__ perm1, const uint32_t* __restrict__ perm2, int64_t m,
                            const uint32_t* __restrict__ row, const uint32_t* __restrict__ col_key,
                            uint32_t* __restrict__ ord, uint32_t* __restrict__ flag)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t e = perm1[perm2[q]];
        ord[q] = e;
        bool first = q == 0;
        if (!first) {
            const uint32_t f = perm1[perm2[q - 1]];
            first = row[f] != row[e] || col_key[f] != col_key[e];
        }
        flag[q] = first ? 1u : 0u;
    }
}

// pos: exclusive scan of the flags (pos[m] = the number of distinct entries)
__global__ void k_sym_write(const uint32_t* __restrict__ ord, const uint32_t* __restrict__ flag,
                            const uint32_t* __restrict__ pos, int64_t m, int64_t n, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col_key, const double* __restrict__ v,
                            uint32_t* __restrict__ row_ptr, uint32_t* __restrict__ col, double* __restrict__ val)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[q]) continue;
        const uint32_t e = ord[q], u = pos[q];
        double s = v[e];
        if (q + 1 < m && !flag[q + 1]) s = s + v[ord[q + 1]];  // the transposed contribution to the same entry
        col[u] = col_key[e];
        val[u] = s;
        if (q == 0 || row[ord[q - 1]] != row[e]) row_ptr[row[e]] = u;
        if (u + 1 == pos[m]) row_ptr[n] = pos[m];
    }
}

}  // namespace
}  // namespace tc

using namespace tc;

extern "C" int tc_knn_device(const float* d_x, int64_t n, int dim, int k, float* d_dist, int32_t* d_idx, void* stream)
{
    if (!d_x || !d_dist || !d_idx || n < 2 || dim < 1 || k < 1 || k > kMaxK || k >= n || n > 0x7FFFFFFF) {
        tc_set_error("tc_knn_device: invalid arguments (need 1 <= k <= %d, k < n)", kMaxK);
        return TC_ERR_INVALID;
    }
    const size_t dyn = (size_t)kQ * k * 8;
    TC_CUDA_TRY(cudaFuncSetAttribute(k_knn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    k_knn<<<(unsigned)((n + kQ - 1) / kQ), kKnnT, dyn, (cudaStream_t)stream>>>(d_x, n, dim, k, d_dist, d_idx);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

extern "C" int tc_perplexity_device(const float* d_dist, int64_t n, int k, double perplexity, int max_iter, double tol,
                                    double* d_p, void* stream)
{
    if (!d_dist || !d_p || n < 1 || k < 1 || !(perplexity > 1.0) || max_iter < 1 || !(tol > 0.0)) {
        tc_set_error("tc_perplexity_device: invalid arguments (perplexity must exceed 1)");
        return TC_ERR_INVALID;
    }
    k_perplexity<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(d_dist, n, k, perplexity, max_iter, tol, d_p);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

extern "C" int tc_symmetrize_device(const int32_t* d_idx, const double* d_p, int64_t n, int k, uint32_t* d_row_ptr,
                                    uint32_t* d_col, double* d_val, int64_t* nnz, void* stream)
{
    const int64_t m = 2 * n * (int64_t)k;
    if (!d_idx || !d_p || !d_row_ptr || !d_col || !d_val || !nnz || n < 2 || k < 1 || m >= 0xFFFFFFFFll) {
        tc_set_error("tc_symmetrize_device: invalid arguments");
        return TC_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t tw = radix_tmp_words(m) > scan_tmp_words(m) ? radix_tmp_words(m) : scan_tmp_words(m);
    // scratch (32-bit words): values (2m); column keys, rows, the two sorts' keys and permutations, their
    // alternates and the sorted order (9 arrays of m); flags (m); positions (m + 1); sort/scan temporaries
    const size_t words = (size_t)m * 2 + (size_t)m * 9 + (size_t)m + (size_t)(m + 1) + (size_t)tw;
    void* buf = nullptr;
    TC_CUDA_TRY(cudaMallocAsync(&buf, words * 4 + 64, s));
    uint32_t* w = static_cast<uint32_t*>(buf);
    double* v = reinterpret_cast<double*>(w);
    uint32_t* colk = w + 2 * m;
    uint32_t* row = colk + m;
    uint32_t* k1 = row + m;
    uint32_t* p1 = k1 + m;
    uint32_t* k2 = p1 + m;
    uint32_t* p2 = k2 + m;
    uint32_t* ak = p2 + m;
    uint32_t* av = ak + m;
    uint32_t* ord = av + m;
    uint32_t* flag = ord + m;
    uint32_t* pos = flag + m;
    uint32_t* tmp = pos + (m + 1);  // ends at w + words
    int rc = TC_OK;
    const double c = 1.0 / (2.0 * (double)n);
    k_sym_entries<<<grid_for(n * k, 256), 256, 0, s>>>(d_idx, d_p, n, k, c, colk, row, v);
    // stable sort by column, then stable by row: rows sorted, columns sorted within a row
    cudaError_t e = cudaMemcpyAsync(k1, colk, (size_t)m * 4, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) rc = radix_sort_u32(k1, p1, ak, av, m, tmp, s, nullptr, 0);
    if (e == cudaSuccess && rc == TC_OK) {
        k_gather_u32<<<grid_for(m, 256), 256, 0, s>>>(row, p1, m, k2);
        rc = radix_sort_u32(k2, p2, ak, av, m, tmp, s, nullptr, 0);
    }
    if (e == cudaSuccess && rc == TC_OK) {
        k_sym_flags<<<grid_for(m, 256), 256, 0, s>>>(p1, p2, m, row, colk, ord, flag);
        rc = exclusive_scan_u32(flag, pos, m, tmp, s);
    }
    if (e == cudaSuccess && rc == TC_OK) {
        k_sym_write<<<grid_for(m, 256), 256, 0, s>>>(ord, flag, pos, m, n, row, colk, v, d_row_ptr, d_col, d_val);
        uint32_t cnt = 0;
        e = cudaMemcpyAsync(&cnt, pos + m, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        *nnz = cnt;
    }
    const cudaError_t ef = cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return tc_cuda_fail(e, "tc_symmetrize_device");
    if (rc) return rc;
    if (ef != cudaSuccess) return tc_cuda_fail(ef, "cudaFreeAsync");
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}
