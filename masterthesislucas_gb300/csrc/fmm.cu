// Force evaluation of the symmetric Morton FMM at the reference's fixed
// order: multipoles M0 + M2 about the centre of mass, local expansion C1, C2,
// C3 (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:622-836), evaluated
// sink by sink from the interaction lists built in lists.cu.
//
// The reference applies each symmetric kernel to both nodes of a pair; here
// each direction is evaluated by its own sink, so nothing is accumulated by
// atomics and results are deterministic:
//   k_m2l     one warp per node A: C(A) += M2L(B -> A) for B in nn(A)
//             (kernelNN, :622-723; the MA0 factor that applyForces later
//             divides out (:488-492) is never applied)
//   k_leaf    one warp per non-empty leaf S:
//             C_S = own C(S) + every ancestor's C shifted to com_S
//                   (applyForces' L2L chain, :482-519, composed per leaf)
//                 + P2L from points t of partners T < S with pass(t, S)
//                   (kernelPN second half, :764-814)
//             g_s = L2P(C_S) (:521-534)
//                 + self P2P over S (the j >= i loop of :176-192)
//                 + for T > S: M2P(T) if pass(s, T) else P2P over T
//                 + for T < S: P2P from the t in T with !pass(t, S)
// where pass(x, B) is the point-node MAC of traverse_SYM_PN (:272-313),
// |x - com_B|^2 > (L_B / theta)^2, evaluated in FP64 like the reference.  For
// a leaf pair the reference tests the points of the first node of the pair
// (the lower Morton index) against the second, which is what fixes the roles
// above.  Geometry is in cell-relative coordinates: offsets between cells are
// integer multiples of the cell size, so FP32 differences lose nothing to the
// absolute position magnitude.
#include "kernels.cuh"
#include "state.cuh"

namespace tc {
namespace {

// C1 of a source with mass m0 and normalised second moment T = M2/M0 (:638-655)
template <typename real>
__device__ inline void far_c1(real Rx, real Ry, real m0, real Txx, real Txy, real Tyy, real D1, real D2, real D3,
                              real& ox, real& oy)
{
    real S1 = Txx + Tyy;
    real S2 = Rx * Rx * Txx + real(2) * Rx * Ry * Txy + Ry * Ry * Tyy;
    real S3x = Rx * Txx + Ry * Txy;
    real S3y = Rx * Txy + Ry * Tyy;
    real base = D1 + real(0.5) * S1 * D2 + real(0.5) * S2 * D3;
    ox = m0 * (Rx * base + S3x * D2);
    oy = m0 * (Ry * base + S3y * D2);
}

// C2 and C3 of a monopole of mass m at offset R (:657-697)
template <typename real>
__device__ inline void add_c2c3(real Rx, real Ry, real m, real D1, real D2, real D3, real* C)
{
    C[L_C2XX] += m * (D1 + Rx * Rx * D2);
    C[L_C2XY] += m * (Rx * Ry * D2);
    C[L_C2YY] += m * (D1 + Ry * Ry * D2);
    C[L_C3XXX] += m * (real(3) * Rx * D2 + Rx * Rx * Rx * D3);
    C[L_C3XXY] += m * (Ry * D2 + Rx * Rx * Ry * D3);
    C[L_C3XYY] += m * (Rx * D2 + Rx * Ry * Ry * D3);
    C[L_C3YYY] += m * (real(3) * Ry * D2 + Ry * Ry * Ry * D3);
}

// evaluate C1 + d.C2 + 1/2 d.(d.C3) (the L2P / L2L C1 formula, :501-531)
template <typename real>
__device__ inline void eval_c1(const real* C, real dx, real dy, real& gx, real& gy)
{
    real txx = dx * C[L_C3XXX] + dy * C[L_C3XXY];
    real txy = dx * C[L_C3XXY] + dy * C[L_C3XYY];
    real tyy = dx * C[L_C3XYY] + dy * C[L_C3YYY];
    gx = C[L_C1X] + (dx * C[L_C2XX] + dy * C[L_C2XY]) + real(0.5) * (dx * txx + dy * txy);
    gy = C[L_C1Y] + (dx * C[L_C2XY] + dy * C[L_C2YY]) + real(0.5) * (dx * txy + dy * tyy);
}

// L2L shift of an expansion by d, added into acc (:497-516)
template <typename real>
__device__ inline void add_shifted(const real* C, real dx, real dy, real* acc)
{
    real gx, gy;
    eval_c1(C, dx, dy, gx, gy);
    acc[L_C1X] += gx;
    acc[L_C1Y] += gy;
    acc[L_C2XX] += C[L_C2XX] + dx * C[L_C3XXX] + dy * C[L_C3XXY];
    acc[L_C2XY] += C[L_C2XY] + dx * C[L_C3XXY] + dy * C[L_C3XYY];
    acc[L_C2YY] += C[L_C2YY] + dx * C[L_C3XYY] + dy * C[L_C3YYY];
    acc[L_C3XXX] += C[L_C3XXX];
    acc[L_C3XXY] += C[L_C3XXY];
    acc[L_C3XYY] += C[L_C3XYY];
    acc[L_C3YYY] += C[L_C3YYY];
}

struct Geo {
    int depth;
    double inv_theta;
    double theta;
    double h_leaf;     // leaf cell size
    int variant;       // 1: the non-symmetric FMM_MORTON leaf stage
};

template <typename real, typename K>
__global__ void __launch_bounds__(128) k_m2l(K ker, int l, real hl, const uint32_t* __restrict__ nn_ptr,
                                             const uint32_t* __restrict__ nn_idx, const real* __restrict__ comrel,
                                             const real* __restrict__ m0r, const real* __restrict__ m2t,
                                             real* __restrict__ loc, double* __restrict__ zpart)
{
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const int lane = threadIdx.x & 31;
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t a = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); a < nl; a += wstride) {
        const uint32_t b0 = nn_ptr[a], b1 = nn_ptr[a + 1];
        const int64_t na = li + a;
        if (b0 == b1) {
            if (lane < L_NCOEF) loc[na * L_NCOEF + lane] = real(0);
            if (lane == 0) zpart[na] = 0.0;
            continue;
        }
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const real cax = comrel[2 * na], cay = comrel[2 * na + 1];
        real C[L_NCOEF];
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = real(0);
        real z = real(0);
        for (uint32_t e = b0 + lane; e < b1; e += 32) {
            const uint32_t b = nn_idx[e];
            const int64_t nb = li + b;
            const int ibx = (int)compact16(b), iby = (int)compact16(b >> 1);
            const real Rx = real(iax - ibx) * hl + (cax - comrel[2 * nb]);
            const real Ry = real(iay - iby) * hl + (cay - comrel[2 * nb + 1]);
            real D1, D2, D3, t;
            ker.far(Rx * Rx + Ry * Ry, D1, D2, D3, t);
            const real mb = m0r[nb];
            real c1x, c1y;
            far_c1(Rx, Ry, mb, m2t[3 * nb], m2t[3 * nb + 1], m2t[3 * nb + 2], D1, D2, D3, c1x, c1y);
            C[L_C1X] += c1x;
            C[L_C1Y] += c1y;
            add_c2c3(Rx, Ry, mb, D1, D2, D3, C);
            z += mb * t;
        }
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = warp_sum(C[c]);
        double zz = warp_sum((double)z) * (double)m0r[na];
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < L_NCOEF; c++) loc[na * L_NCOEF + c] = C[c];
            zpart[na] = zz;
        }
    }
}

// point-node MAC of the non-symmetric solver's traverseBHMP
// (nBodySolverFMM_MORTON.h:201-204): L_B / |x - com_B| < theta
__device__ inline bool pn_pass_m(double2 x, double2 com, double len, double theta)
{
    double dx = x.x - com.x, dy = x.y - com.y;
    return len / sqrt(dx * dx + dy * dy) < theta;
}

// point-node MAC of traverse_SYM_PN, exactly as the reference evaluates it
__device__ inline bool pn_pass(double2 x, double2 com, double len, double inv_theta)
{
    double dx = x.x - com.x, dy = x.y - com.y;
    double dist = dx * dx + dy * dy;
    double thr = len * inv_theta;
    return dist > thr * thr;
}

constexpr int kLeafWarps = 4;

// phase A, one warp per non-empty leaf S: the final local expansion of S at
// com_S (own M2L + shifted ancestors + P2L from the passing points of
// partners T < S), and the number of 32-sink chunks of S
template <typename real, typename K>
__global__ void __launch_bounds__(32 * kLeafWarps)
    k_leaf_local(K ker, Geo geo, const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
                 const double2* __restrict__ com64, const double* __restrict__ bblen, const real* __restrict__ comrel,
                 const real* __restrict__ m0r, const real* __restrict__ loc, const uint32_t* __restrict__ near_ptr,
                 const uint32_t* __restrict__ near_idx, const double2* __restrict__ pos64,
                 const real* __restrict__ prel, real* __restrict__ locfin, double* __restrict__ zloc,
                 uint32_t* __restrict__ nchunk, unsigned long long* __restrict__ counters)
{
    uint32_t n_p2l = 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int dep = geo.depth;
    const uint32_t li = level_index(dep);
    const int64_t nl = (int64_t)1 << (2 * dep);
    const real h = (real)geo.h_leaf;
    const double inv_theta = geo.inv_theta;
    const int64_t wstride = (int64_t)gridDim.x * kLeafWarps;
    for (int64_t si = blockIdx.x * (int64_t)kLeafWarps + w; si < nl; si += wstride) {
        const int64_t S = li + si;
        const uint32_t cS = count[S];
        if (lane == 0) nchunk[si] = (cS + 31u) / 32u;
        if (cS == 0) {
            if (lane == 0) zloc[si] = 0.0;
            continue;
        }
        const int isx = (int)compact16((uint32_t)si), isy = (int)compact16((uint32_t)si >> 1);
        const double2 comS64 = com64[S];
        const double lenS = bblen[S];
        const real csx = comrel[2 * S], csy = comrel[2 * S + 1];
        const real mS = m0r[S];
        const uint32_t e0 = near_ptr[si], e1 = near_ptr[si + 1];
        real C[L_NCOEF];
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = real(0);
        real zA = real(0);
        if (lane <= dep) {
            // lane k shifts the expansion of the ancestor at level k (k == dep is S)
            const int k = lane;
            const uint32_t ai = (uint32_t)((uint64_t)si >> (2 * (dep - k)));
            const int64_t A = level_index(k) + ai;
            real CA[L_NCOEF];
#pragma unroll
            for (int c = 0; c < L_NCOEF; c++) CA[c] = loc[A * L_NCOEF + c];
            const real scale = (real)(1 << (dep - k));
            const real iax = (real)compact16(ai), iay = (real)compact16(ai >> 1);
            // com_S - com_A = (cell centre offset) + (relative COMs)
            const real dx = h * (((real)isx + real(0.5)) - (iax + real(0.5)) * scale) + (csx - comrel[2 * A]);
            const real dy = h * (((real)isy + real(0.5)) - (iay + real(0.5)) * scale) + (csy - comrel[2 * A + 1]);
            add_shifted(CA, dx, dy, C);
        }
        for (uint32_t e = e0; e < e1 && !geo.variant; e++) {  // the non-symmetric solver has no P2L here
            const uint32_t ti = near_idx[e];
            if (ti >= (uint32_t)si) continue;
            const int64_t T = li + ti;
            const uint32_t fT = first[T], cT = count[T];
            const real ox = real(isx - (int)compact16(ti)) * h, oy = real(isy - (int)compact16(ti >> 1)) * h;
            for (uint32_t q = lane; q < cT; q += 32) {
                const uint32_t t = fT + q;
                if (!pn_pass(pos64[t], comS64, lenS, inv_theta)) continue;
                // R' = com_S - x_t
                const real Rx = ox + (csx - prel[2 * t]);
                const real Ry = oy + (csy - prel[2 * t + 1]);
                real D1, D2, D3, tt;
                ker.far(Rx * Rx + Ry * Ry, D1, D2, D3, tt);
                C[L_C1X] += Rx * D1;
                C[L_C1Y] += Ry * D1;
                add_c2c3(Rx, Ry, real(1), D1, D2, D3, C);
                zA += mS * tt;
                n_p2l++;
            }
        }
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = warp_sum(C[c]);
        const double z = (double)warp_sum(zA);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < L_NCOEF; c++) locfin[si * L_NCOEF + c] = C[c];
            zloc[si] = z;
        }
    }
    const unsigned long long c = warp_sum((unsigned long long)n_p2l);
    if (lane == 0 && c) atomicAdd(counters + 2, c);
}

// phase B, one warp per work item (leaf S, chunk of up to 32 sinks of S)
template <typename real, typename K>
__global__ void __launch_bounds__(32 * kLeafWarps)
    k_leaf_near(K ker, Geo geo, const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
                const double2* __restrict__ com64, const double* __restrict__ bblen, const real* __restrict__ comrel,
                const real* __restrict__ m0r, const real* __restrict__ m2t, const real* __restrict__ locfin,
                const uint32_t* __restrict__ near_ptr, const uint32_t* __restrict__ near_idx,
                const uint32_t* __restrict__ chunk_ptr, const double2* __restrict__ pos64,
                const real* __restrict__ prel, const uint32_t* __restrict__ perm, double* __restrict__ grad,
                int accumulate, int scatter, double* __restrict__ zwork, unsigned long long* __restrict__ counters)
{
    __shared__ real s_src[kLeafWarps][32][2];
    uint32_t n_pp = 0, n_m2p = 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int dep = geo.depth;
    const uint32_t li = level_index(dep);
    const int64_t nl = (int64_t)1 << (2 * dep);
    const real h = (real)geo.h_leaf;
    const double inv_theta = geo.inv_theta;
    const uint32_t nwork = chunk_ptr[nl];
    const int64_t wstride = (int64_t)gridDim.x * kLeafWarps;
    for (int64_t wi = blockIdx.x * (int64_t)kLeafWarps + w; wi < nwork; wi += wstride) {
        // leaf of this work item: last si with chunk_ptr[si] <= wi
        int64_t lo = 0, hi = nl;
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (chunk_ptr[mid] <= (uint32_t)wi) lo = mid; else hi = mid;
        }
        const int64_t si = lo;
        const int64_t S = li + si;
        const uint32_t cS = count[S];
        const uint32_t fS = first[S];
        const uint32_t c0 = ((uint32_t)wi - chunk_ptr[si]) * 32u;
        const int isx = (int)compact16((uint32_t)si), isy = (int)compact16((uint32_t)si >> 1);
        const double2 comS64 = com64[S];
        const double lenS = bblen[S];
        const real csx = comrel[2 * S], csy = comrel[2 * S + 1];
        const uint32_t e0 = near_ptr[si], e1 = near_ptr[si + 1];
        real C[L_NCOEF];
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = locfin[si * L_NCOEF + c];

        const uint32_t sl = c0 + lane;
        const bool act = sl < cS;
        const uint32_t s = fS + (act ? sl : 0);
        const real px = prel[2 * s], py = prel[2 * s + 1];
        const double2 x64 = pos64[s];
        real gx = real(0), gy = real(0), zs = real(0);
        if (act) eval_c1(C, px - csx, py - csy, gx, gy);
        for (uint32_t e = e0; e < e1; e++) {
            const uint32_t ti = near_idx[e];
            const int64_t T = li + ti;
            const uint32_t fT = first[T], cT = count[T];
            const real ox = real(isx - (int)compact16(ti)) * h, oy = real(isy - (int)compact16(ti >> 1)) * h;
            // base = x_s - (cell centre of T); each source subtracts its prel
            const real bx = ox + px, by = oy + py;
            if (geo.variant) {
                // non-symmetric: every sink tests every partner T (S itself
                // included): M2P when L_T / |x - com_T| < theta, else P2P over
                // T without the sink itself (traverseBHMP, :199-232)
                const bool pass = act && pn_pass_m(x64, com64[T], bblen[T], geo.theta);
                if (pass) {
                    const real Rx = bx - comrel[2 * T], Ry = by - comrel[2 * T + 1];
                    real D1, D2, D3, t;
                    ker.far(Rx * Rx + Ry * Ry, D1, D2, D3, t);
                    const real mT = m0r[T];
                    real c1x, c1y;
                    far_c1(Rx, Ry, mT, m2t[3 * T], m2t[3 * T + 1], m2t[3 * T + 2], D1, D2, D3, c1x, c1y);
                    gx += c1x;
                    gy += c1y;
                    zs += mT * t;
                    n_m2p++;
                }
                const bool direct = act && !pass;
                if (__any_sync(0xffffffffu, direct)) {
                    for (uint32_t q0 = 0; q0 < cT; q0 += 32) {
                        const uint32_t q = q0 + lane;
                        if (q < cT) {
                            s_src[w][lane][0] = prel[2 * (fT + q)];
                            s_src[w][lane][1] = prel[2 * (fT + q) + 1];
                        }
                        __syncwarp();
                        const uint32_t m = min(32u, cT - q0);
                        if (direct) {
                            const bool self = ti == (uint32_t)si && sl >= q0 && sl < q0 + m;
                            n_pp += m - (self ? 1u : 0u);
                            for (uint32_t j = 0; j < m; j++) {
                                if (self && q0 + j == sl) continue;
                                const real Rx = bx - s_src[w][j][0], Ry = by - s_src[w][j][1];
                                real D1, t;
                                ker.near(Rx * Rx + Ry * Ry, D1, t);
                                gx += D1 * Rx;
                                gy += D1 * Ry;
                                zs += t;
                            }
                        }
                        __syncwarp();
                    }
                }
            } else if (ti == (uint32_t)si) {
                for (uint32_t q0 = 0; q0 < cT; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    if (q < cT) {
                        s_src[w][lane][0] = prel[2 * (fT + q)];
                        s_src[w][lane][1] = prel[2 * (fT + q) + 1];
                    }
                    __syncwarp();
                    const uint32_t m = min(32u, cT - q0);
                    if (act) {
                        n_pp += m - ((sl >= q0 && sl < q0 + m) ? 1u : 0u);
                        for (uint32_t j = 0; j < m; j++) {
                            if (q0 + j == sl) continue;
                            const real Rx = bx - s_src[w][j][0], Ry = by - s_src[w][j][1];
                            real D1, t;
                            ker.near(Rx * Rx + Ry * Ry, D1, t);
                            gx += D1 * Rx;
                            gy += D1 * Ry;
                            zs += t;
                        }
                    }
                    __syncwarp();
                }
            } else if (ti > (uint32_t)si) {
                // S is the first node of the pair: each sink is tested against T
                const bool pass = act && pn_pass(x64, com64[T], bblen[T], inv_theta);
                if (pass) {
                    const real Rx = bx - comrel[2 * T], Ry = by - comrel[2 * T + 1];
                    real D1, D2, D3, t;
                    ker.far(Rx * Rx + Ry * Ry, D1, D2, D3, t);
                    const real mT = m0r[T];
                    real c1x, c1y;
                    far_c1(Rx, Ry, mT, m2t[3 * T], m2t[3 * T + 1], m2t[3 * T + 2], D1, D2, D3, c1x, c1y);
                    gx += c1x;
                    gy += c1y;
                    zs += mT * t;
                    n_m2p++;
                }
                const bool direct = act && !pass;
                if (__any_sync(0xffffffffu, direct)) {
                    for (uint32_t q0 = 0; q0 < cT; q0 += 32) {
                        const uint32_t q = q0 + lane;
                        if (q < cT) {
                            s_src[w][lane][0] = prel[2 * (fT + q)];
                            s_src[w][lane][1] = prel[2 * (fT + q) + 1];
                        }
                        __syncwarp();
                        const uint32_t m = min(32u, cT - q0);
                        if (direct) {
                            n_pp += m;
                            for (uint32_t j = 0; j < m; j++) {
                                const real Rx = bx - s_src[w][j][0], Ry = by - s_src[w][j][1];
                                real D1, t;
                                ker.near(Rx * Rx + Ry * Ry, D1, t);
                                gx += D1 * Rx;
                                gy += D1 * Ry;
                                zs += t;
                            }
                        }
                        __syncwarp();
                    }
                }
            } else {
                // S is the second node: the points of T that fail the MAC
                // against S interact with every sink directly
                for (uint32_t q0 = 0; q0 < cT; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    bool fail = false;
                    real tx = real(0), ty = real(0);
                    if (q < cT) {
                        fail = !pn_pass(pos64[fT + q], comS64, lenS, inv_theta);
                        tx = prel[2 * (fT + q)];
                        ty = prel[2 * (fT + q) + 1];
                    }
                    const uint32_t bal = __ballot_sync(0xffffffffu, fail);
                    if (fail) {
                        const int slot = __popc(bal & ((1u << lane) - 1u));
                        s_src[w][slot][0] = tx;
                        s_src[w][slot][1] = ty;
                    }
                    __syncwarp();
                    const int m = __popc(bal);
                    if (act) {
                        n_pp += (uint32_t)m;
                        for (int j = 0; j < m; j++) {
                            const real Rx = bx - s_src[w][j][0], Ry = by - s_src[w][j][1];
                            real D1, t;
                            ker.near(Rx * Rx + Ry * Ry, D1, t);
                            gx += D1 * Rx;
                            gy += D1 * Ry;
                            zs += t;
                        }
                    }
                    __syncwarp();
                }
            }
        }
        if (act) {
            const int64_t o = scatter ? (int64_t)perm[s] : (int64_t)s;
            double ox2 = (double)gx, oy2 = (double)gy;
            if (accumulate) {
                ox2 += grad[2 * o];
                oy2 += grad[2 * o + 1];
            }
            grad[2 * o] = ox2;
            grad[2 * o + 1] = oy2;
        }
        const double z = warp_sum(act ? (double)zs : 0.0);
        if (lane == 0) zwork[wi] = z;
    }
    const unsigned long long a = warp_sum((unsigned long long)n_pp);
    const unsigned long long b = warp_sum((unsigned long long)n_m2p);
    if (lane == 0 && (a | b)) {
        atomicAdd(counters + 0, a);
        atomicAdd(counters + 1, b);
    }
}

// deterministic sum of the Z partials: per node (M2L), per leaf (P2L) and
// per work item (near field; the count is read from the chunk offsets)
__global__ void k_sum_z(const double* __restrict__ a, int64_t na, const double* __restrict__ b, int64_t nb,
                        const double* __restrict__ c, const uint32_t* __restrict__ nc, double* __restrict__ out,
                        int accumulate)
{
    __shared__ double ws[32];
    double s = 0.0;
    const int64_t ncv = *nc;
    for (int64_t i = threadIdx.x; i < na; i += blockDim.x) s += a[i];
    for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) s += b[i];
    for (int64_t i = threadIdx.x; i < ncv; i += blockDim.x) s += c[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *out = accumulate ? *out + v : v;
    }
}

// final local expansion of every node (what applyForces leaves in the
// reference's node C fields): leaves from the leaf kernel, internal nodes by
// composing the shifted expansions of their ancestors
template <typename real>
__global__ void k_final_locals(int dep, double L, const uint32_t* __restrict__ count,
                               const real* __restrict__ comrel, const real* __restrict__ loc,
                               const real* __restrict__ locfin, double* __restrict__ out, int64_t nn)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
        int l = 0;
        while (l < dep && (int64_t)level_index(l + 1) <= k) l++;
        const uint32_t i = (uint32_t)(k - level_index(l));
        real C[L_NCOEF];
#pragma unroll
        for (int c = 0; c < L_NCOEF; c++) C[c] = real(0);
        if (count[k] != 0) {
            if (l == dep) {
                for (int c = 0; c < L_NCOEF; c++) C[c] = locfin[(int64_t)i * L_NCOEF + c];
            } else {
                const real h = (real)(L / (double)(1u << l));
                const real ix = (real)compact16(i), iy = (real)compact16(i >> 1);
                for (int a = 0; a <= l; a++) {
                    const uint32_t ai = i >> (2 * (l - a));
                    const int64_t A = level_index(a) + ai;
                    real CA[L_NCOEF];
                    for (int c = 0; c < L_NCOEF; c++) CA[c] = loc[A * L_NCOEF + c];
                    const real scale = (real)(1 << (l - a));
                    const real dx = h * ((ix + real(0.5)) - ((real)compact16(ai) + real(0.5)) * scale) +
                                    (comrel[2 * k] - comrel[2 * A]);
                    const real dy = h * ((iy + real(0.5)) - ((real)compact16(ai >> 1) + real(0.5)) * scale) +
                                    (comrel[2 * k + 1] - comrel[2 * A + 1]);
                    add_shifted(CA, dx, dy, C);
                }
            }
        }
        for (int c = 0; c < L_NCOEF; c++) out[k * L_NCOEF + c] = (double)C[c];
    }
}

template <typename real, typename K>
int solve_t(Handle& h, K ker, double* d_grad, int accumulate, int scatter, double* d_total)
{
    cudaStream_t s = h.stream;
    const int dep = h.depth;
    const int64_t nn = h.nnodes;
    const int64_t nleaf = (int64_t)1 << (2 * dep);
    int rc;
    if ((rc = ensure(h.loc, nn * L_NCOEF * sizeof(real))) || (rc = ensure(h.locfin, nleaf * L_NCOEF * sizeof(real))) ||
        (rc = ensure(h.zpart, nn * 8 + 64)))
        return rc;
    if ((rc = ensure(h.counters, 64)) || (rc = record(h, 4))) return rc;
    TC_CUDA_TRY(cudaMemsetAsync(h.counters.p, 0, 64, s));
    double* zp = P<double>(h.zpart);
    real* loc = P<real>(h.loc);
    // the root has no M2L partners
    TC_CUDA_TRY(cudaMemsetAsync(loc, 0, L_NCOEF * sizeof(real), s));
    TC_CUDA_TRY(cudaMemsetAsync(zp, 0, 8, s));
    const uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    const uint32_t* idx = P<uint32_t>(h.idx_pool);
    for (int l = 1; l <= dep; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        const real hl = (real)(h.L / (double)(1u << l));
        k_m2l<real, K><<<grid_for(nl * 32, 128, sm_count() * 64), 128, 0, s>>>(
            ker, l, hl, ptr + h.lists.nn_ptr_off[l], idx + h.lists.nn_idx_off[l], P<real>(h.comrel), P<real>(h.m0r),
            P<real>(h.m2t), loc, zp);
        h.launches++;
    }
    Geo geo;
    geo.depth = dep;
    geo.inv_theta = 1.0 / h.cfg.theta;
    geo.theta = h.cfg.theta;
    geo.h_leaf = h.L / (double)(1u << dep);
    geo.variant = h.variant;
    // work items of the near field: 32-sink chunks of the non-empty leaves
    const int64_t wmax = h.n / 32 + (h.n < nleaf ? h.n : nleaf) + 1;
    if ((rc = ensure(h.chunk, (nleaf + 1) * 4)) || (rc = ensure(h.zwork, wmax * 8)) ||
        (rc = ensure(h.zloc, nleaf * 8)) || (rc = ensure(h.cnt_tmp, nleaf * 4 + 64)) ||
        (rc = ensure(h.tmp, scan_tmp_words(nleaf) * 4)))
        return rc;
    uint32_t* nchunk = P<uint32_t>(h.cnt_tmp);
    uint32_t* chunk_ptr = P<uint32_t>(h.chunk);
    const int64_t nblk = (nleaf + kLeafWarps - 1) / kLeafWarps;
    k_leaf_local<real, K><<<(unsigned)(nblk < sm_count() * 256 ? nblk : sm_count() * 256), 32 * kLeafWarps, 0, s>>>(
        ker, geo, P<uint32_t>(h.count), P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.bblen),
        P<real>(h.comrel), P<real>(h.m0r), loc, ptr + h.lists.near_ptr_off[dep], idx + h.lists.near_idx_off[dep],
        P<double2>(h.pos64), P<real>(h.prel), P<real>(h.locfin), P<double>(h.zloc), nchunk,
        P<unsigned long long>(h.counters));
    if ((rc = exclusive_scan_u32(nchunk, chunk_ptr, nleaf, P<uint32_t>(h.tmp), s))) return rc;
    if ((rc = record(h, 5))) return rc;
    const int64_t wblk = (wmax + kLeafWarps - 1) / kLeafWarps;
    k_leaf_near<real, K><<<(unsigned)(wblk < sm_count() * 256 ? wblk : sm_count() * 256), 32 * kLeafWarps, 0, s>>>(
        ker, geo, P<uint32_t>(h.count), P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.bblen),
        P<real>(h.comrel), P<real>(h.m0r), P<real>(h.m2t), P<real>(h.locfin), ptr + h.lists.near_ptr_off[dep],
        idx + h.lists.near_idx_off[dep], chunk_ptr, P<double2>(h.pos64), P<real>(h.prel), P<uint32_t>(h.perm),
        d_grad, accumulate, scatter, P<double>(h.zwork), P<unsigned long long>(h.counters));
    if ((rc = record(h, 6))) return rc;
    k_sum_z<<<1, 1024, 0, s>>>(zp, nn, P<double>(h.zloc), nleaf, P<double>(h.zwork), chunk_ptr + nleaf, d_total, 1);
    h.launches += 6;
    TC_CUDA_TRY(cudaGetLastError());
    return record(h, 7);
}

}  // namespace

int dump_final_locals(Handle& h, std::vector<double>& out)
{
    out.clear();
    if (!h.loc.p || !h.locfin.p) return TC_OK;
    const int64_t nn = h.nnodes;
    Buf tmp;
    int rc = ensure(tmp, nn * L_NCOEF * 8);
    if (rc) return rc;
    if (h.cfg.precision == TC_PREC_FP64)
        k_final_locals<double><<<grid_for(nn, 128), 128, 0, h.stream>>>(h.depth, h.L, P<uint32_t>(h.count),
                                                                       P<double>(h.comrel), P<double>(h.loc),
                                                                       P<double>(h.locfin), P<double>(tmp), nn);
    else
        k_final_locals<float><<<grid_for(nn, 128), 128, 0, h.stream>>>(h.depth, h.L, P<uint32_t>(h.count),
                                                                      P<float>(h.comrel), P<float>(h.loc),
                                                                      P<float>(h.locfin), P<double>(tmp), nn);
    out.resize(nn * L_NCOEF);
    cudaError_t e = cudaMemcpyAsync(out.data(), tmp.p, nn * L_NCOEF * 8, cudaMemcpyDeviceToHost, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    release(tmp);
    if (e != cudaSuccess) return tc_cuda_fail(e, "dump_final_locals");
    return TC_OK;
}

int solve_fmm(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter)
{
    const double eps2 = h.cfg.softening * h.cfg.softening;
    if (h.cfg.precision == TC_PREC_FP64) {
        if (h.cfg.kernel == TC_KERNEL_GRAVITY) return solve_t<double>(h, KGrav<double>{eps2}, d_grad, accumulate, scatter, d_total);
        return solve_t<double>(h, KTsne<double>{}, d_grad, accumulate, scatter, d_total);
    }
    if (h.cfg.kernel == TC_KERNEL_GRAVITY) return solve_t<float>(h, KGrav<float>{(float)eps2}, d_grad, accumulate, scatter, d_total);
    return solve_t<float>(h, KTsne<float>{}, d_grad, accumulate, scatter, d_total);
}

}  // namespace tc
