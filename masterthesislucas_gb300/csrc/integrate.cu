// Kick-drift-kick leapfrog for the N-body force step, with FP64 energy and
// momentum diagnostics.  Positions, velocities and accelerations stay on the
// device in input order; every step re-sorts and rebuilds the tree at the
// drifted positions (the solver's update + solve on the handle's stream).
//
// Units: G = 1, equal masses m.  The solver returns, per particle, the
// unit-mass field sum_j (x_j - x_i)/(|x_j - x_i|^2 + eps^2)^(3/2) and the pair
// sum total = -2 sum_(i<j) (|x_i - x_j|^2 + eps^2)^(-1/2), so
//   a_i = m * field_i,   U = m^2 * total / 2,   K = m/2 sum |v_i|^2.
// The diagnostics are deterministic: fixed-size per-block partials summed in
// block order by one block.
#include <cmath>

#include "state.cuh"

namespace tc {
namespace {

constexpr int kDiagBlocks = 1024;
constexpr int kDiagThreads = 256;

// v += a dt/2; x += v dt
__global__ void k_kick_drift(double2* __restrict__ x, double2* __restrict__ v, const double2* __restrict__ a, int64_t n,
                             double half_dt, double dt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 vi = v[i];
        const double2 ai = a[i];
        vi.x += ai.x * half_dt;
        vi.y += ai.y * half_dt;
        v[i] = vi;
        double2 xi = x[i];
        xi.x += vi.x * dt;
        xi.y += vi.y * dt;
        x[i] = xi;
    }
}

// a = m * field; v += a dt/2; per-block partial sums of |v|^2, vx, vy
__global__ void __launch_bounds__(kDiagThreads) k_kick_diag(double2* __restrict__ v, double2* __restrict__ a,
                                                            int64_t n, double mass, double half_dt,
                                                            double* __restrict__ part)
{
    double s2 = 0.0, sx = 0.0, sy = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 ai = a[i];
        ai.x *= mass;
        ai.y *= mass;
        a[i] = ai;
        double2 vi = v[i];
        if (half_dt != 0.0) {
            vi.x += ai.x * half_dt;
            vi.y += ai.y * half_dt;
            v[i] = vi;
        }
        s2 += vi.x * vi.x + vi.y * vi.y;
        sx += vi.x;
        sy += vi.y;
    }
    __shared__ double red[3][kDiagThreads / 32];
    s2 = warp_sum(s2);
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = s2;
        red[1][w] = sx;
        red[2][w] = sy;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < kDiagThreads / 32; k++) t += red[threadIdx.x][k];
        part[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// diag = {K, U, Px, Py}
__global__ void k_diag_final(const double* __restrict__ part, int nblk, const double* __restrict__ total, double mass,
                             double* __restrict__ diag)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s2 = 0.0, sx = 0.0, sy = 0.0;
    for (int b = 0; b < nblk; b++) {
        s2 += part[3 * b];
        sx += part[3 * b + 1];
        sy += part[3 * b + 2];
    }
    diag[0] = 0.5 * mass * s2;
    diag[1] = 0.5 * mass * mass * total[0];
    diag[2] = mass * sx;
    diag[3] = mass * sy;
}

int force(tc_handle* t, const double* d_pos, int64_t n, double* d_acc)
{
    Handle& h = t->h;
    int rc = tc_update_tree_device(t, d_pos, n, nullptr, nullptr);
    if (rc) return rc;
    const int launches = h.launches;
    if ((rc = ensure(h.dtotal, 64))) return rc;
    // the solver accumulates its pair sum into the target, as the reference's solveNbody does
    TC_CUDA_TRY(cudaMemsetAsync(h.dtotal.p, 0, 8, h.stream));
    rc = tc_solve_device(t, d_acc, P<double>(h.dtotal), 0, 1);
    h.launches += launches;
    return rc;
}

}  // namespace
}  // namespace tc

using namespace tc;

extern "C" int tc_leapfrog_step(tc_handle* t, double* d_pos_xy, double* d_vel_xy, double* d_acc_xy, int64_t n,
                                double dt, double mass, int init, double* d_diag)
{
    if (!t || !d_pos_xy || !d_vel_xy || !d_acc_xy || !d_diag || n <= 0 || !(mass > 0.0) || !std::isfinite(dt) ||
        (!init && dt == 0.0)) {
        tc_set_error("tc_leapfrog_step: invalid arguments");
        return TC_ERR_INVALID;
    }
    Handle& h = t->h;
    if (h.cfg.kernel != TC_KERNEL_GRAVITY) {
        tc_set_error("tc_leapfrog_step: needs a gravity handle");
        return TC_ERR_INVALID;
    }
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    cudaStream_t s = h.stream;
    int rc;
    Buf& part = h.diagpart;
    if ((rc = ensure(part, kDiagBlocks * 3 * 8))) return rc;
    const int nblk = grid_for(n, kDiagThreads, kDiagBlocks);
    int launches = 0;
    double2* x = reinterpret_cast<double2*>(d_pos_xy);
    double2* v = reinterpret_cast<double2*>(d_vel_xy);
    double2* a = reinterpret_cast<double2*>(d_acc_xy);
    if (init) {  // the acceleration at the initial positions
        if ((rc = force(t, d_pos_xy, n, d_acc_xy))) return rc;
        launches += h.launches;
        k_kick_diag<<<nblk, kDiagThreads, 0, s>>>(v, a, n, mass, 0.0, P<double>(part));
        launches++;
    }
    if (dt != 0.0) {
        k_kick_drift<<<grid_for(n, 256), 256, 0, s>>>(x, v, a, n, 0.5 * dt, dt);
        TC_CUDA_TRY(cudaGetLastError());
        if ((rc = force(t, d_pos_xy, n, d_acc_xy))) return rc;
        launches += 1 + h.launches;
        k_kick_diag<<<nblk, kDiagThreads, 0, s>>>(v, a, n, mass, 0.5 * dt, P<double>(part));
        launches++;
    }
    k_diag_final<<<1, 32, 0, s>>>(P<double>(part), nblk, P<double>(h.dtotal), mass, d_diag);
    TC_CUDA_TRY(cudaGetLastError());
    h.launches = launches + 1;
    return TC_OK;
}
