// Test infrastructure only.  The reference's particle-mesh solver
// (src/nbodysolvers/cpu/nBodySolverPM.h) calls four FFTW functions through the
// vendored header src/library_src/include/fftw3/fftw3.h; no Linux FFTW library
// exists here.  This file defines those four functions with a plain O(n^2)
// discrete Fourier transform per row and column (FFTW's conventions: r2c keeps
// the n1/2 + 1 non-negative frequencies of the last dimension, c2r is the
// unnormalised inverse and ignores the imaginary parts of the self-conjugate
// columns), so that oracle/_ref/libref_oracle.so can run the reference's PM
// code.  The results equal FFTW's to rounding (not bitwise).
#include <cmath>
#include <complex>
#include <vector>

#include <fftw3/fftw3.h>

struct fftw_plan_s {
    int n0 = 0, n1 = 0;
    bool r2c = true;
    double* rin = nullptr;
    fftw_complex* cin = nullptr;
    double* rout = nullptr;
    fftw_complex* cout = nullptr;
};

namespace {

using cd = std::complex<double>;

// exp(sign 2 pi i k / n) for k = 0..n-1
std::vector<cd> twiddles(int n, int sign)
{
    std::vector<cd> w(n);
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < n; k++) {
        const double a = 2.0 * pi * (double)k / (double)n;
        w[k] = cd(std::cos(a), sign * std::sin(a));
    }
    return w;
}

void execute_r2c(const fftw_plan_s& p)
{
    const int n0 = p.n0, n1 = p.n1, h = n1 / 2 + 1;
    const std::vector<cd> w0 = twiddles(n0, -1), w1 = twiddles(n1, -1);
    std::vector<cd> rows((size_t)n0 * h);
    for (int a = 0; a < n0; a++)
        for (int k = 0; k < h; k++) {
            cd s = 0.0;
            for (int b = 0; b < n1; b++) s += p.rin[(size_t)a * n1 + b] * w1[((size_t)k * b) % n1];
            rows[(size_t)a * h + k] = s;
        }
    for (int k = 0; k < h; k++)
        for (int i = 0; i < n0; i++) {
            cd s = 0.0;
            for (int a = 0; a < n0; a++) s += rows[(size_t)a * h + k] * w0[((size_t)i * a) % n0];
            p.cout[(size_t)i * h + k][0] = s.real();
            p.cout[(size_t)i * h + k][1] = s.imag();
        }
}

void execute_c2r(const fftw_plan_s& p)
{
    const int n0 = p.n0, n1 = p.n1, h = n1 / 2 + 1;
    const std::vector<cd> w0 = twiddles(n0, +1), w1 = twiddles(n1, +1);
    std::vector<cd> cols((size_t)n0 * h);
    for (int k = 0; k < h; k++)
        for (int a = 0; a < n0; a++) {
            cd s = 0.0;
            for (int i = 0; i < n0; i++)
                s += cd(p.cin[(size_t)i * h + k][0], p.cin[(size_t)i * h + k][1]) * w0[((size_t)i * a) % n0];
            cols[(size_t)a * h + k] = s;
        }
    for (int a = 0; a < n0; a++)
        for (int b = 0; b < n1; b++) {
            // the row is Hermitian: Y[n1 - k] = conj(Y[k]); its self-conjugate terms contribute their real part
            double s = cols[(size_t)a * h].real();
            int kmax = h - 1;
            if (n1 % 2 == 0) {
                s += cols[(size_t)a * h + n1 / 2].real() * ((b & 1) ? -1.0 : 1.0);
                kmax = n1 / 2 - 1;
            }
            for (int k = 1; k <= kmax; k++) s += 2.0 * (cols[(size_t)a * h + k] * w1[((size_t)k * b) % n1]).real();
            p.rout[(size_t)a * n1 + b] = s;
        }
}

}  // namespace

extern "C" {

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned)
{
    fftw_plan p = new fftw_plan_s;
    p->n0 = n0;
    p->n1 = n1;
    p->r2c = true;
    p->rin = in;
    p->cout = out;
    return p;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned)
{
    fftw_plan p = new fftw_plan_s;
    p->n0 = n0;
    p->n1 = n1;
    p->r2c = false;
    p->cin = in;
    p->rout = out;
    return p;
}

void fftw_execute(const fftw_plan p)
{
    if (p->r2c) execute_r2c(*p);
    else execute_c2r(*p);
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

}  // extern "C"
