/* Oracle shim: unnormalised 3D complex FFT (mixed radix, recursive
 * decimation in time; prime factors fall back to a direct DFT).
 * Test infrastructure for building the reference oracle; not product code. */
#include "openmm/reference/fftpack.h"
#include <cmath>
#include <complex>
#include <vector>

typedef std::complex<double> cplx;

struct fftpack {
    int n[3];
};

static int smallest_factor(int n) {
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0) return p;
    return n;
}

/* out[k] = sum_j in[j*stride] * exp(sign*2*pi*i*j*k/n) */
static void fft1d(const cplx* in, int stride, cplx* out, int n, int sign) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = smallest_factor(n);
    int m = n / p;
    if (p == n) {
        for (int k = 0; k < n; ++k) {
            cplx s = 0;
            for (int j = 0; j < n; ++j) {
                double a = sign * 2.0 * M_PI * (double)((long)j * k % n) / n;
                s += in[j * stride] * cplx(std::cos(a), std::sin(a));
            }
            out[k] = s;
        }
        return;
    }
    /* split into p interleaved sub-sequences of length m */
    std::vector<cplx> sub((size_t)n);
    for (int r = 0; r < p; ++r)
        fft1d(in + r * stride, stride * p, &sub[(size_t)r * m], m, sign);
    for (int k = 0; k < n; ++k) {
        cplx s = 0;
        for (int r = 0; r < p; ++r) {
            double a = sign * 2.0 * M_PI * (double)((long)r * k % n) / n;
            s += sub[(size_t)r * m + (k % m)] * cplx(std::cos(a), std::sin(a));
        }
        out[k] = s;
    }
}

int fftpack_init_3d(fftpack_t* plan, int nx, int ny, int nz) {
    *plan = new fftpack;
    (*plan)->n[0] = nx; (*plan)->n[1] = ny; (*plan)->n[2] = nz;
    return 0;
}

void fftpack_destroy(fftpack_t plan) { delete plan; }

int fftpack_exec_3d(fftpack_t plan, int dir, t_complex* in, t_complex* out) {
    const int nx = plan->n[0], ny = plan->n[1], nz = plan->n[2];
    const int sign = (dir == FFTPACK_FORWARD) ? -1 : 1;
    std::vector<cplx> g((size_t)nx * ny * nz);
    for (size_t i = 0; i < g.size(); ++i) g[i] = cplx(in[i].re, in[i].im);
    int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
    std::vector<cplx> line((size_t)nmax), res((size_t)nmax);
    /* z lines (contiguous) */
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y) {
            cplx* base = &g[((size_t)x * ny + y) * nz];
            fft1d(base, 1, res.data(), nz, sign);
            for (int z = 0; z < nz; ++z) base[z] = res[z];
        }
    /* y lines */
    for (int x = 0; x < nx; ++x)
        for (int z = 0; z < nz; ++z) {
            cplx* base = &g[(size_t)x * ny * nz + z];
            fft1d(base, nz, res.data(), ny, sign);
            for (int y = 0; y < ny; ++y) base[(size_t)y * nz] = res[y];
        }
    /* x lines */
    for (int y = 0; y < ny; ++y)
        for (int z = 0; z < nz; ++z) {
            cplx* base = &g[(size_t)y * nz + z];
            fft1d(base, ny * nz, res.data(), nx, sign);
            for (int x = 0; x < nx; ++x) base[(size_t)x * ny * nz] = res[x];
        }
    for (size_t i = 0; i < g.size(); ++i) { out[i].re = g[i].real(); out[i].im = g[i].imag(); }
    return 0;
}
