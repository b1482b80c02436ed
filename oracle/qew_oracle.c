/*
 * qew_oracle.c -- CPU oracle for the qEW hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Plain-C FP64 restatement of the reference algorithm (IMTEK-Simulation/qEW,
 * src/filtered_noise.h, src/filtered_noise.cpp, src/qew_model.h, src/lbfgs.h,
 * src/dynamics.h, src/rosso_krauth.h, src/fire.h; the seeded field's
 * std::mt19937_64 draws). Only the tests, the smoke check and the benchmark's
 * CPU-baseline leg load this code, and only as the checker.
 *
 * Compile with -ffp-contract=off: the reference is built as ISO C++20 (no GNU
 * extensions), where GCC does not contract a*b+c into an FMA, so expression-
 * by-expression evaluation here reproduces its serial results bit for bit.
 */
#include "qew_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================== */
/* B-spline weights and field sampling                                       */
/* ======================================================================== */

/* filtered_noise.h:33-46 */
void qo_bspline_weights_value(double t, double w[4]) {
    const double t2 = t * t;
    const double t3 = t2 * t;
    const double omt = 1.0 - t;
    w[0] = omt * omt * omt / 6.0;
    w[1] = (4.0 - 6.0 * t2 + 3.0 * t3) / 6.0;
    w[2] = (1.0 + 3.0 * t + 3.0 * t2 - 3.0 * t3) / 6.0;
    w[3] = t3 / 6.0;
}

/* filtered_noise.h:50-62 */
void qo_bspline_weights(double t, double w[4], double dw[4]) {
    qo_bspline_weights_value(t, w);
    const double t2 = t * t;
    const double omt = 1.0 - t;
    dw[0] = -omt * omt / 2.0;
    dw[1] = (-12.0 * t + 9.0 * t2) / 6.0;
    dw[2] = (3.0 + 6.0 * t - 9.0 * t2) / 6.0;
    dw[3] = 3.0 * t2 / 6.0;
}

/* DeviceNoise::locate, filtered_noise.h:77-101 */
static void qo_locate(const qo_noise *nz, double x, double y, int ixn[4],
                      int iyn[4], double *fx, double *fy) {
    const int nx = nz->nx, ny = nz->ny;
    double gx = x / nz->dx;
    double gy = y / nz->dy;
    gx -= floor(gx / (double)nx) * (double)nx;
    gy -= floor(gy / (double)ny) * (double)ny;
    int ix = (int)floor(gx);
    int iy = (int)floor(gy);
    if (ix >= nx) { ix -= nx; gx -= (double)nx; }
    if (iy >= ny) { iy -= ny; gy -= (double)ny; }
    *fx = gx - (double)ix;
    *fy = gy - (double)iy;
    ixn[0] = (ix == 0) ? nx - 1 : ix - 1;
    ixn[1] = ix;
    ixn[2] = (ix + 1 == nx) ? 0 : ix + 1;
    ixn[3] = (ixn[2] + 1 == nx) ? 0 : ixn[2] + 1;
    iyn[0] = (iy == 0) ? ny - 1 : iy - 1;
    iyn[1] = iy;
    iyn[2] = (iy + 1 == ny) ? 0 : iy + 1;
    iyn[3] = (iyn[2] + 1 == ny) ? 0 : iyn[2] + 1;
}

#define COEF(nz, i, j) ((nz)->coef[(size_t)(i) * (size_t)(nz)->ny + (size_t)(j)])

/* DeviceNoise::sample, filtered_noise.h:103-134 */
static void qo_bspline_sample(const qo_noise *nz, double x, double y, double *v,
                              double *dvdx, double *dvdy) {
    int ixn[4], iyn[4];
    double fx, fy;
    qo_locate(nz, x, y, ixn, iyn, &fx, &fy);
    double wx[4], dwx[4], wy[4], dwy[4];
    qo_bspline_weights(fx, wx, dwx);
    qo_bspline_weights(fy, wy, dwy);
    double vv = 0, dgx = 0, dgy = 0;
    for (int a = 0; a < 4; ++a) {
        double row = 0, row_dy = 0;
        for (int b = 0; b < 4; ++b) {
            const double c = COEF(nz, ixn[a], iyn[b]);
            row += c * wy[b];
            row_dy += c * dwy[b];
        }
        vv += wx[a] * row;
        dgx += dwx[a] * row;
        dgy += wx[a] * row_dy;
    }
    *v = vv;
    *dvdx = dgx / nz->dx;
    *dvdy = dgy / nz->dy;
}

/* DeviceNoise::sample_value, filtered_noise.h:138-155 */
static double qo_bspline_value(const qo_noise *nz, double x, double y) {
    int ixn[4], iyn[4];
    double fx, fy;
    qo_locate(nz, x, y, ixn, iyn, &fx, &fy);
    double wx[4], wy[4];
    qo_bspline_weights_value(fx, wx);
    qo_bspline_weights_value(fy, wy);
    double v = 0;
    for (int a = 0; a < 4; ++a) {
        double row = 0;
        for (int b = 0; b < 4; ++b) row += COEF(nz, ixn[a], iyn[b]) * wy[b];
        v += wx[a] * row;
    }
    return v;
}

/* DeviceNoise::sample_dy, filtered_noise.h:159-176 */
static double qo_bspline_dy(const qo_noise *nz, double x, double y) {
    int ixn[4], iyn[4];
    double fx, fy;
    qo_locate(nz, x, y, ixn, iyn, &fx, &fy);
    double wx[4], wy[4], dwy[4];
    qo_bspline_weights_value(fx, wx);
    qo_bspline_weights(fy, wy, dwy);
    double dgy = 0;
    for (int a = 0; a < 4; ++a) {
        double row_dy = 0;
        for (int b = 0; b < 4; ++b) row_dy += COEF(nz, ixn[a], iyn[b]) * dwy[b];
        dgy += wx[a] * row_dy;
    }
    return dgy / nz->dy;
}

/* Analytic test potentials: the Noise functors of the reference's tests
 * (test_qew_model.cpp:22-42, test_lbfgs.cpp:24-38,
 * test_rosso_krauth.cpp:24-31, test_dynamics.cpp:20-28). */
static void qo_analytic_sample(const qo_noise *nz, double x, double y,
                               double *v, double *dvdx, double *dvdy) {
    switch (nz->kind) {
    case QO_NOISE_ZERO:
        *v = 0; *dvdx = 0; *dvdy = 0;
        return;
    case QO_NOISE_CONST:
        *v = nz->p0; *dvdx = 0; *dvdy = 0;
        return;
    case QO_NOISE_HARMONIC: {
        const double d = y - nz->p1;
        *v = 0.5 * nz->p0 * d * d;
        *dvdx = 0;
        *dvdy = nz->p0 * d;
        return;
    }
    case QO_NOISE_WASHBOARD:
        *v = nz->p0 * cos(nz->p1 * y);
        *dvdx = 0;
        *dvdy = -nz->p0 * nz->p1 * sin(nz->p1 * y);
        return;
    case QO_NOISE_SINCOS: {
        const double amp = nz->p0, kx = nz->p1, ky = nz->p2;
        *v = amp * sin(kx * x) * cos(ky * y);
        *dvdx = amp * kx * cos(kx * x) * cos(ky * y);
        *dvdy = -amp * ky * sin(kx * x) * sin(ky * y);
        return;
    }
    default:
        *v = 0; *dvdx = 0; *dvdy = 0;
    }
}

void qo_sample(const qo_noise *nz, double x, double y, double *v, double *dvdx,
               double *dvdy) {
    if (nz->kind == QO_NOISE_BSPLINE)
        qo_bspline_sample(nz, x, y, v, dvdx, dvdy);
    else
        qo_analytic_sample(nz, x, y, v, dvdx, dvdy);
}

/* detail::noise_value, qew_model.h:31-38 */
double qo_sample_value(const qo_noise *nz, double x, double y) {
    if (nz->kind == QO_NOISE_BSPLINE) return qo_bspline_value(nz, x, y);
    double v, a, b;
    qo_analytic_sample(nz, x, y, &v, &a, &b);
    return v;
}

/* detail::noise_dvdy, qew_model.h:40-46 */
double qo_sample_dy(const qo_noise *nz, double x, double y) {
    if (nz->kind == QO_NOISE_BSPLINE) return qo_bspline_dy(nz, x, y);
    double v, a, b;
    qo_analytic_sample(nz, x, y, &v, &a, &b);
    return b;
}

void qo_sample_many(const qo_noise *nz, const double *x, const double *y, int m,
                    double *v, double *dvdx, double *dvdy) {
    for (int k = 0; k < m; ++k) qo_sample(nz, x[k], y[k], &v[k], &dvdx[k], &dvdy[k]);
}

/* ======================================================================== */
/* FFT (stands in for kokkos-fft v1.1.0 / FFTW; forward unnormalised,        */
/* backward scaled by 1/n). Recursive mixed-radix decimation in time with a  */
/* direct DFT for each prime factor: exact for any n, O(n * sum of factors). */
/* ======================================================================== */

static int smallest_factor(int n) {
    if (n % 2 == 0) return 2;
    for (int p = 3; (long)p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* out[k] = sum_j in[j*stride] exp(sign*2*pi*i*j*k/n) */
static void fft_rec(const double *ire, const double *iim, int stride,
                    double *ore, double *oim, int n, int sign) {
    if (n == 1) {
        ore[0] = ire[0];
        oim[0] = iim[0];
        return;
    }
    const int p = smallest_factor(n);
    const int m = n / p;
    for (int r = 0; r < p; ++r)
        fft_rec(ire + (size_t)r * stride, iim + (size_t)r * stride, stride * p,
                ore + (size_t)r * m, oim + (size_t)r * m, m, sign);
    const double two_pi = 2.0 * acos(-1.0);
    double *tre = (double *)malloc(sizeof(double) * 2 * (size_t)p);
    double *tim = tre + p;
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            const double ang = sign * two_pi * (double)((long)r * k % n) / (double)n;
            const double c = cos(ang), s = sin(ang);
            const double xr = ore[(size_t)r * m + k], xi = oim[(size_t)r * m + k];
            tre[r] = xr * c - xi * s;
            tim[r] = xr * s + xi * c;
        }
        for (int q = 0; q < p; ++q) {
            double sr = 0, si = 0;
            for (int r = 0; r < p; ++r) {
                const long e = ((long)r * q) % p;
                const double ang = sign * two_pi * (double)e / (double)p;
                const double c = cos(ang), s = sin(ang);
                sr += tre[r] * c - tim[r] * s;
                si += tre[r] * s + tim[r] * c;
            }
            ore[(size_t)k + (size_t)q * m] = sr;
            oim[(size_t)k + (size_t)q * m] = si;
        }
    }
    free(tre);
}

int qo_fft(double *re, double *im, int n, int inverse) {
    if (n <= 0) return -1;
    double *ire = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!ire) return -1;
    double *iim = ire + n;
    memcpy(ire, re, sizeof(double) * (size_t)n);
    memcpy(iim, im, sizeof(double) * (size_t)n);
    fft_rec(ire, iim, 1, re, im, n, inverse ? 1 : -1);
    if (inverse) {
        for (int k = 0; k < n; ++k) {
            re[k] /= (double)n;
            im[k] /= (double)n;
        }
    }
    free(ire);
    return 0;
}

int qo_rfft(const double *x, int n, double *re, double *im) {
    double *a = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!a) return -1;
    double *b = a + n;
    for (int k = 0; k < n; ++k) { a[k] = x[k]; b[k] = 0; }
    qo_fft(a, b, n, 0);
    for (int k = 0; k < n / 2 + 1; ++k) { re[k] = a[k]; im[k] = b[k]; }
    free(a);
    return 0;
}

int qo_irfft(const double *re, const double *im, int n, double *x) {
    double *a = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    if (!a) return -1;
    double *b = a + n;
    const int nh = n / 2 + 1;
    for (int k = 0; k < nh; ++k) { a[k] = re[k]; b[k] = im[k]; }
    /* Hermitian completion; the imaginary parts of the DC (and, for even n,
     * Nyquist) bins do not contribute to a real output. */
    b[0] = 0;
    if (n % 2 == 0) b[n / 2] = 0;
    for (int k = nh; k < n; ++k) { a[k] = re[n - k]; b[k] = -im[n - k]; }
    qo_fft(a, b, n, 1);
    for (int k = 0; k < n; ++k) x[k] = a[k];
    free(a);
    return 0;
}

/* FilteredNoise::build_coefficients, filtered_noise.cpp:92-136:
 * c = IFFT2(FFT2(field) / (Kx (x) Ky)), K[m] = 2/3 + cos(2 pi m / N) / 3. */
int qo_prefilter(const double *field, int nx, int ny, double *coef) {
    const size_t N = (size_t)nx * ny;
    double *re = (double *)malloc(sizeof(double) * 2 * N);
    double *lre = (double *)malloc(sizeof(double) * 2 * (size_t)(nx > ny ? nx : ny));
    if (!re || !lre) { free(re); free(lre); return -1; }
    double *im = re + N;
    const int nl = nx > ny ? nx : ny;
    double *lim = lre + nl;
    for (size_t k = 0; k < N; ++k) { re[k] = field[k]; im[k] = 0; }
    /* forward along y (contiguous) then x */
    for (int i = 0; i < nx; ++i) qo_fft(re + (size_t)i * ny, im + (size_t)i * ny, ny, 0);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) { lre[i] = re[(size_t)i * ny + j]; lim[i] = im[(size_t)i * ny + j]; }
        qo_fft(lre, lim, nx, 0);
        for (int i = 0; i < nx; ++i) { re[(size_t)i * ny + j] = lre[i]; im[(size_t)i * ny + j] = lim[i]; }
    }
    const double two_pi = 2.0 * acos(-1.0);
    for (int i = 0; i < nx; ++i) {
        const double kx = 2.0 / 3 + cos(two_pi * i / nx) / 3.0;
        for (int j = 0; j < ny; ++j) {
            const double ky = 2.0 / 3 + cos(two_pi * j / ny) / 3.0;
            const double den = kx * ky;
            re[(size_t)i * ny + j] /= den;
            im[(size_t)i * ny + j] /= den;
        }
    }
    /* inverse (each 1-D inverse scales by 1/len: total 1/(nx*ny)) */
    for (int i = 0; i < nx; ++i) qo_fft(re + (size_t)i * ny, im + (size_t)i * ny, ny, 1);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) { lre[i] = re[(size_t)i * ny + j]; lim[i] = im[(size_t)i * ny + j]; }
        qo_fft(lre, lim, nx, 1);
        for (int i = 0; i < nx; ++i) { re[(size_t)i * ny + j] = lre[i]; im[(size_t)i * ny + j] = lim[i]; }
    }
    for (size_t k = 0; k < N; ++k) coef[k] = re[k];
    free(re);
    free(lre);
    return 0;
}

/* ======================================================================== */
/* Seeded field (FilteredNoise's generating constructor)                    */
/* ======================================================================== */

/* The 64-bit Mersenne Twister with the parameters of C++'s std::mt19937_64
 * (Matsumoto and Nishimura, ACM TOMACS 8 (1998); Nishimura, ACM TOMACS 10
 * (2000)): w = 64, n = 312, m = 156, r = 31, a = 0xb5026f5aa96619e9,
 * (u, d) = (29, 0x5555555555555555), (s, b) = (17, 0x71d67fffeda60000),
 * (t, c) = (37, 0xfff7eee000000000), l = 43, seeding multiplier
 * 6364136223846793005. */
void qo_mt64_seed(qo_mt64 *g, uint64_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < 312; ++i)
        g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
    g->idx = 312;
}

uint64_t qo_mt64_next(qo_mt64 *g) {
    const uint64_t upper = ~0ULL << 31, lower = (1ULL << 31) - 1;
    if (g->idx >= 312) {
        for (int i = 0; i < 312; ++i) {
            const uint64_t x = (g->mt[i] & upper) | (g->mt[(i + 1) % 312] & lower);
            uint64_t xa = x >> 1;
            if (x & 1) xa ^= 0xb5026f5aa96619e9ULL;
            g->mt[i] = g->mt[(i + 156) % 312] ^ xa;
        }
        g->idx = 0;
    }
    uint64_t y = g->mt[g->idx++];
    y ^= (y >> 29) & 0x5555555555555555ULL;
    y ^= (y << 17) & 0x71d67fffeda60000ULL;
    y ^= (y << 37) & 0xfff7eee000000000ULL;
    y ^= y >> 43;
    return y;
}

/* std::uniform_real_distribution<double>(a, b) over a 64-bit engine as
 * libstdc++ evaluates it: generate_canonical<double, 53> takes one draw,
 * u = double(x) / 2^64 (nudged below 1 if it rounds up to 1), then
 * u * (b - a) + a. */
double qo_mt64_uniform(qo_mt64 *g, double a, double b) {
    double u = (double)qo_mt64_next(g) / 18446744073709551616.0;
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    return u * (b - a) + a;
}

static double qo_fftfreq(int k, int n) { /* filtered_noise.cpp:18-21 */
    const int ks = (k < (n + 1) / 2) ? k : k - n;
    return (double)ks / (double)n;
}

/* FilteredNoise(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed),
 * filtered_noise.cpp:25-82: masked random phases, inverse FFT2 (1/(nx ny)),
 * real part scaled to population std `amplitude`. field is [nx][ny]. */
int qo_seeded_field(int nx, int ny, double Lx, double Ly, double amplitude, double xi_x,
                    double xi_y, uint64_t seed, double *field) {
    const size_t N = (size_t)nx * ny;
    double *re = (double *)malloc(sizeof(double) * 2 * N);
    const int nl = nx > ny ? nx : ny;
    double *lre = (double *)malloc(sizeof(double) * 2 * (size_t)nl);
    qo_mt64 *g = (qo_mt64 *)malloc(sizeof(qo_mt64));
    if (!re || !lre || !g) { free(re); free(lre); free(g); return -1; }
    double *im = re + N, *lim = lre + nl;
    const double two_pi = 2.0 * acos(-1.0);
    const double dx = Lx / nx, dy = Ly / ny;
    qo_mt64_seed(g, seed);
    for (int i = 0; i < nx; ++i) {
        const double fx = qo_fftfreq(i, nx) / dx;
        for (int j = 0; j < ny; ++j) {
            const double fy = qo_fftfreq(j, ny) / dy;
            const double ph = qo_mt64_uniform(g, 0.0, two_pi);
            const size_t k = (size_t)i * ny + j;
            if ((fx * xi_x) * (fx * xi_x) + (fy * xi_y) * (fy * xi_y) > 1.0) {
                re[k] = 0.0;
                im[k] = 0.0;
            } else {
                re[k] = cos(ph);
                im[k] = sin(ph);
            }
        }
    }
    for (int i = 0; i < nx; ++i) qo_fft(re + (size_t)i * ny, im + (size_t)i * ny, ny, 1);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) { lre[i] = re[(size_t)i * ny + j]; lim[i] = im[(size_t)i * ny + j]; }
        qo_fft(lre, lim, nx, 1);
        for (int i = 0; i < nx; ++i) re[(size_t)i * ny + j] = lre[i];
    }
    double mean = 0.0;
    for (size_t k = 0; k < N; ++k) mean += re[k];
    mean /= (double)N;
    double var = 0.0;
    for (size_t k = 0; k < N; ++k) {
        const double d = re[k] - mean;
        var += d * d;
    }
    const double scale = amplitude / sqrt(var / (double)N);
    for (size_t k = 0; k < N; ++k) field[k] = re[k] * scale;
    free(re);
    free(lre);
    free(g);
    return 0;
}

/* ======================================================================== */
/* Model: objective and gradient (qew_model.h)                              */
/* ======================================================================== */

/* One edge's energy term, detail::objective_eval body, qew_model.h:61-83 */
static inline double qo_edge_energy(int i, int ip, double hi, double hip,
                                    double dx, double lt, double f, int model,
                                    const qo_noise *nz) {
    const double dh_dx = (hip - hi) / dx;
    double line_energy;
    if (model == 0)
        line_energy = lt * dh_dx * dh_dx * 0.5;
    else
        line_energy = lt * (sqrt(1.0 + dh_dx * dh_dx) - 1.0);
    const double xc = (double)(i + ip) * 0.5 * dx;
    const double hc = (hip + hi) * 0.5;
    return dx * (line_energy + qo_sample_value(nz, xc, hc) - f * hi);
}

/* objective(h, p, noise), qew_model.h:102-109 (Kokkos Serial order) */
double qo_objective(const double *h, int n, const qo_params *p,
                    const qo_noise *nz) {
    const double dx = p->physical_size / (double)n;
    double total = 0.0;
    for (int i = 0; i < n; ++i) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        total += qo_edge_energy(i, ip, h[i], h[ip], dx, p->line_tension,
                                p->driving_force, p->model, nz);
    }
    return total;
}

double qo_objective_omp(const double *h, int n, const qo_params *p,
                        const qo_noise *nz) {
    const double dx = p->physical_size / (double)n;
    double total = 0.0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (int i = 0; i < n; ++i) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        total += qo_edge_energy(i, ip, h[i], h[ip], dx, p->line_tension,
                                p->driving_force, p->model, nz);
    }
    return total;
}

/* objective(x0, d, alpha, p, noise) via TrialAt, qew_model.h:112-119,
 * 92-98: the trial point x0 + alpha*d is formed on the fly. */
double qo_objective_trial(const double *x0, const double *d, double alpha,
                          int n, const qo_params *p, const qo_noise *nz) {
    const double dx = p->physical_size / (double)n;
    double total = 0.0;
    for (int i = 0; i < n; ++i) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const double hi = x0[i] + alpha * d[i];
        const double hip = x0[ip] + alpha * d[ip];
        total += qo_edge_energy(i, ip, hi, hip, dx, p->line_tension,
                                p->driving_force, p->model, nz);
    }
    return total;
}

/* gradient(), qew_model.h:149-193: edge pass then per-site combine */
static void qo_gradient_impl(const double *h, int n, const qo_params *p,
                             const qo_noise *nz, double *grad, int par) {
    const double dx = p->physical_size / (double)n;
    const double lt = p->line_tension;
    const double f = p->driving_force;
    const int arc = (p->model == 1);
    double *edvdy = (double *)malloc(sizeof(double) * (size_t)n);
    double *eslope = (double *)malloc(sizeof(double) * (size_t)n);
    (void)par;
#pragma omp parallel for schedule(static) if (par)
    for (int i = 0; i < n; ++i) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const double xc = (double)(i + ip) * 0.5 * dx;
        const double hc = (h[ip] + h[i]) * 0.5;
        edvdy[i] = qo_sample_dy(nz, xc, hc);
        if (arc) {
            const double dh = (h[ip] - h[i]) / dx;
            eslope[i] = dh / sqrt(1.0 + dh * dh);
        }
    }
#pragma omp parallel for schedule(static) if (par)
    for (int i = 0; i < n; ++i) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const int im = (i == 0) ? n - 1 : i - 1;
        double line_force;
        if (!arc) {
            const double d2h = h[im] + h[ip] - 2.0 * h[i];
            line_force = -lt * d2h / (dx * dx);
        } else {
            line_force = lt * (eslope[im] - eslope[i]) / dx;
        }
        grad[i] = dx * (line_force + 0.5 * (edvdy[im] + edvdy[i]) - f);
    }
    free(edvdy);
    free(eslope);
}

void qo_gradient(const double *h, int n, const qo_params *p,
                 const qo_noise *nz, double *grad) {
    qo_gradient_impl(h, n, p, nz, grad, 0);
}

/* fire_minimize, fire.h:41-131: v += dt F; P = F.v; adapt dt / alpha; mix v
 * toward F; h += dt v; F refreshed. Serial sums in index order. */
void qo_fire_minimize(double *h, int n, const qo_params *p, const qo_noise *nz,
                      const qo_fire_params *fp, qo_fire_result *res) {
    double *g = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    double *v = g + n;
    for (int i = 0; i < n; ++i) v[i] = 0.0;
    double dt = (fp->dt_init > 0) ? fp->dt_init : 0.1 * fp->dt_max;
    double alpha = fp->alpha_start;
    int n_pos = 0;
    qo_gradient(h, n, p, nz, g);
    for (int it = 0; it < fp->max_iter; ++it) {
        double m = 0.0;
        for (int i = 0; i < n; ++i) {
            const double a = fabs(g[i]);
            if (a > m) m = a;
        }
        if (m < fp->ftol) {
            res->iterations = it;
            res->max_force = m;
            res->converged = 1;
            free(g);
            return;
        }
        for (int i = 0; i < n; ++i) v[i] -= dt * g[i];
        double P = 0.0;
        for (int i = 0; i < n; ++i) P += -g[i] * v[i];
        if (P > 0) {
            if (n_pos > fp->n_min) {
                dt = fmin(dt * fp->f_inc, fp->dt_max);
                alpha *= fp->f_alpha;
            }
            ++n_pos;
        } else {
            for (int i = 0; i < n; ++i) v[i] = 0.0;
            dt *= fp->f_dec;
            alpha = fp->alpha_start;
            n_pos = 0;
        }
        double nv2 = 0.0, nf2 = 0.0;
        for (int i = 0; i < n; ++i) nv2 += v[i] * v[i];
        for (int i = 0; i < n; ++i) nf2 += g[i] * g[i];
        const double nf = sqrt(nf2);
        if (nf > 0) {
            const double a = alpha;
            const double scale = alpha * sqrt(nv2) / nf;
            for (int i = 0; i < n; ++i) v[i] = (1.0 - a) * v[i] - scale * g[i];
        }
        for (int i = 0; i < n; ++i) h[i] += dt * v[i];
        qo_gradient(h, n, p, nz, g);
    }
    double m = 0.0;
    for (int i = 0; i < n; ++i) {
        const double a = fabs(g[i]);
        if (a > m) m = a;
    }
    res->iterations = fp->max_iter;
    res->max_force = m;
    res->converged = 0;
    free(g);
}

void qo_gradient_omp(const double *h, int n, const qo_params *p,
                     const qo_noise *nz, double *grad) {
    qo_gradient_impl(h, n, p, nz, grad, 1);
}

int qo_omp_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ======================================================================== */
/* L-BFGS (lbfgs.h:94-287)                                                   */
/* ======================================================================== */

void qo_lbfgs_default_params(qo_lbfgs_params *lp) { /* lbfgs.h:32-52 */
    lp->m = 8;
    lp->ftol = 1e-6;
    lp->max_iter = 10000;
    lp->c1 = 1e-4;
    lp->ls_shrink = 0.5;
    lp->max_ls = 30;
    lp->curvature_eps = 1e-12;
    lp->precondition = 0;
    lp->precond_shift = 0;
    lp->ls_fallback = 0;
}

static double qo_dot(int n, const double *a, const double *b) { /* lbfgs.h:65-71 */
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static double qo_max_abs(int n, const double *a) { /* lbfgs.h:73-83 */
    double s = 0;
    for (int i = 0; i < n; ++i) {
        const double v = fabs(a[i]);
        if (v > s) s = v;
    }
    return s;
}

static void qo_axpy(int n, double c, const double *x, double *y) { /* lbfgs.h:85-88 */
    for (int i = 0; i < n; ++i) y[i] += c * x[i];
}

/* Elastic-Hessian eigenvalues and the preconditioner, lbfgs.h:127-146 */
static double qo_precond_shift(int n, double kappa, double physical_size,
                               double shift) {
    if (shift <= 0) {
        const double pi = 3.14159265358979323846;
        const double dx = physical_size / (double)n;
        const double s1 = sin(pi / (double)n);
        shift = (kappa / dx) * 4 * s1 * s1;
    }
    return shift;
}

static void qo_precond_eig(int n, double kappa, double physical_size,
                           double shift, double *eig) {
    const double pi = 3.14159265358979323846;
    const double dx = physical_size / (double)n;
    const double sh = qo_precond_shift(n, kappa, physical_size, shift);
    for (int k = 0; k < n / 2 + 1; ++k) {
        const double s = sin(pi * (double)k / (double)n);
        eig[k] = (kappa / dx) * 4 * s * s + sh;
    }
}

/* d = irfft(rfft(q) / eig), lbfgs.h:173-180 */
static void qo_precond_apply_eig(const double *q, int n, const double *eig,
                                 double *re, double *im, double *d) {
    qo_rfft(q, n, re, im);
    for (int k = 0; k < n / 2 + 1; ++k) {
        re[k] = re[k] / eig[k];
        im[k] = im[k] / eig[k];
    }
    qo_irfft(re, im, n, d);
}

int qo_precond_apply(const double *q, int n, double kappa, double physical_size,
                     double shift, double *d) {
    double *eig = (double *)malloc(sizeof(double) * 3 * (size_t)(n / 2 + 1));
    if (!eig) return -1;
    double *re = eig + (n / 2 + 1), *im = re + (n / 2 + 1);
    qo_precond_eig(n, kappa, physical_size, shift, eig);
    qo_precond_apply_eig(q, n, eig, re, im, d);
    free(eig);
    return 0;
}

int qo_lbfgs_minimize(double *h, int n, const qo_params *p,
                      const qo_noise *nz, const qo_lbfgs_params *lp,
                      qo_lbfgs_result *res) {
    const int m = lp->m;
    const size_t nb = sizeof(double) * (size_t)n;
    double *g = (double *)malloc(nb), *g_new = (double *)malloc(nb);
    double *d = (double *)malloc(nb), *q = (double *)malloc(nb);
    double *s_tmp = (double *)malloc(nb), *y_tmp = (double *)malloc(nb);
    double **S = (double **)malloc(sizeof(double *) * (size_t)(m > 0 ? m : 1));
    double **Y = (double **)malloc(sizeof(double *) * (size_t)(m > 0 ? m : 1));
    double *rho = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    int *slots = (int *)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    double *la = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    for (int k = 0; k < m; ++k) {
        S[k] = (double *)calloc((size_t)n, sizeof(double));
        Y[k] = (double *)calloc((size_t)n, sizeof(double));
    }
    int nslots = 0;
    double gamma = 1.0;
    const int nh = n / 2 + 1;
    double *eig = NULL, *qre = NULL, *qim = NULL;
    if (lp->precondition) {
        eig = (double *)malloc(sizeof(double) * (size_t)nh);
        qre = (double *)malloc(sizeof(double) * (size_t)nh);
        qim = (double *)malloc(sizeof(double) * (size_t)nh);
        qo_precond_eig(n, p->line_tension, p->physical_size, lp->precond_shift, eig);
    }
    memset(res, 0, sizeof(*res));

    qo_gradient(h, n, p, nz, g);
    int ls_fail_streak = 0;
    double phi = 0;
    int done = 0;

    for (int it = 0; it < lp->max_iter && !done; ++it) {
        const double gmax = qo_max_abs(n, g);
        if (gmax < lp->ftol) { /* lbfgs.h:155-161 */
            res->iterations = it;
            res->max_force = gmax;
            res->converged = 1;
            done = 1;
            break;
        }
        /* two-loop recursion, lbfgs.h:163-191 */
        memcpy(q, g, nb);
        const int hs = nslots;
        for (int idx = hs - 1; idx >= 0; --idx) {
            const int row = slots[idx];
            const double a = rho[row] * qo_dot(n, S[row], q);
            la[idx] = a;
            qo_axpy(n, -a, Y[row], q);
        }
        if (lp->precondition) {
            qo_precond_apply_eig(q, n, eig, qre, qim, d);
        } else {
            const double g0 = (nslots == 0) ? 1.0 : gamma;
            for (int i = 0; i < n; ++i) d[i] = g0 * q[i];
        }
        for (int idx = 0; idx < hs; ++idx) {
            const int row = slots[idx];
            const double b = rho[row] * qo_dot(n, Y[row], d);
            qo_axpy(n, la[idx] - b, S[row], d);
        }
        for (int i = 0; i < n; ++i) d[i] = -d[i];

        /* descent check, lbfgs.h:193-200 */
        double dphi0 = qo_dot(n, g, d);
        if (dphi0 >= 0) {
            nslots = 0;
            for (int i = 0; i < n; ++i) d[i] = -g[i];
            dphi0 = -qo_dot(n, g, g);
        }
        /* Armijo backtracking, lbfgs.h:202-238 */
        if (it == 0) {
            phi = qo_objective(h, n, p, nz);
            ++res->n_func_evals;
        }
        const double phi0 = phi;
        double alpha = 1.0;
        if (!lp->precondition && nslots == 0) {
            const double gn = sqrt(qo_dot(n, g, g));
            alpha = 1.0 / (gn > 1.0 ? gn : 1.0);
        }
        int ok = 0, have_gn = 0;
        for (int ls = 0; ls < lp->max_ls; ++ls) {
            const double phi_trial = qo_objective_trial(h, d, alpha, n, p, nz);
            ++res->n_func_evals;
            if (phi_trial <= phi0 + lp->c1 * alpha * dphi0) {
                phi = phi_trial;
                ok = 1;
                break;
            }
            if (lp->ls_fallback) {
                /* Extension, not in the reference: approximate-Wolfe test of
                 * Hager & Zhang (2005) on the slope at q = h + alpha d. */
                for (int i = 0; i < n; ++i) q[i] = h[i] + alpha * d[i];
                qo_gradient(q, n, p, nz, g_new);
                const double dphia = qo_dot(n, g_new, d);
                ++res->n_func_evals;
                if (dphia >= 0.9 * dphi0 && dphia <= (2.0 * 0.1 - 1.0) * dphi0 &&
                    phi_trial <= phi0 + 1e-10 * fabs(phi0)) {
                    phi = phi_trial;
                    ok = 1;
                    have_gn = 1;
                    break;
                }
            }
            alpha *= lp->ls_shrink;
        }
        if (!ok) {
            if (nslots == 0 || ++ls_fail_streak > 2) {
                res->iterations = it;
                res->max_force = gmax;
                res->converged = 0;
                done = 1;
                break;
            }
            nslots = 0;
            ++res->n_ls_restarts;
            continue;
        }
        ls_fail_streak = 0;
        /* commit, lbfgs.h:241-244 */
        const double al = alpha;
        for (int i = 0; i < n; ++i) h[i] += al * d[i];
        /* curvature pair, lbfgs.h:246-279 */
        if (!have_gn) qo_gradient(h, n, p, nz, g_new);
        double sy = 0, ss = 0, yy = 0;
        for (int i = 0; i < n; ++i) {
            const double s = al * d[i];
            const double y = g_new[i] - g[i];
            s_tmp[i] = s;
            y_tmp[i] = y;
            sy += s * y;
            ss += s * s;
            yy += y * y;
        }
        if (sy > lp->curvature_eps * sqrt(ss * yy)) {
            int row;
            if (nslots < m) {
                row = nslots;
            } else {
                row = slots[0];
                memmove(slots, slots + 1, sizeof(int) * (size_t)(nslots - 1));
                --nslots;
            }
            double *t = S[row]; S[row] = s_tmp; s_tmp = t;
            t = Y[row]; Y[row] = y_tmp; y_tmp = t;
            rho[row] = 1.0 / sy;
            gamma = sy / yy;
            slots[nslots++] = row;
        } else {
            ++res->n_curvature_skips;
        }
        double *t = g; g = g_new; g_new = t;
    }
    if (!done) { /* lbfgs.h:283-286 */
        res->iterations = lp->max_iter;
        res->max_force = qo_max_abs(n, g);
        res->converged = 0;
    }
    for (int k = 0; k < m; ++k) { free(S[k]); free(Y[k]); }
    free(S); free(Y); free(rho); free(slots); free(la);
    free(g); free(g_new); free(d); free(q); free(s_tmp); free(y_tmp);
    free(eig); free(qre); free(qim);
    return 0;
}

/* ======================================================================== */
/* Langevin step (dynamics.h:34-64) with supplied increments                 */
/* ======================================================================== */

void qo_langevin_step(double *h, int n, const qo_params *p, const qo_noise *nz,
                      double drift, double diff, const double *xi,
                      double *grad) {
    qo_gradient(h, n, p, nz, grad);
    const double a = drift, b = diff;
    if (b > 0) {
        for (int i = 0; i < n; ++i) h[i] += -a * grad[i] + b * xi[i];
    } else {
        for (int i = 0; i < n; ++i) h[i] += -a * grad[i];
    }
}

/* ======================================================================== */
/* Rosso-Krauth (rosso_krauth.h)                                             */
/* ======================================================================== */

/* rk_site_velocity, rosso_krauth.h:51-82 */
double qo_rk_site_velocity(int i, int n, double dx, double lt, double f,
                           int model, double hi, double hl, double hr,
                           const qo_noise *nz) {
    const int im = (i == 0) ? n - 1 : i - 1;
    const int ip = (i + 1 == n) ? 0 : i + 1;
    double line_force;
    if (model == 0) {
        line_force = -lt * (hl + hr - 2.0 * hi) / (dx * dx);
    } else {
        const double dhr = (hr - hi) / dx;
        const double dhl = (hi - hl) / dx;
        line_force = lt * (dhl / sqrt(1.0 + dhl * dhl) - dhr / sqrt(1.0 + dhr * dhr)) / dx;
    }
    const double xcl = (double)(im + i) * 0.5 * dx;
    const double hcl = (hl + hi) * 0.5;
    const double xcr = (double)(i + ip) * 0.5 * dx;
    const double hcr = (hi + hr) * 0.5;
    const double dvl = qo_sample_dy(nz, xcl, hcl);
    const double dvr = qo_sample_dy(nz, xcr, hcr);
    const double grad = dx * (line_force + 0.5 * (dvl + dvr) - f);
    return -grad;
}

/* rk_forward_zero, rosso_krauth.h:88-124 */
double qo_rk_forward_zero(int i, int n, double dx, double lt, double f,
                          int model, double hi, double hl, double hr,
                          const qo_noise *nz, const qo_rk_params *rp,
                          int *found) {
    const double v0 = qo_rk_site_velocity(i, n, dx, lt, f, model, hi, hl, hr, nz);
    if (v0 <= 0) {
        *found = 1;
        return hi;
    }
    double a = hi;
    double advanced = 0;
    while (advanced < rp->max_advance) {
        const double b = a + rp->dstep;
        const double vb = qo_rk_site_velocity(i, n, dx, lt, f, model, b, hl, hr, nz);
        if (vb <= 0) {
            double lo = a, hicur = b;
            for (int k = 0; k < 60 && (hicur - lo) > rp->root_tol; ++k) {
                const double mid = 0.5 * (lo + hicur);
                const double vm = qo_rk_site_velocity(i, n, dx, lt, f, model, mid, hl, hr, nz);
                if (vm > 0)
                    lo = mid;
                else
                    hicur = mid;
            }
            *found = 1;
            return 0.5 * (lo + hicur);
        }
        a = b;
        advanced += rp->dstep;
    }
    *found = 0;
    return a;
}

/* rk_block, rosso_krauth.h:128-194 */
int qo_rk_block(double *h, int n, const qo_params *p, const qo_noise *nz,
                const qo_rk_params *rp, qo_rk_result *res) {
    memset(res, 0, sizeof(*res));
    if (n % 2 != 0) return -1;
    const double dx = p->physical_size / (double)n;
    const double lt = p->line_tension;
    const double f = p->driving_force;
    const int model = p->model;
    double *adv = (double *)calloc((size_t)n, sizeof(double));
    double mean_h0 = 0;
    for (int i = 0; i < n; ++i) mean_h0 += h[i];
    mean_h0 /= (double)n;
    double cum_adv = 0;
    for (int sweep = 0; sweep < rp->max_sweeps; ++sweep) {
        for (int color = 0; color < 2; ++color) {
            /* sites of one colour are independent (their neighbours are of the
             * other colour), so the threads give the serial loop's numbers */
#pragma omp parallel for schedule(dynamic, 16) if (n >= 512)
            for (int i = color; i < n; i += 2) {
                const int im = (i == 0) ? n - 1 : i - 1;
                const int ip = (i + 1 == n) ? 0 : i + 1;
                int found = 0;
                const double hnew = qo_rk_forward_zero(i, n, dx, lt, f, model, h[i],
                                                       h[im], h[ip], nz, rp, &found);
                adv[i] = hnew - h[i];
                h[i] = hnew;
            }
        }
        double total_adv = 0;
        for (int i = 0; i < n; ++i) total_adv += adv[i];
        cum_adv += total_adv;
        const double mean_adv = cum_adv / (double)n;
        res->sweeps = sweep + 1;
        res->total_advance = total_adv;
        res->mean_h = mean_h0 + mean_adv;
        if (mean_adv > rp->runaway) {
            res->runaway = 1;
            res->blocked = 0;
            free(adv);
            return 0;
        }
        if (total_adv < rp->sweep_tol) {
            res->blocked = 1;
            res->runaway = 0;
            free(adv);
            return 0;
        }
    }
    res->blocked = 0;
    res->runaway = 0;
    free(adv);
    return 0;
}

/* Force bisection for f_c. The reference only ramps (qew_runs.h:226-241) and
 * brackets f_c from above; the protocol used here is: start from a blocked
 * configuration h at f_lo and an unblocked force f_hi; repeatedly test the
 * midpoint force by rk_block restarted from the last BLOCKED configuration
 * (no-passing makes that the unique first blocked state ahead of it); a
 * blocked midpoint becomes the new f_lo and its configuration the new start,
 * anything else (runaway or timeout, as in the ramp) the new f_hi. Stop when
 * (f_hi - f_lo) <= rtol * f_hi or after max_steps. On return h holds the
 * blocked configuration at f_lo (the critical configuration) and
 * f_c = (f_lo + f_hi) / 2. */
int qo_depinning_bisect(double *h, int n, const qo_params *p,
                        const qo_noise *nz, const qo_rk_params *rp,
                        double f_lo, double f_hi, double rtol, int max_steps,
                        double *f_c, double *f_lo_out, double *f_hi_out,
                        int *n_blocks) {
    return qo_depinning_bisect_ex(h, n, p, nz, rp, f_lo, f_hi, rtol, max_steps, f_c,
                                  f_lo_out, f_hi_out, n_blocks, NULL, NULL);
}

/* The same, recording each block's verdict (0 blocked, 1 runaway, 2 neither:
 * max_sweeps reached) in verdicts[] (max_steps entries, may be NULL) and the
 * sweeps of every block in *sweeps (may be NULL). */
int qo_depinning_bisect_ex(double *h, int n, const qo_params *p,
                           const qo_noise *nz, const qo_rk_params *rp,
                           double f_lo, double f_hi, double rtol, int max_steps,
                           double *f_c, double *f_lo_out, double *f_hi_out,
                           int *n_blocks, int *verdicts, long *sweeps) {
    if (n % 2 != 0) return -1;
    if (sweeps) *sweeps = 0;
    double *work = (double *)malloc(sizeof(double) * (size_t)n);
    qo_params pp = *p;
    int steps = 0;
    while ((f_hi - f_lo) > rtol * f_hi && steps < max_steps) {
        const double fm = 0.5 * (f_lo + f_hi);
        memcpy(work, h, sizeof(double) * (size_t)n);
        pp.driving_force = fm;
        qo_rk_result r;
        qo_rk_block(work, n, &pp, nz, rp, &r);
        if (verdicts) verdicts[steps] = r.blocked ? 0 : (r.runaway ? 1 : 2);
        if (sweeps) *sweeps += r.sweeps;
        ++steps;
        if (r.blocked) {
            f_lo = fm;
            memcpy(h, work, sizeof(double) * (size_t)n);
        } else {
            f_hi = fm;
        }
    }
    free(work);
    *f_c = 0.5 * (f_lo + f_hi);
    *f_lo_out = f_lo;
    *f_hi_out = f_hi;
    *n_blocks = steps;
    return 0;
}

/* ======================================================================== */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and Box-Muller (1958)   */
/* ======================================================================== */

static void philox_round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k[0];
    const uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
}

static void philox4x32_10(uint32_t c[4], uint64_t seed) {
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        philox_round(c, k);
    }
}

/* Increment i of step `step`: block j = i/2 of counter (j, step) gives two
 * 53-bit uniforms u1 in (0,1], u2 in [0,1); Box-Muller
 * r = sqrt(-2 ln u1), z0 = r cos(2 pi u2), z1 = r sin(2 pi u2). */
static void philox_normals_impl(uint64_t seed, uint64_t step, int n, double *out, int par) {
    const double two_pi = 6.283185307179586476925286766559;
#pragma omp parallel for schedule(static) if (par)
    for (int j = 0; j < (n + 1) / 2; ++j) {
        uint32_t c[4] = {(uint32_t)j, 0u, (uint32_t)step, (uint32_t)(step >> 32)};
        philox4x32_10(c, seed);
        const uint64_t a = (((uint64_t)c[0] << 32) | c[1]) >> 11;
        const uint64_t b = (((uint64_t)c[2] << 32) | c[3]) >> 11;
        const double u1 = ((double)a + 1.0) * (1.0 / 9007199254740992.0);
        const double u2 = (double)b * (1.0 / 9007199254740992.0);
        const double r = sqrt(-2.0 * log(u1));
        const double ang = two_pi * u2;
        out[2 * j] = r * cos(ang);
        if (2 * j + 1 < n) out[2 * j + 1] = r * sin(ang);
    }
}

void qo_philox_normals(uint64_t seed, uint64_t step, int n, double *out) {
    philox_normals_impl(seed, step, n, out, 0);
}

/* LangevinDynamics::step (dynamics.h:34-64) with its own increments: the
 * Philox normals of (seed, step) drawn inside the step, as the reference
 * draws from its generator pool; par = 1 runs the gradient, the draws and
 * the update on all OpenMP threads (the timed CPU form). */
void qo_langevin_step_philox(double *h, int n, const qo_params *p, const qo_noise *nz,
                             double drift, double diff, uint64_t seed, uint64_t step,
                             double *grad, double *xi, int par) {
    qo_gradient_impl(h, n, p, nz, grad, par);
    const double a = drift, b = diff;
    if (b > 0) {
        philox_normals_impl(seed, step, n, xi, par);
#pragma omp parallel for schedule(static) if (par)
        for (int i = 0; i < n; ++i) h[i] += -a * grad[i] + b * xi[i];
    } else {
#pragma omp parallel for schedule(static) if (par)
        for (int i = 0; i < n; ++i) h[i] += -a * grad[i];
    }
}

void qo_omp_set_threads(int k) {
#ifdef _OPENMP
    omp_set_num_threads(k > 0 ? k : 1);
#else
    (void)k;
#endif
}
