/*
 * fdm_oracle.c -- FP64 CPU restatement of the reference FDM LLG path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA engine and the
 * timed CPU baseline. The product library never links or calls this code.
 * Each function names the reference code it follows (paths relative to the
 * mzrptu/fullmag tree).
 */
#include "fdm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define FO_MU0 (4.0 * M_PI * 1e-7) /* crates/fullmag-engine/src/lib.rs:37 */
#define FO_ASYMPTOTIC_DISTANCE 40  /* crates/fullmag-fdm-demag/src/newell.rs:231 */

int fo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void fo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------- */
/* Newell base functions: crates/fullmag-fdm-demag/src/newell.rs:21-131       */
/* ------------------------------------------------------------------------- */

double fo_newell_f(double x, double y, double z) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    if (r2 < 1e-300) return 0.0;
    const double r = sqrt(r2);
    double acc = (2.0 * x2 - y2 - z2) * r / 6.0;
    const double sxz = x2 + z2;
    if (sxz > 1e-300) {
        const double t = 2.0 * y * (y + r) / sxz;
        if (t > -1.0) acc += y * (z2 - x2) / 4.0 * log1p(t);
    }
    const double sxy = x2 + y2;
    if (sxy > 1e-300) {
        const double t = 2.0 * z * (z + r) / sxy;
        if (t > -1.0) acc += z * (y2 - x2) / 4.0 * log1p(t);
    }
    if (fabs(x) > 1e-300) acc -= x * y * z * atan(y * z / (x * r));
    return acc;
}

double fo_newell_g(double x, double y, double z) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    if (r2 < 1e-300) return 0.0;
    const double r = sqrt(r2);
    double acc = -x * y * r / 3.0;
    const double sxy = x2 + y2;
    if (sxy > 1e-300) {
        const double t = 2.0 * z * (z + r) / sxy;
        if (t > -1.0) acc += x * y * z * log1p(t) / 2.0;
    }
    const double syz = y2 + z2;
    if (syz > 1e-300) {
        const double t = 2.0 * x * (x + r) / syz;
        if (t > -1.0) acc += y * (3.0 * z2 - y2) * log1p(t) / 12.0;
    }
    const double sxz = x2 + z2;
    if (sxz > 1e-300) {
        const double t = 2.0 * y * (y + r) / sxz;
        if (t > -1.0) acc += x * (3.0 * z2 - x2) * log1p(t) / 12.0;
    }
    if (fabs(z) > 1e-300) acc -= z2 * z / 6.0 * atan(x * y / (z * r));
    if (fabs(y) > 1e-300) acc -= y2 * z / 2.0 * atan(x * z / (y * r));
    if (fabs(x) > 1e-300) acc -= x2 * z / 2.0 * atan(y * z / (x * r));
    return acc;
}

/* Kahan-Neumaier compensated sum (newell.rs:133-149). */
static double neumaier_sum(const double *v, int n) {
    double s = 0.0, c = 0.0;
    for (int i = 0; i < n; ++i) {
        const double t = s + v[i];
        if (fabs(s) >= fabs(v[i])) c += (s - t) + v[i];
        else c += (v[i] - t) + s;
        s = t;
    }
    return s + c;
}

/* 27-point second-difference stencil on a precomputed f or g table whose
 * entry (a,b,c) holds the value at signed offset (a-1, b-1, c-1)
 * (newell.rs:150-210). */
static double stencil27(int i, int j, int k, const double *t, int sx, int sy, double vol) {
    double terms[27];
    int n = 0;
    /* weight of offset (da,db,dc) with da,db,dc in {-1,0,1}:
     * product over axes of (2 if d==0 else -1) = 8, -4, 2, -1 as in the reference */
    for (int dc = -1; dc <= 1; ++dc)
        for (int db = -1; db <= 1; ++db)
            for (int da = -1; da <= 1; ++da) {
                const double wa = da == 0 ? 2.0 : -1.0;
                const double wb = db == 0 ? 2.0 : -1.0;
                const double wc = dc == 0 ? 2.0 : -1.0;
                const long idx = (long)(k + 1 + dc) * sy * sx + (long)(j + 1 + db) * sx + (i + 1 + da);
                terms[n++] = wa * wb * wc * t[idx];
            }
    return neumaier_sum(terms, 27) / (4.0 * M_PI * vol);
}

/* Point-dipole asymptotics (newell.rs:212-229). */
static double asym_diag(double x, double y, double z, double vol) {
    const double r2 = x * x + y * y + z * z, r = sqrt(r2), r3 = r2 * r;
    return (1.0 / r3 - 3.0 * x * x / (r3 * r2)) / (4.0 * M_PI) * vol;
}
static double asym_off(double x, double y, double z, double vol) {
    const double r2 = x * x + y * y + z * z, r = sqrt(r2), r5 = r2 * r2 * r;
    return -3.0 * x * y / (4.0 * M_PI * r5) * vol;
}

/* compute_newell_kernels (newell.rs:254-519). */
int fo_newell_kernels(int nx, int ny, int nz, double dx, double dy, double dz, double *out) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return -1;
    const int px = 2 * nx, py = 2 * ny, pz = 2 * nz;
    const long plen = (long)px * py * pz;
    const int sx = (nx < FO_ASYMPTOTIC_DISTANCE ? nx : FO_ASYMPTOTIC_DISTANCE) + 2;
    const int sy = (ny < FO_ASYMPTOTIC_DISTANCE ? ny : FO_ASYMPTOTIC_DISTANCE) + 2;
    const int sz = (nz < FO_ASYMPTOTIC_DISTANCE ? nz : FO_ASYMPTOTIC_DISTANCE) + 2;
    const long flen = (long)sx * sy * sz;
    double *tab = (double *)malloc(sizeof(double) * 6 * flen);
    if (!tab) return -2;
    double *fxx = tab, *fyy = tab + flen, *fzz = tab + 2 * flen;
    double *gxy = tab + 3 * flen, *gxz = tab + 4 * flen, *gyz = tab + 5 * flen;

#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < sz; ++c)
        for (int b = 0; b < sy; ++b)
            for (int a = 0; a < sx; ++a) {
                const double x = (a - 1) * dx, y = (b - 1) * dy, z = (c - 1) * dz;
                const long id = (long)c * sy * sx + (long)b * sx + a;
                fxx[id] = fo_newell_f(x, y, z);
                fyy[id] = fo_newell_f(y, x, z);
                fzz[id] = fo_newell_f(z, y, x);
                gxy[id] = fo_newell_g(x, y, z);
                gxz[id] = fo_newell_g(x, z, y);
                gyz[id] = fo_newell_g(y, z, x);
            }

    memset(out, 0, sizeof(double) * 6 * plen);
    double *nxx = out, *nyy = out + plen, *nzz = out + 2 * plen;
    double *nxy = out + 3 * plen, *nxz = out + 4 * plen, *nyz = out + 5 * plen;
    const double vol = dx * dy * dz;
    const int AD = FO_ASYMPTOTIC_DISTANCE;

#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double vxx, vyy, vzz, vxy, vxz, vyz;
                const long d2 = (long)i * i + (long)j * j + (long)k * k;
                if (i >= AD || j >= AD || k >= AD || d2 >= (long)AD * AD) {
                    const double x = i * dx, y = j * dy, z = k * dz;
                    vxx = asym_diag(x, y, z, vol);
                    vyy = asym_diag(y, x, z, vol);
                    vzz = asym_diag(z, y, x, vol);
                    vxy = asym_off(x, y, z, vol);
                    vxz = asym_off(x, z, y, vol);
                    vyz = asym_off(y, z, x, vol);
                } else {
                    vxx = stencil27(i, j, k, fxx, sx, sy, vol);
                    vyy = stencil27(i, j, k, fyy, sx, sy, vol);
                    vzz = stencil27(i, j, k, fzz, sx, sy, vol);
                    vxy = stencil27(i, j, k, gxy, sx, sy, vol);
                    vxz = stencil27(i, j, k, gxz, sx, sy, vol);
                    vyz = stencil27(i, j, k, gyz, sx, sy, vol);
                }
                /* octant placement with parity signs (newell.rs:393-425) */
                const int nxs = i == 0 ? 1 : 2, nys = j == 0 ? 1 : 2, nzs = k == 0 ? 1 : 2;
                for (int a = 0; a < nxs; ++a) {
                    const int ix = a == 0 ? i : px - i;
                    const double sxg = a == 0 ? 1.0 : -1.0;
                    for (int b = 0; b < nys; ++b) {
                        const int iy = b == 0 ? j : py - j;
                        const double syg = b == 0 ? 1.0 : -1.0;
                        for (int c = 0; c < nzs; ++c) {
                            const int iz = c == 0 ? k : pz - k;
                            const double szg = c == 0 ? 1.0 : -1.0;
                            const long p = (long)iz * py * px + (long)iy * px + ix;
                            nxx[p] = vxx;
                            nyy[p] = vyy;
                            nzz[p] = vzz;
                            nxy[p] = vxy * sxg * syg;
                            nxz[p] = vxz * sxg * szg;
                            nyz[p] = vyz * syg * szg;
                        }
                    }
                }
            }
    free(tab);
    return 0;
}

/* Open-boundary tensor at a signed offset (i, j, k) cells: first-octant value at the
 * absolute offsets (stencil on the f/g table, or the asymptotic form past the asymptotic
 * distance) with the parity signs of the octant placement (newell.rs:356-425). */
typedef struct {
    const double *tab;  /* six tables of sx*sy*sz values, offsets -1 .. s-2 */
    int sx, sy, sz;
    long flen;
    double dx, dy, dz, vol;
} newell_ctx;

static int newell_ctx_init(newell_ctx *c, long rx, long ry, long rz, double dx, double dy, double dz) {
    const int AD = FO_ASYMPTOTIC_DISTANCE;
    c->sx = (int)((rx < AD ? rx : AD) + 2);
    c->sy = (int)((ry < AD ? ry : AD) + 2);
    c->sz = (int)((rz < AD ? rz : AD) + 2);
    c->flen = (long)c->sx * c->sy * c->sz;
    c->dx = dx, c->dy = dy, c->dz = dz, c->vol = dx * dy * dz;
    double *t = (double *)malloc(sizeof(double) * 6 * (size_t)c->flen);
    if (!t) return -2;
    const long flen = c->flen;
#pragma omp parallel for schedule(dynamic)
    for (int cc = 0; cc < c->sz; ++cc)
        for (int b = 0; b < c->sy; ++b)
            for (int a = 0; a < c->sx; ++a) {
                const double x = (a - 1) * dx, y = (b - 1) * dy, z = (cc - 1) * dz;
                const long id = (long)cc * c->sy * c->sx + (long)b * c->sx + a;
                t[id] = fo_newell_f(x, y, z);
                t[flen + id] = fo_newell_f(y, x, z);
                t[2 * flen + id] = fo_newell_f(z, y, x);
                t[3 * flen + id] = fo_newell_g(x, y, z);
                t[4 * flen + id] = fo_newell_g(x, z, y);
                t[5 * flen + id] = fo_newell_g(y, z, x);
            }
    c->tab = t;
    return 0;
}

static void newell_at(const newell_ctx *c, long i, long j, long k, double v[6]) {
    const long ai = i < 0 ? -i : i, aj = j < 0 ? -j : j, ak = k < 0 ? -k : k;
    const long AD = FO_ASYMPTOTIC_DISTANCE;
    if (ai >= AD || aj >= AD || ak >= AD || ai * ai + aj * aj + ak * ak >= AD * AD) {
        const double x = ai * c->dx, y = aj * c->dy, z = ak * c->dz;
        v[0] = asym_diag(x, y, z, c->vol);
        v[1] = asym_diag(y, x, z, c->vol);
        v[2] = asym_diag(z, y, x, c->vol);
        v[3] = asym_off(x, y, z, c->vol);
        v[4] = asym_off(x, z, y, c->vol);
        v[5] = asym_off(y, z, x, c->vol);
    } else {
        for (int q = 0; q < 6; ++q) v[q] = stencil27((int)ai, (int)aj, (int)ak, c->tab + q * c->flen, c->sx, c->sy, c->vol);
    }
    const double sx = i < 0 ? -1.0 : 1.0, sy = j < 0 ? -1.0 : 1.0, sz = k < 0 ? -1.0 : 1.0;
    v[3] *= sx * sy;
    v[4] *= sx * sz;
    v[5] *= sy * sz;
}

int fo_periodic_newell_kernels(int nx, int ny, int nz, double dx, double dy, double dz, const int32_t periodic[3],
                               const uint32_t images[3], double *out) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return -1;
    const int n3[3] = {nx, ny, nz};
    int pd[3], im[3];
    long reach[3];
    for (int a = 0; a < 3; ++a) {
        pd[a] = periodic[a] ? n3[a] : 2 * n3[a];
        im[a] = periodic[a] ? (int)images[a] : 0;
        reach[a] = (long)n3[a] * (1 + 2 * (long)im[a]);
    }
    newell_ctx c;
    if (newell_ctx_init(&c, reach[0], reach[1], reach[2], dx, dy, dz)) return -2;
    const long plen = (long)pd[0] * pd[1] * pd[2];
#pragma omp parallel for schedule(dynamic)
    for (long id = 0; id < plen; ++id) {
        const long i = id % pd[0], j = (id / pd[0]) % pd[1], k = id / ((long)pd[0] * pd[1]);
        const long idx3[3] = {i, j, k};
        long off[3] = {0, 0, 0};
        int live = 1;
        for (int a = 0; a < 3; ++a) {
            /* open axis: index i < n is the offset i, i > n the offset i - 2n, i == n empty */
            if (periodic[a]) off[a] = idx3[a];
            else if (idx3[a] < n3[a]) off[a] = idx3[a];
            else if (idx3[a] > n3[a]) off[a] = idx3[a] - pd[a];
            else live = 0;
        }
        double acc[6] = {0, 0, 0, 0, 0, 0};
        if (live)
            for (int mz = -im[2]; mz <= im[2]; ++mz)
                for (int my = -im[1]; my <= im[1]; ++my)
                    for (int mx = -im[0]; mx <= im[0]; ++mx) {
                        double v[6];
                        newell_at(&c, off[0] + (long)mx * nx, off[1] + (long)my * ny, off[2] + (long)mz * nz, v);
                        for (int q = 0; q < 6; ++q) acc[q] += v[q];
                    }
        for (int q = 0; q < 6; ++q) out[q * plen + id] = acc[q];
    }
    free((void *)c.tab);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Mixed-radix FFT (own implementation; stands in for rustfft 6.4.1)          */
/* ------------------------------------------------------------------------- */

typedef struct fft_plan {
    int n;
    int nf;
    int f[64];
    int maxp;
    double *w; /* w[2e], w[2e+1] = cos, -sin of 2*pi*e/n */
    /* lengths with a prime factor above 61: Bluestein's chirp-z algorithm (Bluestein 1970)
     * through a power-of-two transform of length M >= 2n - 1, the way rustfft handles such
     * lengths: X_k = c_k sum_j (x_j c_j) conj(c_{k-j}), c_j = e^{-i pi j^2 / n} */
    int blue, M;
    struct fft_plan *sub;
    double *chirp; /* c_j, j < n */
    double *bhat;  /* FFT_M of conj(c_j) wrapped to j in (-n, n) */
} fft_plan;

static void fft_rec(const struct fft_plan *P, const double *in, long is, double *out, int n, int fi, int inv, double *tmp);

static int plan_init(fft_plan *P, int n) {
    P->n = n;
    P->nf = 0;
    P->maxp = 4;
    P->blue = 0;
    P->M = 0;
    P->sub = NULL;
    P->chirp = P->bhat = NULL;
    int m = n;
    while (m % 4 == 0) { P->f[P->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { P->f[P->nf++] = 2; m /= 2; }
    for (int q = 3; (long)q * q <= m; q += 2)
        while (m % q == 0) { P->f[P->nf++] = q; m /= q; }
    if (m > 1) P->f[P->nf++] = m;
    for (int i = 0; i < P->nf; ++i)
        if (P->f[i] > P->maxp) P->maxp = P->f[i];
    P->w = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    if (!P->w) return -1;
    for (int e = 0; e < n; ++e) {
        const double ang = 2.0 * M_PI * (double)e / (double)n;
        P->w[2 * e] = cos(ang);
        P->w[2 * e + 1] = -sin(ang);
    }
    if (P->maxp > 61) {
        P->blue = 1;
        int M = 1;
        while (M < 2 * n - 1) M <<= 1;
        P->M = M;
        P->sub = (fft_plan *)calloc(1, sizeof(fft_plan));
        P->chirp = (double *)malloc(sizeof(double) * 2 * (size_t)n);
        P->bhat = (double *)calloc(2 * (size_t)M, sizeof(double));
        double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)M);
        double *ftmp = (double *)malloc(sizeof(double) * 8);
        if (!P->sub || !P->chirp || !P->bhat || !tmp || !ftmp || plan_init(P->sub, M)) {
            free(tmp);
            free(ftmp);
            return -1;
        }
        for (long j = 0; j < n; ++j) {
            /* j^2 mod 2n keeps the angle exact */
            const long q = (j * j) % (2L * n);
            const double ang = M_PI * (double)q / (double)n;
            P->chirp[2 * j] = cos(ang);
            P->chirp[2 * j + 1] = -sin(ang);
        }
        for (long j = 0; j < n; ++j) {
            const double br = P->chirp[2 * j], bi = -P->chirp[2 * j + 1];
            P->bhat[2 * j] = br;
            P->bhat[2 * j + 1] = bi;
            if (j > 0) {
                P->bhat[2 * (M - j)] = br;
                P->bhat[2 * (M - j) + 1] = bi;
            }
        }
        memcpy(tmp, P->bhat, sizeof(double) * 2 * (size_t)M);
        fft_rec(P->sub, tmp, 1, P->bhat, M, 0, 0, ftmp);
        free(tmp);
        free(ftmp);
    }
    return 0;
}

static void plan_free(fft_plan *P) {
    free(P->w);
    P->w = NULL;
    if (P->sub) {
        plan_free(P->sub);
        free(P->sub);
        P->sub = NULL;
    }
    free(P->chirp);
    free(P->bhat);
    P->chirp = P->bhat = NULL;
}

/* Bluestein transform of x (length n, contiguous) into out; the inverse (unnormalised,
 * conjugate kernel) as conj(forward(conj x)).  work holds 4 M doubles. */
static void fft_blue(const fft_plan *P, const double *x, double *out, int inv, double *work, double *tmp) {
    const int n = P->n, M = P->M;
    const double sg = inv ? -1.0 : 1.0;
    double *a = work, *A = work + 2 * (size_t)M;
    memset(a, 0, sizeof(double) * 2 * (size_t)M);
    for (int j = 0; j < n; ++j) {
        const double xr = x[2 * j], xi = sg * x[2 * j + 1];
        const double cr = P->chirp[2 * j], ci = P->chirp[2 * j + 1];
        a[2 * j] = xr * cr - xi * ci;
        a[2 * j + 1] = xr * ci + xi * cr;
    }
    fft_rec(P->sub, a, 1, A, M, 0, 0, tmp);
    for (int k = 0; k < M; ++k) {
        const double ar = A[2 * k], ai = A[2 * k + 1], br = P->bhat[2 * k], bi = P->bhat[2 * k + 1];
        A[2 * k] = ar * br - ai * bi;
        A[2 * k + 1] = ar * bi + ai * br;
    }
    fft_rec(P->sub, A, 1, a, M, 0, 1, tmp);
    const double inv_m = 1.0 / (double)M;
    for (int k = 0; k < n; ++k) {
        const double vr = a[2 * k] * inv_m, vi = a[2 * k + 1] * inv_m;
        const double cr = P->chirp[2 * k], ci = P->chirp[2 * k + 1];
        out[2 * k] = vr * cr - vi * ci;
        out[2 * k + 1] = sg * (vr * ci + vi * cr);
    }
}

/* Decimation in time: X[k + q m] = sum_r W_p^{rq} W_n^{rk} DFT_m(x[r::p])[k]. */
static void fft_rec(const fft_plan *P, const double *in, long is, double *out, int n, int fi,
                    int inv, double *tmp) {
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    const int p = P->f[fi];
    const int m = n / p;
    for (int r = 0; r < p; ++r) fft_rec(P, in + 2 * r * is, is * p, out + 2 * (long)r * m, m, fi + 1, inv, tmp);
    const long N = P->n;
    const long tws = N / n;
    const double sg = inv ? -1.0 : 1.0; /* conjugate twiddles for the inverse */
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            const double re = out[2 * ((long)r * m + k)], im = out[2 * ((long)r * m + k) + 1];
            const long e = ((long)r * k % n) * tws;
            const double wr = P->w[2 * e], wi = sg * P->w[2 * e + 1];
            tmp[2 * r] = re * wr - im * wi;
            tmp[2 * r + 1] = re * wi + im * wr;
        }
        if (p == 2) {
            out[2 * k] = tmp[0] + tmp[2];
            out[2 * k + 1] = tmp[1] + tmp[3];
            out[2 * (k + m)] = tmp[0] - tmp[2];
            out[2 * (k + m) + 1] = tmp[1] - tmp[3];
        } else if (p == 4) {
            const double a0r = tmp[0] + tmp[4], a0i = tmp[1] + tmp[5];
            const double a1r = tmp[0] - tmp[4], a1i = tmp[1] - tmp[5];
            const double b0r = tmp[2] + tmp[6], b0i = tmp[3] + tmp[7];
            const double dr = tmp[2] - tmp[6], di = tmp[3] - tmp[7];
            /* forward: b1 = -i*d ; inverse: b1 = +i*d */
            const double b1r = inv ? -di : di;
            const double b1i = inv ? dr : -dr;
            out[2 * k] = a0r + b0r;
            out[2 * k + 1] = a0i + b0i;
            out[2 * (k + 2 * m)] = a0r - b0r;
            out[2 * (k + 2 * m) + 1] = a0i - b0i;
            out[2 * (k + m)] = a1r + b1r;
            out[2 * (k + m) + 1] = a1i + b1i;
            out[2 * (k + 3 * m)] = a1r - b1r;
            out[2 * (k + 3 * m) + 1] = a1i - b1i;
        } else {
            const long pstep = N / p;
            for (int q = 0; q < p; ++q) {
                double sr = 0.0, si = 0.0;
                for (int r = 0; r < p; ++r) {
                    const long e = ((long)r * q % p) * pstep;
                    const double wr = P->w[2 * e], wi = sg * P->w[2 * e + 1];
                    sr += tmp[2 * r] * wr - tmp[2 * r + 1] * wi;
                    si += tmp[2 * r] * wi + tmp[2 * r + 1] * wr;
                }
                out[2 * (k + (long)q * m)] = sr;
                out[2 * (k + (long)q * m) + 1] = si;
            }
        }
    }
}

/* Transform one line gathered with a stride (in complex elements). */
static void fft_line(const fft_plan *P, double *base, long stride, int inv, double *lin, double *lout,
                     double *tmp) {
    const int n = P->n;
    for (int i = 0; i < n; ++i) {
        lin[2 * i] = base[2 * i * stride];
        lin[2 * i + 1] = base[2 * i * stride + 1];
    }
    if (P->blue) fft_blue(P, lin, lout, inv, tmp + 8, tmp);
    else fft_rec(P, lin, 1, lout, n, 0, inv, tmp);
    for (int i = 0; i < n; ++i) {
        base[2 * i * stride] = lout[2 * i];
        base[2 * i * stride + 1] = lout[2 * i + 1];
    }
}

int fo_fft1d(double *data, int n, int inverse) {
    if (n <= 0) return -1;
    fft_plan P;
    if (plan_init(&P, n)) return -2;
    double *buf = (double *)malloc(sizeof(double) * (4 * (size_t)n + 2 * (size_t)P.maxp + 8 + 4 * (size_t)P.M));
    if (!buf) { plan_free(&P); return -2; }
    fft_line(&P, data, 1, inverse, buf, buf + 2 * n, buf + 4 * n);
    free(buf);
    plan_free(&P);
    return 0;
}

/* x, then y, then z lines, as fft3_core (crates/fullmag-engine/src/fdm_fft.rs:445-573). */
int fo_fft3d(double *data, int px, int py, int pz, int inverse) {
    fft_plan Px, Py, Pz;
    if (plan_init(&Px, px) || plan_init(&Py, py) || plan_init(&Pz, pz)) return -2;
    int maxn = px > py ? px : py;
    if (pz > maxn) maxn = pz;
    int maxp = Px.maxp > Py.maxp ? Px.maxp : Py.maxp;
    if (Pz.maxp > maxp) maxp = Pz.maxp;
    int maxm = Px.M > Py.M ? Px.M : Py.M;
    if (Pz.M > maxm) maxm = Pz.M;
    maxp += 4 + 2 * maxm; /* the tmp area also holds Bluestein's work arrays */
    const long sxy = (long)px * py;
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * (4 * (size_t)maxn + 2 * (size_t)maxp));
#pragma omp for schedule(static)
        for (long row = 0; row < (long)py * pz; ++row)
            fft_line(&Px, data + 2 * row * px, 1, inverse, buf, buf + 2 * maxn, buf + 4 * maxn);
#pragma omp for schedule(static)
        for (long col = 0; col < (long)px * pz; ++col) {
            const long z = col / px, x = col % px;
            fft_line(&Py, data + 2 * (z * sxy + x), px, inverse, buf, buf + 2 * maxn, buf + 4 * maxn);
        }
        if (pz > 1) {
#pragma omp for schedule(static)
            for (long col = 0; col < sxy; ++col)
                fft_line(&Pz, data + 2 * col, sxy, inverse, buf, buf + 2 * maxn, buf + 4 * maxn);
        }
        free(buf);
    }
    plan_free(&Px);
    plan_free(&Py);
    plan_free(&Pz);
    return 0;
}

/* compute_newell_kernel_spectra / _thin_film_2d (fdm_fft.rs:334-437). */
int fo_newell_spectra(int nx, int ny, int nz, double dx, double dy, double dz, int thin_film_2d,
                      double *out) {
    if (thin_film_2d && nz != 1) return -1;
    const int px = 2 * nx, py = 2 * ny, pz = 2 * nz;
    const long plen3 = (long)px * py * pz;
    double *real = (double *)malloc(sizeof(double) * 6 * plen3);
    if (!real) return -2;
    int rc = fo_newell_kernels(nx, ny, nz, dx, dy, dz, real);
    if (rc) { free(real); return rc; }
    const long P = thin_film_2d ? (long)px * py : plen3;
    for (int c = 0; c < 6; ++c) {
        double *o = out + 2 * P * c;
        const double *r = real + plen3 * c;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < P; ++i) {
            o[2 * i] = r[i]; /* thin film: the z = 0 plane is the first px*py values */
            o[2 * i + 1] = 0.0;
        }
        rc = fo_fft3d(o, px, py, thin_film_2d ? 1 : pz, 0);
        if (rc) break;
    }
    free(real);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Problem: fields, RHS, integrators                                          */
/* ------------------------------------------------------------------------- */

struct fo_problem {
    fo_params p;
    long n;
    uint8_t *mask;
    double *m; /* AoS current state */
    double t;
    double step;
    int px, py, pz;
    long P;
    double *kern[6]; /* complex spectra (interleaved), full padded grid */
    double *bm[3];   /* complex M */
    double *bh[3];   /* complex H */
    double u[3], c1[3], c2[3], c3[3];
    /* integrator buffers (AoS) */
    double *m0, *mst, *heff, *hscr, *k[7], *fsal;
    int fsal_valid;
    /* ABM3 history f_n, f_{n-1}, f_{n-2} and its start-up state (llg_abm3_fp32.cu:115-266) */
    double *abm_h[3];
    int abm_startup;
    double abm_last_dt;
    /* torque prefactors (api.cpp:250-300, context.hpp:321-339) */
    int has_zl, has_slon, has_sot;
    double zl_u[3], slon_pf, slon_P, sot_amp, sot_s[3];
    double *kmap[5]; /* per-cell Ku1 Ku2 Kc1 Kc2 Kc3 or NULL */
    double *h_oe;    /* Oersted field for I = 1 A (AoS) or NULL */
    double oe_scale; /* current I(t) of the evaluations in progress */
    /* thermal field: step counter (advanced once per completed step), the counter and
     * amplitude of the evaluations in progress, and the dt the amplitude is taken at */
    uint64_t th_step, th_eval;
    double th_sigma, th_dt;
    double *hmap; /* optional per-cell applied field (AoS, A/m) */
    uint32_t *region; /* optional region ids */
    double *lut;      /* FO_MAX_REGIONS^2 inter-region exchange stiffness (J/m) when region != NULL */
    /* boundary correction (copies of the plan arrays) */
    double *phi, *face[6], *delta[6];
    int32_t *ctidx, *csidx;
    double *ctensor;
};

/* a cell takes part when the mask allows it and, with a boundary tier, its volume
 * fraction is positive */
static inline int active(const fo_problem *pr, long i) {
    return (pr->mask == NULL || pr->mask[i] != 0) && (pr->p.boundary_tier == 0 || pr->phi[i] > 0.0);
}
static inline double phi_w(const fo_problem *pr, long i) { return pr->p.boundary_tier > 0 ? pr->phi[i] : 1.0; }

static void norm3(const double *a, double *o) {
    double n = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (n < 1e-30) n = 1e-30;
    o[0] = a[0] / n;
    o[1] = a[1] / n;
    o[2] = a[2] / n;
}

static double *dalloc(long n) { return (double *)calloc((size_t)n, sizeof(double)); }

void fo_destroy(fo_problem *pr) {
    if (!pr) return;
    free(pr->mask);
    free(pr->m);
    for (int c = 0; c < 6; ++c) free(pr->kern[c]);
    for (int c = 0; c < 3; ++c) { free(pr->bm[c]); free(pr->bh[c]); }
    free(pr->m0); free(pr->mst); free(pr->heff); free(pr->hscr); free(pr->fsal); free(pr->hmap);
    free(pr->region); free(pr->lut);
    for (int s = 0; s < 7; ++s) free(pr->k[s]);
    for (int s = 0; s < 3; ++s) free(pr->abm_h[s]);
    for (int s = 0; s < 5; ++s) free(pr->kmap[s]);
    free(pr->h_oe);
    free(pr->phi);
    for (int q = 0; q < 6; ++q) { free(pr->face[q]); free(pr->delta[q]); }
    free(pr->ctidx); free(pr->csidx); free(pr->ctensor);
    free(pr);
}

static double *dcopy(const double *src, long n) {
    if (!src) return NULL;
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(d, src, sizeof(double) * (size_t)n);
    return d;
}

/* A new state or field invalidates the FSAL derivative and the ABM3 history. */
static void invalidate_history(fo_problem *pr) {
    pr->fsal_valid = 0;
    pr->abm_startup = 0;
    pr->abm_last_dt = 0.0;
}

fo_problem *fo_create(const fo_params *p, const double *m0_aos) {
    if (!p || p->nx <= 0 || p->ny <= 0 || p->nz <= 0) return NULL;
    fo_problem *pr = (fo_problem *)calloc(1, sizeof(fo_problem));
    if (!pr) return NULL;
    pr->p = *p;
    pr->th_dt = 1e-13;
    pr->p.active_mask = NULL;
    pr->p.region_mask = NULL;
    pr->p.exchange_lut = NULL;
    {
        const double *src[5] = {p->ku1_field, p->ku2_field, p->kc1_field, p->kc2_field, p->kc3_field};
        const long nc = (long)p->nx * p->ny * p->nz;
        for (int k = 0; k < 5; ++k)
            if (src[k]) {
                pr->kmap[k] = (double *)malloc(sizeof(double) * (size_t)nc);
                memcpy(pr->kmap[k], src[k], sizeof(double) * (size_t)nc);
            }
        pr->p.ku1_field = pr->p.ku2_field = pr->p.kc1_field = pr->p.kc2_field = pr->p.kc3_field = NULL;
    }
    if (p->has_oersted && p->oersted_radius > 0.0) {
        /* field of a z-directed cylinder for I = 1 A at the cell centres: H_phi = r / (2 pi R^2)
         * inside, 1 / (2 pi r) outside, zero on the axis (context.cu:844-905) */
        const long nc = (long)p->nx * p->ny * p->nz;
        const double R = p->oersted_radius, cx = p->oersted_center[0], cy = p->oersted_center[1];
        pr->h_oe = dalloc(3 * nc);
        for (long i = 0; i < nc; ++i) {
            const long ix = i % p->nx, iy = (i / p->nx) % p->ny;
            const double ddx = (ix + 0.5) * p->dx - cx, ddy = (iy + 0.5) * p->dy - cy;
            const double r = sqrt(ddx * ddx + ddy * ddy);
            if (r < 1e-30) continue;
            const double hphi = r < R ? r / (2.0 * M_PI * R * R) : 1.0 / (2.0 * M_PI * r);
            pr->h_oe[3 * i] = -hphi * ddy / r;
            pr->h_oe[3 * i + 1] = hphi * ddx / r;
        }
    }
    pr->n = (long)p->nx * p->ny * p->nz;
    const long n3 = 3 * pr->n;
    pr->phi = dcopy(p->volume_fraction, pr->n);
    for (int q = 0; q < 6; ++q) {
        pr->face[q] = dcopy(p->face[q], pr->n);
        pr->delta[q] = dcopy(p->delta[q], pr->n);
    }
    if (p->boundary_tier > 0 && (!pr->phi || (p->boundary_tier == 1 && !pr->face[0]) || (p->boundary_tier == 2 && !pr->delta[0]))) {
        fo_destroy(pr);
        return NULL;
    }
    if (p->corr_targets > 0) {
        const long ns = (long)p->corr_targets * p->corr_stencil;
        pr->ctidx = (int32_t *)malloc(sizeof(int32_t) * p->corr_targets);
        memcpy(pr->ctidx, p->corr_target_idx, sizeof(int32_t) * p->corr_targets);
        pr->csidx = (int32_t *)malloc(sizeof(int32_t) * (size_t)ns);
        memcpy(pr->csidx, p->corr_source_idx, sizeof(int32_t) * (size_t)ns);
        pr->ctensor = dcopy(p->corr_tensor, 6 * ns);
    }
    pr->p.volume_fraction = pr->phi;
    pr->p.corr_target_idx = NULL;
    pr->p.corr_source_idx = NULL;
    pr->p.corr_tensor = NULL;
    for (int q = 0; q < 6; ++q) pr->p.face[q] = pr->p.delta[q] = NULL;
    if (p->active_mask) {
        pr->mask = (uint8_t *)malloc((size_t)pr->n);
        memcpy(pr->mask, p->active_mask, (size_t)pr->n);
    }
    if (p->region_mask) {  /* api.cpp:405-420: default table A on the diagonal */
        pr->region = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)pr->n);
        memcpy(pr->region, p->region_mask, sizeof(uint32_t) * (size_t)pr->n);
        pr->lut = dalloc((long)FO_MAX_REGIONS * FO_MAX_REGIONS);
        if (p->exchange_lut) memcpy(pr->lut, p->exchange_lut, sizeof(double) * FO_MAX_REGIONS * FO_MAX_REGIONS);
        else for (int r = 0; r < FO_MAX_REGIONS; ++r) pr->lut[r * FO_MAX_REGIONS + r] = p->a_ex;
    }
    pr->m = dalloc(n3);
    pr->m0 = dalloc(n3); pr->mst = dalloc(n3); pr->heff = dalloc(n3); pr->hscr = dalloc(n3);
    pr->fsal = dalloc(n3);
    for (int s = 0; s < 7; ++s) pr->k[s] = dalloc(n3);
    if (p->integrator == 3)
        for (int s = 0; s < 3; ++s) pr->abm_h[s] = dalloc(n3);
    {
        const double MU_B = 9.274009994e-24, E_CH = 1.60217662e-19, HBAR = 1.054571817e-34;
        const double *j = p->current_density;
        const int has_j = j[0] != 0.0 || j[1] != 0.0 || j[2] != 0.0;
        pr->has_zl = has_j && p->stt_degree > 0.0 && p->ms > 0.0;
        if (pr->has_zl) {
            const double b = p->stt_degree * MU_B / (E_CH * p->ms * (1.0 + p->stt_beta * p->stt_beta));
            for (int c = 0; c < 3; ++c) pr->zl_u[c] = b * j[c];
        }
        const double p2 = p->stt_p[0] * p->stt_p[0] + p->stt_p[1] * p->stt_p[1] + p->stt_p[2] * p->stt_p[2];
        pr->has_slon = p2 > 0.0 && p->stt_lambda > 0.0 && has_j && p->ms > 0.0 && p->dz > 0.0;
        if (pr->has_slon) {
            const double js = sqrt(j[0] * j[0] + j[1] * j[1] + j[2] * j[2]);
            pr->slon_pf = js * HBAR / (2.0 * E_CH * FO_MU0 * p->ms * p->dz);
            pr->slon_P = p->stt_degree > 0.0 ? p->stt_degree : 1.0;
        }
        const double t = p->sot_thickness > 0.0 ? p->sot_thickness : 1.0e-9;
        pr->has_sot = p->has_sot && p->ms > 0.0;
        if (pr->has_sot) {
            const double *sg = p->sot_sigma;
            const double len = sqrt(sg[0] * sg[0] + sg[1] * sg[1] + sg[2] * sg[2]);
            const double inv = len > 1e-30 ? 1.0 / len : 0.0;
            for (int c = 0; c < 3; ++c) pr->sot_s[c] = sg[c] * inv;
            pr->sot_amp = fabs(p->sot_je) * HBAR / (2.0 * E_CH * FO_MU0 * p->ms * t);
        }
    }
    norm3(p->u_axis, pr->u);
    norm3(p->c1, pr->c1);
    norm3(p->c2, pr->c2);
    pr->c3[0] = pr->c1[1] * pr->c2[2] - pr->c1[2] * pr->c2[1];
    pr->c3[1] = pr->c1[2] * pr->c2[0] - pr->c1[0] * pr->c2[2];
    pr->c3[2] = pr->c1[0] * pr->c2[1] - pr->c1[1] * pr->c2[0];
    const int any_periodic = p->periodic[0] || p->periodic[1] || p->periodic[2];
    if (p->enable_demag && any_periodic) {
        /* FftWorkspace::new_with_boundary (fdm_fft.rs:140-233): periodic axes unpadded, the
         * truncated image-sum tensor transformed by the full complex 3-D FFT */
        pr->px = p->periodic[0] ? p->nx : 2 * p->nx;
        pr->py = p->periodic[1] ? p->ny : 2 * p->ny;
        pr->pz = p->periodic[2] ? p->nz : 2 * p->nz;
        pr->P = (long)pr->px * pr->py * pr->pz;
        double *real = dalloc(6 * pr->P);
        if (!real || fo_periodic_newell_kernels(p->nx, p->ny, p->nz, p->dx, p->dy, p->dz, p->periodic, p->image_counts, real)) {
            free(real);
            fo_destroy(pr);
            return NULL;
        }
        for (int c = 0; c < 6; ++c) {
            pr->kern[c] = dalloc(2 * pr->P);
            for (long i = 0; i < pr->P; ++i) pr->kern[c][2 * i] = real[c * pr->P + i];
            fo_fft3d(pr->kern[c], pr->px, pr->py, pr->pz, 0);
        }
        free(real);
        for (int c = 0; c < 3; ++c) { pr->bm[c] = dalloc(2 * pr->P); pr->bh[c] = dalloc(2 * pr->P); }
    } else if (p->enable_demag) {
        pr->px = 2 * p->nx; pr->py = 2 * p->ny; pr->pz = 2 * p->nz;
        pr->P = (long)pr->px * pr->py * pr->pz;
        double *sp = dalloc(12 * pr->P);
        if (!sp || fo_newell_spectra(p->nx, p->ny, p->nz, p->dx, p->dy, p->dz, 0, sp)) {
            free(sp);
            fo_destroy(pr);
            return NULL;
        }
        for (int c = 0; c < 6; ++c) {
            pr->kern[c] = dalloc(2 * pr->P);
            memcpy(pr->kern[c], sp + 2 * pr->P * c, sizeof(double) * 2 * pr->P);
        }
        free(sp);
        for (int c = 0; c < 3; ++c) { pr->bm[c] = dalloc(2 * pr->P); pr->bh[c] = dalloc(2 * pr->P); }
    }
    if (m0_aos) fo_set_m(pr, m0_aos);
    return pr;
}

int fo_set_m(fo_problem *pr, const double *m_aos) {
    for (long i = 0; i < pr->n; ++i)
        for (int c = 0; c < 3; ++c) pr->m[3 * i + c] = active(pr, i) ? m_aos[3 * i + c] : 0.0;
    invalidate_history(pr);
    return 0;
}

int fo_get_m(const fo_problem *pr, double *m_aos) {
    memcpy(m_aos, pr->m, sizeof(double) * 3 * pr->n);
    return 0;
}

/* Per-cell applied field added to H_eff at active cells (the field map of the
 * adjoint entry points of the engine); NULL removes it. */
int fo_set_field_map(fo_problem *pr, const double *h_aos) {
    free(pr->hmap);
    pr->hmap = NULL;
    if (h_aos) {
        pr->hmap = dalloc(3 * pr->n);
        for (long i = 0; i < pr->n; ++i)
            for (int c = 0; c < 3; ++c) pr->hmap[3 * i + c] = active(pr, i) ? h_aos[3 * i + c] : 0.0;
    }
    invalidate_history(pr);
    return 0;
}

/* exchange_field_add_into (fdm_fields.rs:445-527), Neumann clamp (fdm_types.rs:126-132). */
/* x-, x+, y-, y+, z-, z+ neighbours of cell i: clamped to the cell on an open axis
 * (Neumann), wrapped around on a periodic one (neighbor_index, fdm_types.rs:126-132). */
static void axis_neighbours(const fo_params *p, long i, long nb[6]) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
    const long sxy = (long)nx * ny;
    nb[0] = x > 0 ? i - 1 : (p->periodic[0] ? i + nx - 1 : i);
    nb[1] = x < nx - 1 ? i + 1 : (p->periodic[0] ? i - (nx - 1) : i);
    nb[2] = y > 0 ? i - nx : (p->periodic[1] ? i + sxy - nx : i);
    nb[3] = y < ny - 1 ? i + nx : (p->periodic[1] ? i - sxy + nx : i);
    nb[4] = z > 0 ? i - sxy : (p->periodic[2] ? i + sxy * (nz - 1) : i);
    nb[5] = z < nz - 1 ? i + sxy : (p->periodic[2] ? i - sxy * (nz - 1) : i);
}

static void exchange_add(const fo_problem *pr, const double *m, double *h) {
    const fo_params *p = &pr->p;
    const double pref = 2.0 * p->a_ex / (FO_MU0 * p->ms);
    const double ix2 = 1.0 / (p->dx * p->dx), iy2 = 1.0 / (p->dy * p->dy), iz2 = 1.0 / (p->dz * p->dz);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        if (!active(pr, i)) continue;
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
        long nb[6];
        axis_neighbours(p, i, nb);
        for (int q = 0; q < 6; ++q)
            if (!active(pr, nb[q])) nb[q] = i;
        if (p->boundary_tier > 0) {
            /* T0: 2/(mu0 Ms phi_eff) sum_faces f A_ij (m_j - m_i)/d^2; T1: the same with
             * 2 A_ij / (d (d + delta_opposite)) per face and neighbours with m_j = 0 left out;
             * phi_eff = max(phi, phi_floor).  A_ij = A without regions (entering once). */
            const long off[6] = {1, -1, nx, -(long)nx, (long)nx * ny, -(long)nx * ny};
            const int has[6] = {x + 1 < nx, x > 0, y + 1 < ny, y > 0, z + 1 < nz, z > 0};
            const double d[6] = {p->dx, p->dx, p->dy, p->dy, p->dz, p->dz};
            double acc[3] = {0.0, 0.0, 0.0};
            for (int q = 0; q < 6; ++q) {
                if (q >= 4 && nz <= 1) continue;
                if (!has[q]) continue;
                const long j = i + off[q];
                const double A = pr->region ? pr->lut[pr->region[i] * FO_MAX_REGIONS + pr->region[j]] : p->a_ex;
                double w;
                if (p->boundary_tier == 1) {
                    const double f = pr->face[q][i];
                    if (!(f > 0.0)) continue;
                    w = A * f / (d[q] * d[q]);
                } else {
                    const double dsel = fmax(pr->delta[q][i], p->delta_min), dopp = fmax(pr->delta[q ^ 1][i], p->delta_min);
                    if (!(dsel > 0.0)) continue;
                    if (m[3 * j] == 0.0 && m[3 * j + 1] == 0.0 && m[3 * j + 2] == 0.0) continue;
                    w = A * 2.0 / (d[q] * (d[q] + dopp));
                }
                for (int c = 0; c < 3; ++c) acc[c] += w * (m[3 * j + c] - m[3 * i + c]);
            }
            const double s = 2.0 / (FO_MU0 * p->ms * fmax(pr->phi[i], p->phi_floor));
            for (int c = 0; c < 3; ++c) h[3 * i + c] += s * acc[c];
            continue;
        }
        if (pr->region) {  /* exchange_fp32.cu:48-104: 2/(mu0 Ms) sum_q A[r_i][r_q] (m_q - m_i)/d^2 */
            const double w[6] = {ix2, ix2, iy2, iy2, iz2, iz2};
            const double s = 2.0 / (FO_MU0 * p->ms);
            const uint32_t rc = pr->region[i];
            for (int c = 0; c < 3; ++c) {
                const double mc = m[3 * i + c];
                double acc = 0.0;
                for (int q = 0; q < 6; ++q)
                    acc += pr->lut[rc * FO_MAX_REGIONS + pr->region[nb[q]]] * (m[3 * nb[q] + c] - mc) * w[q];
                h[3 * i + c] += s * acc;
            }
            continue;
        }
        for (int c = 0; c < 3; ++c) {
            const double mc = m[3 * i + c];
            h[3 * i + c] += pref * ((m[3 * nb[1] + c] - 2.0 * mc + m[3 * nb[0] + c]) * ix2 +
                                    (m[3 * nb[3] + c] - 2.0 * mc + m[3 * nb[2] + c]) * iy2 +
                                    (m[3 * nb[5] + c] - 2.0 * mc + m[3 * nb[4] + c]) * iz2);
        }
    }
}

/* demag_field_add_into (fdm_fields.rs:528-609). */
static void demag_add(fo_problem *pr, const double *m, double *h) {
    const fo_params *p = &pr->p;
    const int nx = p->nx, ny = p->ny, nz = p->nz, px = pr->px, py = pr->py, pz = pr->pz;
    const long P = pr->P;
    for (int c = 0; c < 3; ++c) memset(pr->bm[c], 0, sizeof(double) * 2 * P);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
        const long d = (long)x + (long)px * (y + (long)py * z);
        for (int c = 0; c < 3; ++c) pr->bm[c][2 * d] = active(pr, i) ? m[3 * i + c] * p->ms * phi_w(pr, i) : 0.0;
    }
    for (int c = 0; c < 3; ++c) fo_fft3d(pr->bm[c], px, py, pz, 0);
    double *const *K = pr->kern;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < P; ++i) {
        const double mxr = pr->bm[0][2 * i], mxi = pr->bm[0][2 * i + 1];
        const double myr = pr->bm[1][2 * i], myi = pr->bm[1][2 * i + 1];
        const double mzr = pr->bm[2][2 * i], mzi = pr->bm[2][2 * i + 1];
#define CMR(k, ar, ai) (K[k][2 * i] * (ar) - K[k][2 * i + 1] * (ai))
#define CMI(k, ar, ai) (K[k][2 * i] * (ai) + K[k][2 * i + 1] * (ar))
        /* components: 0 xx, 1 yy, 2 zz, 3 xy, 4 xz, 5 yz */
        pr->bh[0][2 * i] = -(CMR(0, mxr, mxi) + CMR(3, myr, myi) + CMR(4, mzr, mzi));
        pr->bh[0][2 * i + 1] = -(CMI(0, mxr, mxi) + CMI(3, myr, myi) + CMI(4, mzr, mzi));
        pr->bh[1][2 * i] = -(CMR(3, mxr, mxi) + CMR(1, myr, myi) + CMR(5, mzr, mzi));
        pr->bh[1][2 * i + 1] = -(CMI(3, mxr, mxi) + CMI(1, myr, myi) + CMI(5, mzr, mzi));
        pr->bh[2][2 * i] = -(CMR(4, mxr, mxi) + CMR(5, myr, myi) + CMR(2, mzr, mzi));
        pr->bh[2][2 * i + 1] = -(CMI(4, mxr, mxi) + CMI(5, myr, myi) + CMI(2, mzr, mzi));
#undef CMR
#undef CMI
    }
    for (int c = 0; c < 3; ++c) fo_fft3d(pr->bh[c], px, py, pz, 1);
    const double norm = 1.0 / (double)P;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        if (!active(pr, i)) continue;
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
        const long s = (long)x + (long)px * (y + (long)py * z);
        for (int c = 0; c < 3; ++c) h[3 * i + c] += pr->bh[c][2 * s] * norm;
    }
    (void)nz;
    /* sparse boundary correction (targets in order; a repeated target accumulates) */
    for (uint32_t t = 0; t < p->corr_targets; ++t) {
        const int32_t ti = pr->ctidx[t];
        if (ti < 0) continue;
        for (uint32_t q = 0; q < p->corr_stencil; ++q) {
            const int32_t si = pr->csidx[(size_t)t * p->corr_stencil + q];
            if (si < 0) continue;
            const double *N = pr->ctensor + ((size_t)t * p->corr_stencil + q) * 6;
            const double w = (pr->phi ? pr->phi[si] : 1.0) * p->ms;
            const double Mx = w * m[3 * si], My = w * m[3 * si + 1], Mz = w * m[3 * si + 2];
            h[3 * ti] -= N[0] * Mx + N[1] * My + N[2] * Mz;
            h[3 * ti + 1] -= N[1] * Mx + N[3] * My + N[4] * Mz;
            h[3 * ti + 2] -= N[2] * Mx + N[4] * My + N[5] * Mz;
        }
    }
}

/* Uniaxial + cubic anisotropy field (fdm_fields.rs:648-705, 910-1047). The Kc3 term
 * follows the CUDA reference (native/backends/fdm/src/demag_fp32.cu:295-318). */
/* Anisotropy constant k (0 Ku1, 1 Ku2, 2 Kc1, 3 Kc2, 4 Kc3) at cell i: the per-cell map when
 * there is one, else the uniform value. */
static inline double kval(const fo_problem *pr, int k, long i, double uniform) {
    return pr->kmap[k] ? pr->kmap[k][i] : uniform;
}

static void anis_field_cell(const fo_problem *pr, const double *m, long i, double *h) {
    const fo_params *p = &pr->p;
    const double ms = p->ms > 1e-30 ? p->ms : 1e-30;
    if (p->has_uniaxial) {
        const double mu = m[0] * pr->u[0] + m[1] * pr->u[1] + m[2] * pr->u[2];
        const double cf = 2.0 * kval(pr, 0, i, p->ku1) / (FO_MU0 * ms) * mu + 4.0 * kval(pr, 1, i, p->ku2) / (FO_MU0 * ms) * mu * mu * mu;
        for (int c = 0; c < 3; ++c) h[c] += pr->u[c] * cf;
    }
    if (p->has_cubic) {
        const double m1 = m[0] * pr->c1[0] + m[1] * pr->c1[1] + m[2] * pr->c1[2];
        const double m2 = m[0] * pr->c2[0] + m[1] * pr->c2[1] + m[2] * pr->c2[2];
        const double m3 = m[0] * pr->c3[0] + m[1] * pr->c3[1] + m[2] * pr->c3[2];
        const double pf = 2.0 / (FO_MU0 * ms);
        const double s1 = m1 * m1, s2 = m2 * m2, s3 = m3 * m3;
        const double sig = s1 * s2 + s2 * s3 + s1 * s3;
        const double kc1 = kval(pr, 2, i, p->kc1), kc2 = kval(pr, 3, i, p->kc2), kc3 = kval(pr, 4, i, p->kc3);
        const double p3 = -4.0 * kc3 / (FO_MU0 * ms);
        const double g1 = -pf * (kc1 * m1 * (s2 + s3) + kc2 * m1 * s2 * s3) + p3 * sig * m1 * (s2 + s3);
        const double g2 = -pf * (kc1 * m2 * (s1 + s3) + kc2 * m2 * s1 * s3) + p3 * sig * m2 * (s1 + s3);
        const double g3 = -pf * (kc1 * m3 * (s1 + s2) + kc2 * m3 * s1 * s2) + p3 * sig * m3 * (s1 + s2);
        for (int c = 0; c < 3; ++c) h[c] += pr->c1[c] * g1 + pr->c2[c] * g2 + pr->c3[c] * g3;
    }
}

/* llg_rhs_from_field (fdm_fields.rs:2151-2162). */
static void rhs_cell(const fo_params *p, const double *m, const double *h, double *k) {
    const double gb = p->gamma / (1.0 + p->alpha * p->alpha);
    const double pr0 = m[1] * h[2] - m[2] * h[1];
    const double pr1 = m[2] * h[0] - m[0] * h[2];
    const double pr2 = m[0] * h[1] - m[1] * h[0];
    const double d0 = m[1] * pr2 - m[2] * pr1;
    const double d1 = m[2] * pr0 - m[0] * pr2;
    const double d2 = m[0] * pr1 - m[1] * pr0;
    const double s = p->disable_precession ? 0.0 : 1.0;
    k[0] = -gb * (s * pr0 + p->alpha * d0);
    k[1] = -gb * (s * pr1 + p->alpha * d1);
    k[2] = -gb * (s * pr2 + p->alpha * d2);
}

/* Full field evaluation: effective_field_into_ws (fdm_fields.rs:1153-1182). */
/* Neighbours x-, x+, y-, y+, z-, z+ of cell i with the Neumann clamp and the active mask
 * (a missing or inactive neighbour is the cell itself; demag_fp32.cu:324-340). */
static void clamped_neighbours(const fo_problem *pr, long i, long nb[6]) {
    axis_neighbours(&pr->p, i, nb);
    for (int q = 0; q < 6; ++q)
        if (!active(pr, nb[q])) nb[q] = i;
}

/* Central differences d m_c / d axis over 2 d with the clamped neighbours: g[c][axis]. */
static void central_gradient(const fo_problem *pr, const double *m, long i, double g[3][3]) {
    const fo_params *p = &pr->p;
    long nb[6];
    clamped_neighbours(pr, i, nb);
    const double inv[3] = {0.5 / p->dx, 0.5 / p->dy, 0.5 / p->dz};
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) g[c][a] = (m[3 * nb[2 * a + 1] + c] - m[3 * nb[2 * a] + c]) * inv[a];
}

/* DMI and magnetoelastic field at active cell i added to h (demag_fp32.cu:319-376):
 * interfacial 2D/(mu0 Ms) (dmz/dx, dmz/dy, -(dmx/dx + dmy/dy)), bulk 2D/(mu0 Ms) curl m,
 * magnetoelastic -1/(mu0 Ms) (2 B1 m_i e_ii + B2 sum_{j != i} m_j e_ij). */
static void dmi_mel_field_cell(const fo_problem *pr, const double *m, long i, double *h) {
    const fo_params *p = &pr->p;
    if (p->ms <= 0.0) return;
    if (p->has_interfacial_dmi || p->has_bulk_dmi) {
        double g[3][3];
        central_gradient(pr, m, i, g);
        const double pf = 2.0 / (FO_MU0 * p->ms);
        if (p->has_interfacial_dmi) {
            const double k = pf * p->dmi_d_interfacial;
            h[0] += k * g[2][0];
            h[1] += k * g[2][1];
            h[2] -= k * (g[0][0] + g[1][1]);
        }
        if (p->has_bulk_dmi) {
            const double k = pf * p->dmi_d_bulk;
            h[0] += k * (g[2][1] - g[1][2]);
            h[1] += k * (g[0][2] - g[2][0]);
            h[2] += k * (g[1][0] - g[0][1]);
        }
    }
    if (p->has_magnetoelastic) {
        const double *mi = m + 3 * i;
        const double a = -1.0 / (FO_MU0 * p->ms), b1 = p->mel_b1, b2 = p->mel_b2;
        const double e11 = p->mel_strain[0], e22 = p->mel_strain[1], e33 = p->mel_strain[2];
        const double e23 = 0.5 * p->mel_strain[3], e13 = 0.5 * p->mel_strain[4], e12 = 0.5 * p->mel_strain[5];
        h[0] += a * (2.0 * b1 * mi[0] * e11 + b2 * (mi[1] * e12 + mi[2] * e13));
        h[1] += a * (2.0 * b1 * mi[1] * e22 + b2 * (mi[0] * e12 + mi[2] * e23));
        h[2] += a * (2.0 * b1 * mi[2] * e33 + b2 * (mi[0] * e13 + mi[1] * e23));
    }
}

/* DMI energy density at active cell i (reductions_fp64.cu:647-710): interfacial
 * D [mz (dmx/dx + dmy/dy) - mx dmz/dx - my dmz/dy], bulk D m.(curl m). */
static double dmi_energy_cell(const fo_problem *pr, const double *m, long i) {
    const fo_params *p = &pr->p;
    if (!(p->has_interfacial_dmi || p->has_bulk_dmi)) return 0.0;
    double g[3][3];
    central_gradient(pr, m, i, g);
    const double *mi = m + 3 * i;
    double e = 0.0;
    if (p->has_interfacial_dmi)
        e += p->dmi_d_interfacial * (mi[2] * (g[0][0] + g[1][1]) - mi[0] * g[2][0] - mi[1] * g[2][1]);
    if (p->has_bulk_dmi)
        e += p->dmi_d_bulk * (mi[0] * (g[2][1] - g[1][2]) + mi[1] * (g[0][2] - g[2][0]) + mi[2] * (g[1][0] - g[0][1]));
    return e;
}

/* Thermal field (crates/fullmag-engine/src/fdm_fields.rs:818-896).  sigma at step size dt
 * (the fixed step; 1e-13 s, the reference's default thermal_dt, for adaptive integrators). */
static double thermal_sigma(const fo_params *p, double dt) {
    if (!(p->temperature > 0.0) || !(p->ms > 0.0) || !(dt > 0.0)) return 0.0;
    const double kb = 1.380649e-23, mu0 = 1.2566370614359173e-6;
    const double gamma0 = p->gamma * (1.0 + p->alpha * p->alpha);
    return sqrt(2.0 * p->alpha * kb * p->temperature / (gamma0 * mu0 * p->ms * p->dx * p->dy * p->dz * dt));
}

/* SplitMix64 output function (Vigna's published finaliser). */
static uint64_t splitmix64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Uniform in (0, 1] from the key seed + step C1 + cell C2 + stream C3 (wrapping). */
static double counter_uniform(uint64_t seed, uint64_t step, uint64_t cell, uint64_t stream) {
    const uint64_t key = seed + step * 0x9E3779B97F4A7C15ull + cell * 0x517CC1B727220A95ull + stream * 0x6C62272E07BB0142ull;
    return ((double)(splitmix64_mix(key) >> 11) + 1.0) / (9007199254740992.0 + 1.0);
}

/* Adds sigma (r1 cos t1, r1 sin t1, r2 cos t2) at cell i, Box-Muller on four uniforms. */
static void thermal_add(const fo_problem *pr, long i, double *h) {
    const uint64_t seed = pr->p.thermal_seed, st = pr->th_eval, ci = (uint64_t)i;
    double u1 = counter_uniform(seed, st, ci, 0), u3 = counter_uniform(seed, st, ci, 2);
    if (u1 < 1e-300) u1 = 1e-300;
    if (u3 < 1e-300) u3 = 1e-300;
    const double u2 = counter_uniform(seed, st, ci, 1), u4 = counter_uniform(seed, st, ci, 3);
    const double r1 = sqrt(-2.0 * log(u1)), r2 = sqrt(-2.0 * log(u3));
    const double t1 = 2.0 * M_PI * u2, t2 = 2.0 * M_PI * u4;
    h[0] += pr->th_sigma * r1 * cos(t1);
    h[1] += pr->th_sigma * r1 * sin(t1);
    h[2] += pr->th_sigma * r2 * cos(t2);
}

/* Current of the Oersted conductor at time t (demag_fp32.cu:586-606). */
static double oersted_scale(const fo_params *p, double t) {
    double I = p->oersted_current;
    if (p->oersted_kind == 1) I *= sin(2.0 * M_PI * p->oersted_freq * t + p->oersted_phase) + p->oersted_offset;
    else if (p->oersted_kind == 2) I *= (t >= p->oersted_t_on && t < p->oersted_t_off) ? 1.0 : 0.0;
    return I;
}

static void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Spin-transfer and spin-orbit torques added to dm/dt at active cell i
 * (native/backends/fdm/src/llg_fp32.cu:65-195):
 *   Zhang-Li   -m x (m x D) - beta m x D, D = (u.grad) m by upwind differences (the
 *              upwind neighbour when it exists, taken without the mask as the reference
 *              does, else no contribution along that axis)
 *   Slonczewski beta_STT g [m x (m x p) + eps' m x p], g = P L^2 / ((L^2 + 1) + (L^2 - 1) m.p)
 *   SOT        amp (-xi_DL ((m.s) m - s) + xi_FL m x s) */
static void torque_add(const fo_problem *pr, const double *m, long i, double *k) {
    const fo_params *p = &pr->p;
    const double *mi = m + 3 * i;
    if (pr->has_zl) {
        const int nx = p->nx, ny = p->ny, nz = p->nz;
        const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
        const int pos[3] = {x, y, z}, ext[3] = {nx, ny, nz};
        const long stride[3] = {1, nx, (long)nx * ny};
        const double inv[3] = {1.0 / p->dx, 1.0 / p->dy, 1.0 / p->dz};
        double D[3] = {0, 0, 0};
        for (int a = 0; a < 3; ++a) {
            const double u = pr->zl_u[a];
            /* a periodic axis always has the upwind neighbour, wrapped (fdm_fields.rs:1288-1320) */
            const int wrap = p->periodic[a] != 0;
            if (u > 0.0 && (pos[a] > 0 || wrap)) {
                const double *q = m + 3 * (pos[a] > 0 ? i - stride[a] : i + stride[a] * (ext[a] - 1));
                for (int c = 0; c < 3; ++c) D[c] += u * (mi[c] - q[c]) * inv[a];
            } else if (u < 0.0 && (pos[a] < ext[a] - 1 || wrap)) {
                const double *q = m + 3 * (pos[a] < ext[a] - 1 ? i + stride[a] : i - stride[a] * (ext[a] - 1));
                for (int c = 0; c < 3; ++c) D[c] += u * (q[c] - mi[c]) * inv[a];
            }
        }
        double c1[3], c2[3];
        cross3(mi, D, c1);
        cross3(mi, c1, c2);
        for (int c = 0; c < 3; ++c) k[c] += -c2[c] - p->stt_beta * c1[c];
    }
    if (pr->has_slon) {
        const double L2 = p->stt_lambda * p->stt_lambda;
        const double mp = mi[0] * p->stt_p[0] + mi[1] * p->stt_p[1] + mi[2] * p->stt_p[2];
        const double g = pr->slon_P * L2 / ((L2 + 1.0) + (L2 - 1.0) * mp);
        double c1[3], c2[3];
        cross3(mi, p->stt_p, c1);
        cross3(mi, c1, c2);
        for (int c = 0; c < 3; ++c) k[c] += pr->slon_pf * g * (c2[c] + p->stt_epsilon_prime * c1[c]);
    }
    if (pr->has_sot) {
        const double *sv = pr->sot_s;
        const double ms_ = mi[0] * sv[0] + mi[1] * sv[1] + mi[2] * sv[2];
        double fl[3];
        cross3(mi, sv, fl);
        for (int c = 0; c < 3; ++c) k[c] += pr->sot_amp * (-p->sot_xi_dl * (ms_ * mi[c] - sv[c]) + p->sot_xi_fl * fl[c]);
    }
}

static void eval_fields(fo_problem *pr, const double *m, double *h_ex, double *h_d, double *h_eff,
                        double *rhs) {
    const fo_params *p = &pr->p;
    const long n3 = 3 * pr->n;
    memset(h_ex, 0, sizeof(double) * n3);
    memset(h_d, 0, sizeof(double) * n3);
    if (p->enable_exchange) exchange_add(pr, m, h_ex);
    if (p->enable_demag) demag_add(pr, m, h_d);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        double h[3] = {h_ex[3 * i] + h_d[3 * i], h_ex[3 * i + 1] + h_d[3 * i + 1], h_ex[3 * i + 2] + h_d[3 * i + 2]};
        if (active(pr, i)) {
            if (p->has_external_field)
                for (int c = 0; c < 3; ++c) h[c] += p->h_ext[c];
            if (pr->hmap)
                for (int c = 0; c < 3; ++c) h[c] += pr->hmap[3 * i + c];
            anis_field_cell(pr, m + 3 * i, i, h);
            dmi_mel_field_cell(pr, m, i, h);
            if (pr->h_oe)
                for (int c = 0; c < 3; ++c) h[c] += pr->oe_scale * pr->h_oe[3 * i + c];
            if (pr->th_sigma > 0.0) thermal_add(pr, i, h);
        }
        for (int c = 0; c < 3; ++c) h_eff[3 * i + c] = h[c];
        if (rhs) {
            rhs_cell(p, m + 3 * i, h, rhs + 3 * i);
            if (active(pr, i)) torque_add(pr, m, i, rhs + 3 * i);
        }
    }
}

int fo_fields(fo_problem *pr, const double *m_aos, double *h_ex, double *h_demag, double *h_ext,
              double *h_eff, double *rhs) {
    const long n3 = 3 * pr->n;
    pr->oe_scale = oersted_scale(&pr->p, pr->t);
    pr->th_eval = pr->th_step;
    pr->th_sigma = thermal_sigma(&pr->p, pr->th_dt);
    double *m = dalloc(n3), *a = dalloc(n3), *b = dalloc(n3), *e = dalloc(n3), *r = dalloc(n3);
    for (long i = 0; i < pr->n; ++i)
        for (int c = 0; c < 3; ++c) m[3 * i + c] = active(pr, i) ? m_aos[3 * i + c] : 0.0;
    eval_fields(pr, m, a, b, e, r);
    if (h_ex) memcpy(h_ex, a, sizeof(double) * n3);
    if (h_demag) memcpy(h_demag, b, sizeof(double) * n3);
    if (h_eff) memcpy(h_eff, e, sizeof(double) * n3);
    if (rhs) memcpy(rhs, r, sizeof(double) * n3);
    if (h_ext)
        for (long i = 0; i < pr->n; ++i)
            for (int c = 0; c < 3; ++c)
                h_ext[3 * i + c] = (pr->p.has_external_field && active(pr, i)) ? pr->p.h_ext[c] : 0.0;
    free(m); free(a); free(b); free(e); free(r);
    return 0;
}

static double vmax_norm(const double *v, long n) {
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (long i = 0; i < n; ++i) {
        const double s = sqrt(v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
        if (s > mx) mx = s;
    }
    return mx;
}

/* Energies: C ABI conventions (native/backends/fdm/src/reductions_fp64.cu:123-342,605-642)
 * and the CPU forms (fdm_fields.rs:349-355, 2168-2273). */
static void energies(fo_problem *pr, const double *m, const double *h_ex, const double *h_d,
                     const double *h_eff, const double *rhs, fo_stats *st) {
    const fo_params *p = &pr->p;
    const double V = p->dx * p->dy * p->dz;
    const double ix2 = 1.0 / (p->dx * p->dx), iy2 = 1.0 / (p->dy * p->dy), iz2 = 1.0 / (p->dz * p->dz);
    double epair = 0.0, exf = 0.0, ed = 0.0, eext = 0.0, euni = 0.0, ecub = 0.0, eacpu = 0.0, edmi = 0.0;
#pragma omp parallel for reduction(+ : epair, exf, ed, eext, euni, ecub, eacpu, edmi) schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        if (!active(pr, i)) continue;
        const double *mi = m + 3 * i;
        edmi += V * dmi_energy_cell(pr, m, i);
        if (p->enable_exchange) {
            /* forward pairs; on a periodic axis the last cell pairs with the first */
            long all[6];
            axis_neighbours(p, i, all);
            long nb[3] = {all[1], all[3], all[5]};
            const double w[3] = {ix2, iy2, iz2};
            for (int q = 0; q < 3; ++q) {
                if (nb[q] == i || !active(pr, nb[q])) continue;
                const double a = m[3 * nb[q]] - mi[0], b = m[3 * nb[q] + 1] - mi[1], c = m[3 * nb[q] + 2] - mi[2];
                const double A = pr->region ? pr->lut[pr->region[i] * FO_MAX_REGIONS + pr->region[nb[q]]] : p->a_ex;
                epair += A * V * phi_w(pr, i) * (a * a + b * b + c * c) * w[q];
            }
            exf += -0.5 * FO_MU0 * p->ms * V * (mi[0] * h_ex[3 * i] + mi[1] * h_ex[3 * i + 1] + mi[2] * h_ex[3 * i + 2]);
        }
        const double ph = phi_w(pr, i);
        if (p->enable_demag)
            ed += -0.5 * FO_MU0 * p->ms * V * ph * (mi[0] * h_d[3 * i] + mi[1] * h_d[3 * i + 1] + mi[2] * h_d[3 * i + 2]);
        if (p->has_external_field)
            eext += -FO_MU0 * p->ms * V * ph * (mi[0] * p->h_ext[0] + mi[1] * p->h_ext[1] + mi[2] * p->h_ext[2]);
        if (pr->hmap)
            eext += -FO_MU0 * p->ms * V *
                    (mi[0] * pr->hmap[3 * i] + mi[1] * pr->hmap[3 * i + 1] + mi[2] * pr->hmap[3 * i + 2]);
        if (p->has_uniaxial) {
            const double mu = mi[0] * pr->u[0] + mi[1] * pr->u[1] + mi[2] * pr->u[2];
            const double s = mu * mu;
            euni += -V * ph * (kval(pr, 0, i, p->ku1) * s + kval(pr, 1, i, p->ku2) * s * s);
        }
        if (p->has_cubic) {
            const double m1 = mi[0] * pr->c1[0] + mi[1] * pr->c1[1] + mi[2] * pr->c1[2];
            const double m2 = mi[0] * pr->c2[0] + mi[1] * pr->c2[1] + mi[2] * pr->c2[2];
            const double m3 = mi[0] * pr->c3[0] + mi[1] * pr->c3[1] + mi[2] * pr->c3[2];
            const double s1 = m1 * m1, s2 = m2 * m2, s3 = m3 * m3;
            const double sig = s1 * s2 + s2 * s3 + s1 * s3;
            ecub += V * ph * (kval(pr, 2, i, p->kc1) * sig + kval(pr, 3, i, p->kc2) * s1 * s2 * s3 + kval(pr, 4, i, p->kc3) * sig * sig);
        }
        if (p->has_uniaxial || p->has_cubic) {
            double ha[3] = {0, 0, 0};
            anis_field_cell(pr, mi, i, ha);
            eacpu += -0.5 * FO_MU0 * p->ms * V * (mi[0] * ha[0] + mi[1] * ha[1] + mi[2] * ha[2]);
        }
    }
    st->e_exchange = epair;
    st->e_exchange_field = exf;
    st->e_demag = ed;
    st->e_external = eext;
    st->e_uniaxial = euni;
    st->e_cubic = ecub;
    st->e_anis_cpu = eacpu;
    st->e_dmi = edmi;
    st->e_total = epair + ed + eext + euni + ecub + edmi;
    st->max_h_eff = vmax_norm(h_eff, pr->n);
    st->max_h_demag = p->enable_demag ? vmax_norm(h_d, pr->n) : 0.0;
    st->max_rhs = vmax_norm(rhs, pr->n);
}

/* Statistics at the current state with the Oersted current at t_oe and the thermal field of
 * step counter th (the evaluation of the state itself, or the last evaluation of a step). */
static int observe_at(fo_problem *pr, fo_stats *st, double t_oe, uint64_t th) {
    const long n3 = 3 * pr->n;
    pr->oe_scale = oersted_scale(&pr->p, t_oe);
    pr->th_eval = th;
    pr->th_sigma = thermal_sigma(&pr->p, pr->th_dt);
    double *a = dalloc(n3), *b = dalloc(n3), *r = dalloc(n3);
    eval_fields(pr, pr->m, a, b, pr->heff, r);
    memset(st, 0, sizeof(*st));
    energies(pr, pr->m, a, b, pr->heff, r, st);
    st->step = pr->step;
    st->time = pr->t;
    free(a); free(b); free(r);
    return 0;
}

int fo_observe(fo_problem *pr, fo_stats *st) { return observe_at(pr, st, pr->t, pr->th_step); }

static void rhs_of(fo_problem *pr, const double *m, double *k) {
    const long n3 = 3 * pr->n;
    double *a = dalloc(n3), *b = dalloc(n3);
    eval_fields(pr, m, a, b, pr->heff, k);
    free(a); free(b);
}

/* out = normalize(m0 + dt * sum_j c_j k_j) (vector::normalized, zero stays zero). */
static void stage_combine(const fo_problem *pr, double *out, const double *m0, int nk, double *const *ks,
                          const double *cs, double dt) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        double v[3];
        for (int c = 0; c < 3; ++c) {
            double acc = 0.0;
            for (int j = 0; j < nk; ++j) acc += cs[j] * ks[j][3 * i + c];
            v[c] = m0[3 * i + c] + acc * dt;
        }
        const double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
        for (int c = 0; c < 3; ++c) out[3 * i + c] = v[c] * inv;
    }
}

/* Dormand-Prince 5(4) tableau (fdm_integrators.rs:441-468). */
static const double DP_A[6][5] = {
    {1.0 / 5.0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0},
    {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0}};
static const double DP_B6 = 11.0 / 84.0;
static const double DP_E[7] = {71.0 / 57600.0, 0.0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0,
                               22.0 / 525.0, -1.0 / 40.0};

/* max error norm (fdm_integrators.rs:828-873; native/backends/fdm/src/llg_dp45_fp32.cu:108-128,175-184). */
static double dp45_error(const fo_problem *pr, double dt) {
    const fo_params *p = &pr->p;
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        double e[3] = {0, 0, 0};
        for (int s = 0; s < 7; ++s)
            for (int c = 0; c < 3; ++c) e[c] += DP_E[s] * pr->k[s][3 * i + c];
        const double en = dt * sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        double v = en;
        if (p->dp45_norm == 1 && p->rtol > 0.0) {
            const double *m0 = pr->m0 + 3 * i;
            double yn = sqrt(m0[0] * m0[0] + m0[1] * m0[1] + m0[2] * m0[2]);
            if (yn < 1e-30) yn = 1e-30;
            v = en / (p->max_error + p->rtol * yn);
        }
        if (v > mx) mx = v;
    }
    return mx;
}

static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Heun from pr->m0 into pr->m (fdm_integrators.rs:87-153). */
static void heun_step(fo_problem *pr, double dt) {
    rhs_of(pr, pr->m0, pr->k[0]);
    const double c1[1] = {1.0};
    stage_combine(pr, pr->mst, pr->m0, 1, pr->k, c1, dt);
    rhs_of(pr, pr->mst, pr->k[1]);
    const double c2[2] = {0.5, 0.5};
    stage_combine(pr, pr->m, pr->m0, 2, pr->k, c2, dt);
}

/* Bogacki-Shampine 3(2) error max_i dt |sum_j E_j k_j| over k1..k4 (the ABI's absolute
 * max-norm; native/backends/fdm/src/llg_rk23_fp32.cu:78-94,218). */
static const double BS_E[4] = {-5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -1.0 / 8.0};
static double rk23_error(const fo_problem *pr, double dt) {
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        double e[3] = {0, 0, 0};
        for (int s = 0; s < 4; ++s)
            for (int c = 0; c < 3; ++c) e[c] += BS_E[s] * pr->k[s][3 * i + c];
        const double en = dt * sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        if (en > mx) mx = en;
    }
    return mx;
}

int fo_step(fo_problem *pr, double dt, fo_stats *st) {
    const fo_params *p = &pr->p;
    const long n3 = 3 * pr->n;
    memcpy(pr->m0, pr->m, sizeof(double) * n3);
    /* every stage of a step (and of its retries) sees the Oersted current at the step's
     * start, as the GPU backend evaluates it from the time before the update, and the
     * thermal field of the step counter, which advances once per completed step
     * (fdm_problem.rs:244-245); its amplitude takes the fixed step, or 1e-13 s for the
     * adaptive integrators (the reference's thermal_dt when no fixed step is set,
     * fdm_problem.rs:92, cpu_reference.rs:287-290) */
    const double t_start = pr->t;
    const int adaptive = p->integrator == 2 || p->integrator == 5;
    pr->th_dt = adaptive ? 1e-13 : dt;
    pr->oe_scale = oersted_scale(p, pr->t);
    pr->th_eval = pr->th_step;
    pr->th_sigma = thermal_sigma(p, pr->th_dt);
    double rejected = 0.0, suggested = 0.0;
    if (p->integrator == 1) { /* Heun: fdm_integrators.rs:87-153 */
        heun_step(pr, dt);
    } else if (p->integrator == 3) {
        /* ABM3 with the GPU backend's start-up rule (llg_abm3_fp32.cu:115-266): a Heun
         * step while fewer than 3 steps built the history or when dt moved by more than
         * 10 %; then the Adams-Bashforth predictor, f at the prediction, the
         * Adams-Moulton corrector.  The newest history entry is f at the accepted state
         * after a Heun step and f at the prediction after an ABM3 step. */
        if (pr->abm_last_dt > 0.0 && fabs(dt - pr->abm_last_dt) / pr->abm_last_dt > 0.1) pr->abm_startup = 0;
        double **h = pr->abm_h;
        if (pr->abm_startup < 3) {
            heun_step(pr, dt);
            double *t = h[2];
            h[2] = h[1];
            h[1] = h[0];
            h[0] = t;
            pr->oe_scale = oersted_scale(p, pr->t + dt);  /* evaluated after the time update */
            pr->th_eval = pr->th_step + 1;
            rhs_of(pr, pr->m, h[0]);
            pr->abm_startup += 1;
        } else {
            double *hp[3] = {h[0], h[1], h[2]};
            const double cp[3] = {23.0 / 12.0, -16.0 / 12.0, 5.0 / 12.0};
            stage_combine(pr, pr->mst, pr->m0, 3, hp, cp, dt);
            rhs_of(pr, pr->mst, pr->k[0]);
            double *hc[3] = {pr->k[0], h[0], h[1]};
            const double cc[3] = {5.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0};
            stage_combine(pr, pr->m, pr->m0, 3, hc, cc, dt);
            double *t = h[2];
            h[2] = h[1];
            h[1] = h[0];
            h[0] = t;
            memcpy(h[0], pr->k[0], sizeof(double) * n3);
        }
        pr->abm_last_dt = dt;
    } else if (p->integrator == 5) {
        /* Bogacki-Shampine 3(2) + FSAL with the ABI's step control
         * (llg_rk23_fp32.cu:150-265): stages N(m0 + dt/2 k1), N(m0 + 3dt/4 k2), solution
         * N(m0 + dt (2/9 k1 + 1/3 k2 + 4/9 k3)), k4 at the solution. */
        static const double B[3] = {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0};
        for (;;) {
            if (pr->fsal_valid) memcpy(pr->k[0], pr->fsal, sizeof(double) * n3);
            else rhs_of(pr, pr->m0, pr->k[0]);
            const double a2[1] = {0.5}, a3[1] = {0.75};
            stage_combine(pr, pr->mst, pr->m0, 1, &pr->k[0], a2, dt);
            rhs_of(pr, pr->mst, pr->k[1]);
            stage_combine(pr, pr->mst, pr->m0, 1, &pr->k[1], a3, dt);
            rhs_of(pr, pr->mst, pr->k[2]);
            stage_combine(pr, pr->mst, pr->m0, 3, pr->k, B, dt);
            rhs_of(pr, pr->mst, pr->k[3]);
            const double err = rk23_error(pr, dt);
            if (err <= p->max_error || dt <= p->dt_min) {
                memcpy(pr->m, pr->mst, sizeof(double) * n3);
                memcpy(pr->fsal, pr->k[3], sizeof(double) * n3);
                pr->fsal_valid = 1;
                suggested = err > 0.0 ? clampd(p->headroom * dt * pow(p->max_error / err, 1.0 / 3.0), p->dt_min, p->dt_max)
                                      : p->dt_max;
                break;
            }
            rejected += 1.0;
            dt = clampd(p->headroom * dt * pow(p->max_error / err, 1.0 / 3.0), p->dt_min, p->dt_max);
            pr->fsal_valid = 0;
        }
    } else if (p->integrator == 4) { /* RK4: fdm_integrators.rs:155-262 */
        rhs_of(pr, pr->m0, pr->k[0]);
        const double h[1] = {0.5}, f[1] = {1.0};
        stage_combine(pr, pr->mst, pr->m0, 1, &pr->k[0], h, dt);
        rhs_of(pr, pr->mst, pr->k[1]);
        stage_combine(pr, pr->mst, pr->m0, 1, &pr->k[1], h, dt);
        rhs_of(pr, pr->mst, pr->k[2]);
        stage_combine(pr, pr->mst, pr->m0, 1, &pr->k[2], f, dt);
        rhs_of(pr, pr->mst, pr->k[3]);
        const double w[4] = {1.0 / 6.0, 2.0 / 6.0, 2.0 / 6.0, 1.0 / 6.0};
        stage_combine(pr, pr->m, pr->m0, 4, pr->k, w, dt);
    } else if (p->integrator == 2) { /* DP45 + FSAL: fdm_integrators.rs:429-681 (CPU norm) or
                                        llg_dp45_fp32.cu:188-342 (ABI norm) */
        const int cpu = p->dp45_norm == 1;
        if (cpu) dt = clampd(dt, p->dt_min, p->dt_max);
        for (;;) {
            if (pr->fsal_valid) memcpy(pr->k[0], pr->fsal, sizeof(double) * n3);
            else rhs_of(pr, pr->m0, pr->k[0]);
            for (int s = 0; s < 5; ++s) {
                stage_combine(pr, pr->mst, pr->m0, s + 1, pr->k, DP_A[s], dt);
                rhs_of(pr, pr->mst, pr->k[s + 1]);
            }
            double bw[6] = {DP_A[5][0], DP_A[5][1], DP_A[5][2], DP_A[5][3], DP_A[5][4], DP_B6};
            stage_combine(pr, pr->mst, pr->m0, 6, pr->k, bw, dt);
            rhs_of(pr, pr->mst, pr->k[6]);
            const double err = dp45_error(pr, dt);
            const double thr = (cpu && p->rtol > 0.0) ? 1.0 : p->max_error;
            if (err <= thr || dt <= p->dt_min) {
                memcpy(pr->m, pr->mst, sizeof(double) * n3);
                memcpy(pr->fsal, pr->k[6], sizeof(double) * n3);
                pr->fsal_valid = 1;
                if (cpu) {
                    double ratio = p->headroom * pow(thr / (err > 1e-30 ? err : 1e-30), 0.2);
                    ratio = clampd(ratio, p->shrink_limit, p->growth_limit);
                    suggested = clampd(dt * ratio, p->dt_min, p->dt_max);
                } else {
                    suggested = err > 0.0 ? clampd(p->headroom * dt * pow(p->max_error / err, 0.2), p->dt_min, p->dt_max)
                                          : p->dt_max;
                }
                break;
            }
            rejected += 1.0;
            if (cpu) {
                double ratio = clampd(p->headroom * pow(thr / err, 0.2), p->shrink_limit, p->growth_limit);
                dt = clampd(dt * ratio, p->dt_min, p->dt_max);
            } else {
                dt = clampd(p->headroom * dt * pow(p->max_error / err, 0.2), p->dt_min, p->dt_max);
            }
            pr->fsal_valid = 0;
        }
    } else {
        return -1;
    }
    pr->t += dt;
    pr->step += 1.0;
    pr->th_step += 1;
    /* the statistics of a step come from its last evaluation: at the new state after the
     * time and counter update for the fixed-step integrators, the first-same-as-last
     * derivative (inside the step) for DP45 and RK23 */
    if (adaptive) observe_at(pr, st, t_start, pr->th_step - 1);
    else fo_observe(pr, st);
    st->dt_used = dt;
    st->suggested_next_dt = suggested;
    st->rejected_attempts = rejected;
    return 0;
}

/* ---- Tangent-linear RK4 (checks the engine's reverse-mode gradients) ----
 * Differentiates the fixed-step RK4 of fo_step (fdm_integrators.rs:155-262) with
 * respect to the initial state and the field map, in FP64:
 *   dk   = -gb [s (dm x H + m x dH) + alpha (dm x (m x H) + m x (dm x H + m x dH))]
 *   dH   = H_lin(dm) + J_anis(m) dm + dh_map      (H_lin: exchange + demag, linear)
 *   d N(v) = (dv - u (u . dv)) / |v|,  u = N(v). */
static void tangent_rhs(fo_problem *pr, const double *m, const double *dm, const double *dh, double *k,
                        double *dk, double *ha, double *hb, double *dha, double *dhb) {
    const fo_params *p = &pr->p;
    const long n3 = 3 * pr->n;
    double *heff = pr->heff, *dheff = pr->hscr;
    eval_fields(pr, m, ha, hb, heff, k);
    memset(dha, 0, sizeof(double) * n3);
    memset(dhb, 0, sizeof(double) * n3);
    if (p->enable_exchange) exchange_add(pr, dm, dha);
    if (p->enable_demag) demag_add(pr, dm, dhb);
    const double gb = p->gamma / (1.0 + p->alpha * p->alpha);
    const double s = p->disable_precession ? 0.0 : 1.0;
    const double ms = p->ms > 1e-30 ? p->ms : 1e-30;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        const double *mi = m + 3 * i, *dmi = dm + 3 * i, *H = heff + 3 * i;
        double dH[3] = {dha[3 * i] + dhb[3 * i], dha[3 * i + 1] + dhb[3 * i + 1], dha[3 * i + 2] + dhb[3 * i + 2]};
        if (active(pr, i)) {
            if (dh)
                for (int c = 0; c < 3; ++c) dH[c] += dh[3 * i + c];
            if (p->has_uniaxial) {
                const double mu = mi[0] * pr->u[0] + mi[1] * pr->u[1] + mi[2] * pr->u[2];
                const double dmu = dmi[0] * pr->u[0] + dmi[1] * pr->u[1] + dmi[2] * pr->u[2];
                const double cf = (2.0 * kval(pr, 0, i, p->ku1) + 12.0 * kval(pr, 1, i, p->ku2) * mu * mu) / (FO_MU0 * ms) * dmu;
                for (int c = 0; c < 3; ++c) dH[c] += cf * pr->u[c];
            }
        }
        for (int c = 0; c < 3; ++c) dheff[3 * i + c] = dH[c];
        const double P_[3] = {mi[1] * H[2] - mi[2] * H[1], mi[2] * H[0] - mi[0] * H[2], mi[0] * H[1] - mi[1] * H[0]};
        const double dP[3] = {dmi[1] * H[2] - dmi[2] * H[1] + mi[1] * dH[2] - mi[2] * dH[1],
                              dmi[2] * H[0] - dmi[0] * H[2] + mi[2] * dH[0] - mi[0] * dH[2],
                              dmi[0] * H[1] - dmi[1] * H[0] + mi[0] * dH[1] - mi[1] * dH[0]};
        const double dQ[3] = {dmi[1] * P_[2] - dmi[2] * P_[1] + mi[1] * dP[2] - mi[2] * dP[1],
                              dmi[2] * P_[0] - dmi[0] * P_[2] + mi[2] * dP[0] - mi[0] * dP[2],
                              dmi[0] * P_[1] - dmi[1] * P_[0] + mi[0] * dP[1] - mi[1] * dP[0]};
        for (int c = 0; c < 3; ++c) dk[3 * i + c] = -gb * (s * dP[c] + p->alpha * dQ[c]);
    }
}

/* out = N(y0 + dt sum c_j k_j), dout = dN(v)[dy0 + dt sum c_j dk_j]. */
static void tangent_combine(const fo_problem *pr, double *out, double *dout, const double *y0, const double *dy0,
                            int nk, double *const *ks, double *const *dks, const double *cs, double dt) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < pr->n; ++i) {
        double v[3], dv[3];
        for (int c = 0; c < 3; ++c) {
            double a = 0.0, da = 0.0;
            for (int j = 0; j < nk; ++j) {
                a += cs[j] * ks[j][3 * i + c];
                da += cs[j] * dks[j][3 * i + c];
            }
            v[c] = y0[3 * i + c] + a * dt;
            dv[c] = dy0[3 * i + c] + da * dt;
        }
        const double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
        double u[3], ud = 0.0;
        for (int c = 0; c < 3; ++c) {
            u[c] = v[c] * inv;
            ud += u[c] * dv[c];
        }
        for (int c = 0; c < 3; ++c) {
            out[3 * i + c] = u[c];
            dout[3 * i + c] = (dv[c] - u[c] * ud) * inv;
        }
    }
}

int fo_tangent_rk4(fo_problem *pr, double dt, uint64_t n_steps, const double *dh_aos, const double *dm0_aos,
                   double *dm_out) {
    const fo_params *p = &pr->p;
    if (p->has_cubic) return -1;
    const long n = pr->n, n3 = 3 * n;
    double *y0 = pr->m0, *ys = pr->mst, *ks[4], *dks[4];
    double *dy0 = dalloc(n3), *dys = dalloc(n3), *ha = dalloc(n3), *hb = dalloc(n3), *dha = dalloc(n3),
           *dhb = dalloc(n3), *ynext = dalloc(n3), *dynext = dalloc(n3);
    for (int s = 0; s < 4; ++s) {
        ks[s] = pr->k[s];
        dks[s] = dalloc(n3);
    }
    if (dm0_aos)
        for (long i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) dy0[3 * i + c] = active(pr, i) ? dm0_aos[3 * i + c] : 0.0;
    memcpy(y0, pr->m, sizeof(double) * n3);
    const double half[1] = {0.5}, one[1] = {1.0}, w[4] = {1.0 / 6.0, 2.0 / 6.0, 2.0 / 6.0, 1.0 / 6.0};
    for (uint64_t st = 0; st < n_steps; ++st) {
        tangent_rhs(pr, y0, dy0, dh_aos, ks[0], dks[0], ha, hb, dha, dhb);
        tangent_combine(pr, ys, dys, y0, dy0, 1, &ks[0], &dks[0], half, dt);
        tangent_rhs(pr, ys, dys, dh_aos, ks[1], dks[1], ha, hb, dha, dhb);
        tangent_combine(pr, ys, dys, y0, dy0, 1, &ks[1], &dks[1], half, dt);
        tangent_rhs(pr, ys, dys, dh_aos, ks[2], dks[2], ha, hb, dha, dhb);
        tangent_combine(pr, ys, dys, y0, dy0, 1, &ks[2], &dks[2], one, dt);
        tangent_rhs(pr, ys, dys, dh_aos, ks[3], dks[3], ha, hb, dha, dhb);
        tangent_combine(pr, ynext, dynext, y0, dy0, 4, ks, dks, w, dt);
        memcpy(y0, ynext, sizeof(double) * n3);
        memcpy(dy0, dynext, sizeof(double) * n3);
        pr->t += dt;
        pr->step += 1.0;
    }
    memcpy(pr->m, y0, sizeof(double) * n3);
    if (dm_out) memcpy(dm_out, dy0, sizeof(double) * n3);
    invalidate_history(pr);
    free(dy0); free(dys); free(ha); free(hb); free(dha); free(dhb); free(ynext); free(dynext);
    for (int s = 0; s < 4; ++s) free(dks[s]);
    return 0;
}

/* Direct real-space sum H_i = -sum_j N(r_i - r_j) Ms m_j over the padded tensor. */
static int demag_direct_periodic(fo_problem *pr, const double *m_aos, double *h_demag) {
    const fo_params *p = &pr->p;
    const int n3[3] = {p->nx, p->ny, p->nz};
    int im[3];
    long reach[3];
    for (int a = 0; a < 3; ++a) {
        im[a] = p->periodic[a] ? (int)p->image_counts[a] : 0;
        reach[a] = (long)n3[a] * (1 + 2 * (long)im[a]);
    }
    newell_ctx c;
    if (newell_ctx_init(&c, reach[0], reach[1], reach[2], p->dx, p->dy, p->dz)) return -2;
    const long n = pr->n;
#pragma omp parallel for schedule(dynamic)
    for (long i = 0; i < n; ++i) {
        double h[3] = {0, 0, 0};
        if (active(pr, i)) {
            const long pi[3] = {i % p->nx, (i / p->nx) % p->ny, i / ((long)p->nx * p->ny)};
            for (long j = 0; j < n; ++j) {
                if (!active(pr, j)) continue;
                const long pj[3] = {j % p->nx, (j / p->nx) % p->ny, j / ((long)p->nx * p->ny)};
                long d[3];
                for (int a = 0; a < 3; ++a) {
                    d[a] = pi[a] - pj[a];
                    if (p->periodic[a] && d[a] < 0) d[a] += n3[a];  /* offset modulo n, in [0, n) */
                }
                double K[6] = {0, 0, 0, 0, 0, 0};
                for (int mz = -im[2]; mz <= im[2]; ++mz)
                    for (int my = -im[1]; my <= im[1]; ++my)
                        for (int mx = -im[0]; mx <= im[0]; ++mx) {
                            double v[6];
                            newell_at(&c, d[0] + (long)mx * p->nx, d[1] + (long)my * p->ny, d[2] + (long)mz * p->nz, v);
                            for (int q = 0; q < 6; ++q) K[q] += v[q];
                        }
                const double Mx = p->ms * m_aos[3 * j], My = p->ms * m_aos[3 * j + 1], Mz = p->ms * m_aos[3 * j + 2];
                h[0] -= K[0] * Mx + K[3] * My + K[4] * Mz;
                h[1] -= K[3] * Mx + K[1] * My + K[5] * Mz;
                h[2] -= K[4] * Mx + K[5] * My + K[2] * Mz;
            }
        }
        for (int q = 0; q < 3; ++q) h_demag[3 * i + q] = h[q];
    }
    free((void *)c.tab);
    return 0;
}

int fo_demag_direct(fo_problem *pr, const double *m_aos, double *h_demag) {
    const fo_params *p = &pr->p;
    if (p->periodic[0] || p->periodic[1] || p->periodic[2]) return demag_direct_periodic(pr, m_aos, h_demag);
    const int nx = p->nx, ny = p->ny, nz = p->nz, px = 2 * nx, py = 2 * ny, pz = 2 * nz;
    const long plen = (long)px * py * pz;
    double *kr = dalloc(6 * plen);
    if (!kr) return -2;
    fo_newell_kernels(nx, ny, nz, p->dx, p->dy, p->dz, kr);
    const long n = pr->n;
#pragma omp parallel for schedule(dynamic)
    for (long i = 0; i < n; ++i) {
        double h[3] = {0, 0, 0};
        if (active(pr, i)) {
            const int xi = (int)(i % nx), yi = (int)((i / nx) % ny), zi = (int)(i / ((long)nx * ny));
            for (long j = 0; j < n; ++j) {
                if (!active(pr, j)) continue;
                const int xj = (int)(j % nx), yj = (int)((j / nx) % ny), zj = (int)(j / ((long)nx * ny));
                const int ddx = (xi - xj + px) % px, ddy = (yi - yj + py) % py, ddz = (zi - zj + pz) % pz;
                const long q = (long)ddx + (long)px * (ddy + (long)py * ddz);
                const double Mx = p->ms * m_aos[3 * j], My = p->ms * m_aos[3 * j + 1], Mz = p->ms * m_aos[3 * j + 2];
                h[0] -= kr[q] * Mx + kr[3 * plen + q] * My + kr[4 * plen + q] * Mz;
                h[1] -= kr[3 * plen + q] * Mx + kr[plen + q] * My + kr[5 * plen + q] * Mz;
                h[2] -= kr[4 * plen + q] * Mx + kr[5 * plen + q] * My + kr[2 * plen + q] * Mz;
            }
        }
        for (int c = 0; c < 3; ++c) h_demag[3 * i + c] = h[c];
    }
    free(kr);
    return 0;
}
