/*
 * lc2_oracle.c -- FP64 CPU restatement of the LC2 similarity path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path. Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load
 * this code. See lc2_oracle.h for the reference file:line each routine
 * follows. Compiled with -ffp-contract=off so results do not depend on
 * whether the host compiler fuses multiply-adds.
 */
#include "lc2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline size_t idx3(const int d[3], int x, int y, int z) {
    return (size_t)x + (size_t)d[0] * ((size_t)y + (size_t)d[1] * (size_t)z);
}

/* ------------------------------------------------------------------------ */
/* Geometry                                                                  */
/* ------------------------------------------------------------------------ */

void or_virtual_geom(int ndim, const or_geom* f, const float* sv, or_geom* out) {
    /* interpolator.cu:337-339 (3D), :1093-1094 (2D): float products, ceil. */
    for (int a = 0; a < 3; ++a) {
        out->origin[a] = f->origin[a];
        out->spacing[a] = sv[a];
        if (a < ndim) {
            float ext = (float)f->dim[a] * f->spacing[a];
            out->dim[a] = (int)ceil((double)(ext / sv[a]));
        } else {
            out->dim[a] = 1;
        }
    }
    if (ndim == 2) {
        out->spacing[2] = 1.0f;
        out->origin[2] = 0.0f;
    }
}

/* ------------------------------------------------------------------------ */
/* Resampling (interpolator.cu:69-232)                                       */
/* ------------------------------------------------------------------------ */

static double sample3(const or_geom* sg, const float* src, double px, double py, double pz) {
    const int* d = sg->dim;
    if (!(px >= 0.0 && px <= (double)(d[0] - 1) && py >= 0.0 && py <= (double)(d[1] - 1) &&
          pz >= 0.0 && pz <= (double)(d[2] - 1)))
        return 0.0;
    int fx = (int)floor(px), fy = (int)floor(py), fz = (int)floor(pz);
    int cx = (int)ceil(px), cy = (int)ceil(py), cz = (int)ceil(pz);
    double rx = px - fx, ry = py - fy, rz = pz - fz;
    /* z, then y, then x (interpolator.cu:96-128) */
    double lu = src[idx3(d, fx, fy, fz)] + rz * ((double)src[idx3(d, fx, fy, cz)] - src[idx3(d, fx, fy, fz)]);
    double ru = src[idx3(d, cx, fy, fz)] + rz * ((double)src[idx3(d, cx, fy, cz)] - src[idx3(d, cx, fy, fz)]);
    double rb = src[idx3(d, cx, cy, fz)] + rz * ((double)src[idx3(d, cx, cy, cz)] - src[idx3(d, cx, cy, fz)]);
    double lb = src[idx3(d, fx, cy, fz)] + rz * ((double)src[idx3(d, fx, cy, cz)] - src[idx3(d, fx, cy, fz)]);
    double l = lu + ry * (lb - lu);
    double r = ru + ry * (rb - ru);
    return l + rx * (r - l);
}

static double sample2(const or_geom* sg, const float* src, double px, double py) {
    const int* d = sg->dim;
    if (!(px >= 0.0 && px <= (double)(d[0] - 1) && py >= 0.0 && py <= (double)(d[1] - 1)))
        return 0.0;
    int fx = (int)floor(px), fy = (int)floor(py);
    int cx = (int)ceil(px), cy = (int)ceil(py);
    double rx = px - fx, ry = py - fy;
    /* y, then x (interpolator.cu:199-207) */
    double xl = src[idx3(d, fx, fy, 0)] + ry * ((double)src[idx3(d, fx, cy, 0)] - src[idx3(d, fx, fy, 0)]);
    double xr = src[idx3(d, cx, fy, 0)] + ry * ((double)src[idx3(d, cx, cy, 0)] - src[idx3(d, cx, fy, 0)]);
    return xl + rx * (xr - xl);
}

void or_resample(int ndim, const or_geom* vg, const or_geom* sg, const float* src,
                 const float* mat, double* out) {
    const int* vd = vg->dim;
    long long total = (long long)vd[0] * vd[1] * vd[2];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < total; ++i) {
        int x = (int)(i % vd[0]);
        int y = (int)((i / vd[0]) % vd[1]);
        int z = (int)(i / ((long long)vd[0] * vd[1]));
        /* virtual pixel -> mm (spatialMappers.cuh:69-83) */
        double lx = x * (double)vg->spacing[0] + vg->origin[0];
        double ly = y * (double)vg->spacing[1] + vg->origin[1];
        if (ndim == 3) {
            double lz = z * (double)vg->spacing[2] + vg->origin[2];
            /* Spatial3DMapper::operator* (spatialMappers.cuh:289-311) */
            double mx = (double)mat[0] * lx + (double)mat[1] * ly + (double)mat[2] * lz + mat[3];
            double my = (double)mat[4] * lx + (double)mat[5] * ly + (double)mat[6] * lz + mat[7];
            double mz = (double)mat[8] * lx + (double)mat[9] * ly + (double)mat[10] * lz + mat[11];
            /* mm -> pixel (spatialMappers.cuh:85-99) */
            double px = (mx - sg->origin[0]) / sg->spacing[0];
            double py = (my - sg->origin[1]) / sg->spacing[1];
            double pz = (mz - sg->origin[2]) / sg->spacing[2];
            out[i] = sample3(sg, src, px, py, pz);
        } else {
            /* Spatial2DMapper::operator* (spatialMappers.cuh:926-942) */
            double mx = (double)mat[0] * lx + (double)mat[1] * ly + mat[2];
            double my = (double)mat[3] * lx + (double)mat[4] * ly + mat[5];
            double px = (mx - sg->origin[0]) / sg->spacing[0];
            double py = (my - sg->origin[1]) / sg->spacing[1];
            out[i] = sample2(sg, src, px, py);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Sobel (cu_lc2_2d.cu:25-86,548-578; cu_lc2_3d.cu:100-179,977-1005)         */
/* ------------------------------------------------------------------------ */

static inline double at0(const int d[3], const double* a, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= d[0] || y >= d[1] || z >= d[2]) return 0.0;
    return a[idx3(d, x, y, z)];
}

void or_sobel(int ndim, const int dim[3], const double* in, double* out) {
    static const double h[3] = {1.0, 2.0, 1.0};
    static const double hp[3] = {-1.0, 0.0, 1.0};
    long long total = (long long)dim[0] * dim[1] * dim[2];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < total; ++i) {
        int x = (int)(i % dim[0]);
        int y = (int)((i / dim[0]) % dim[1]);
        int z = (int)(i / ((long long)dim[0] * dim[1]));
        double gx = 0, gy = 0, gz = 0;
        if (ndim == 2) {
            for (int fy = 0; fy < 3; ++fy)
                for (int fx = 0; fx < 3; ++fx) {
                    double v = at0(dim, in, x + fx - 1, y + fy - 1, z);
                    gx += hp[fx] * h[fy] * v;
                    gy += h[fx] * hp[fy] * v;
                }
            out[i] = sqrt(gx * gx + gy * gy);
        } else {
            for (int fz = 0; fz < 3; ++fz)
                for (int fy = 0; fy < 3; ++fy)
                    for (int fx = 0; fx < 3; ++fx) {
                        double v = at0(dim, in, x + fx - 1, y + fy - 1, z + fz - 1);
                        gx += hp[fx] * h[fy] * h[fz] * v;
                        gy += h[fx] * hp[fy] * h[fz] * v;
                        gz += h[fx] * h[fy] * hp[fz] * v;
                    }
            out[i] = sqrt(gx * gx + gy * gy + gz * gz);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Weighting factor and per-patch measure (direct, two-pass)                */
/* ------------------------------------------------------------------------ */

static int patch_inside(int ndim, const int d[3], int x, int y, int z, int r) {
    if (x - r < 0 || y - r < 0 || x + r >= d[0] || y + r >= d[1]) return 0;
    if (ndim == 3 && (z - r < 0 || z + r >= d[2])) return 0;
    return 1;
}

void or_sigma(int ndim, const int dim[3], int r, const double* U, double* sigma) {
    long long total = (long long)dim[0] * dim[1] * dim[2];
    int rz = (ndim == 3) ? r : 0;
    long long n = (long long)(2 * r + 1) * (2 * r + 1) * (2 * rz + 1);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < total; ++i) {
        int x = (int)(i % dim[0]);
        int y = (int)((i / dim[0]) % dim[1]);
        int z = (int)(i / ((long long)dim[0] * dim[1]));
        double s = 0.0;
        long long cnt = 0;
        /* zero padding outside the grid counts as "not > threshold" */
        for (int dz = -rz; dz <= rz; ++dz)
            for (int dy = -r; dy <= r; ++dy)
                for (int dx = -r; dx <= r; ++dx) {
                    double v = at0(dim, U, x + dx, y + dy, z + dz);
                    if (v > OR_ZERO_THRESHOLD) {
                        ++cnt;
                        s += v;
                    }
                }
        double out = 0.0;
        if (cnt == n) {
            double mean = s / (double)n, var = 0.0;
            for (int dz = -rz; dz <= rz; ++dz)
                for (int dy = -r; dy <= r; ++dy)
                    for (int dx = -r; dx <= r; ++dx) {
                        double v = U[idx3(dim, x + dx, y + dy, z + dz)] - mean;
                        var += v * v;
                    }
            var /= (double)(n - 1);
            if (var > OR_ZERO_THRESHOLD) out = sqrt(var);
        }
        sigma[i] = out;
    }
}

/* Explained sum of squares of the LS fit u ~ a m + b g + c from centred
 * moments, with the rank rule of lc2_oracle.h. */
static double explained_ss(double n, double cmm, double cgg, double cmg, double cum, double cug) {
    int keep_m = cmm / (n - 1.0) > OR_DEGEN_VAR;
    int keep_g = cgg / (n - 1.0) > OR_DEGEN_VAR;
    if (keep_m && keep_g) {
        double det = cmm * cgg - cmg * cmg;
        if (det <= OR_COLLINEAR * cmm * cgg) {
            /* collinear: one direction spans both columns */
            return cum * cum / cmm;
        }
        return (cgg * cum * cum - 2.0 * cmg * cum * cug + cmm * cug * cug) / det;
    }
    if (keep_m) return cum * cum / cmm;
    if (keep_g) return cug * cug / cgg;
    return 0.0;
}

static double clip_measure(double sigma, double expl, double n) {
    double m = expl / ((n - 1.0) * sigma);
    if (isnan(m) || isinf(m) || !(m > 0.0)) return 0.0;
    return m;
}

void or_measure_direct(int ndim, const int dim[3], int r, const double* U, const double* M,
                       const double* G, const double* sigma, double* measure) {
    long long total = (long long)dim[0] * dim[1] * dim[2];
    int rz = (ndim == 3) ? r : 0;
    double n = (double)((2 * r + 1) * (2 * r + 1) * (2 * rz + 1));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < total; ++i) {
        int x = (int)(i % dim[0]);
        int y = (int)((i / dim[0]) % dim[1]);
        int z = (int)(i / ((long long)dim[0] * dim[1]));
        measure[i] = 0.0;
        if (!(sigma[i] > OR_ZERO_THRESHOLD)) continue;
        if (!patch_inside(ndim, dim, x, y, z, r)) continue; /* cu_lc2_3d.cu:787-789 */
        double su = 0, sm = 0, sg = 0;
        for (int dz = -rz; dz <= rz; ++dz)
            for (int dy = -r; dy <= r; ++dy)
                for (int dx = -r; dx <= r; ++dx) {
                    size_t j = idx3(dim, x + dx, y + dy, z + dz);
                    su += U[j];
                    sm += M[j];
                    sg += G[j];
                }
        double mu = su / n, mm = sm / n, mg = sg / n;
        double cmm = 0, cgg = 0, cmg = 0, cum = 0, cug = 0;
        for (int dz = -rz; dz <= rz; ++dz)
            for (int dy = -r; dy <= r; ++dy)
                for (int dx = -r; dx <= r; ++dx) {
                    size_t j = idx3(dim, x + dx, y + dy, z + dz);
                    double u = U[j] - mu, m = M[j] - mm, g = G[j] - mg;
                    cmm += m * m;
                    cgg += g * g;
                    cmg += m * g;
                    cum += u * m;
                    cug += u * g;
                }
        measure[i] = clip_measure(sigma[i], explained_ss(n, cmm, cgg, cmg, cum, cug), n);
    }
}

/* ------------------------------------------------------------------------ */
/* Box-sum path                                                              */
/* ------------------------------------------------------------------------ */

/* In-place zero-padded box sum of half width r along axis `ax`. */
static void box_axis(double* a, const int d[3], int r, int ax, double* scratch_all, int nthr) {
    int n_ax = d[ax];
    long long lines = (long long)d[0] * d[1] * d[2] / n_ax;
    size_t stride = (ax == 0) ? 1 : (ax == 1) ? (size_t)d[0] : (size_t)d[0] * d[1];
#pragma omp parallel for schedule(static) num_threads(nthr)
    for (long long l = 0; l < lines; ++l) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* pre = scratch_all + (size_t)tid * (n_ax + 1);
        size_t base;
        if (ax == 0) {
            base = (size_t)l * d[0];
        } else if (ax == 1) {
            long long x = l % d[0], z = l / d[0];
            base = (size_t)x + (size_t)z * d[0] * d[1];
        } else {
            base = (size_t)l;
        }
        pre[0] = 0.0;
        for (int i = 0; i < n_ax; ++i) pre[i + 1] = pre[i] + a[base + stride * i];
        for (int i = 0; i < n_ax; ++i) {
            int lo = i - r, hi = i + r;
            if (lo < 0) lo = 0;
            if (hi > n_ax - 1) hi = n_ax - 1;
            a[base + stride * i] = pre[hi + 1] - pre[lo];
        }
    }
}

static void box_all(double* a, int ndim, const int d[3], int r, double* scratch, int nthr) {
    box_axis(a, d, r, 0, scratch, nthr);
    box_axis(a, d, r, 1, scratch, nthr);
    if (ndim == 3) box_axis(a, d, r, 2, scratch, nthr);
}

void or_lc2_boxsum(int ndim, const int dim[3], int r, const double* U, const double* M,
                   const double* G, const double* sigma_in, double* measure_out, double* sums,
                   int nthreads) {
    size_t N = (size_t)dim[0] * dim[1] * dim[2];
    int nthr = nthreads;
#ifdef _OPENMP
    if (nthr <= 0) nthr = omp_get_max_threads();
#else
    nthr = 1;
#endif
    int rz = (ndim == 3) ? r : 0;
    double n = (double)((2 * r + 1) * (2 * r + 1) * (2 * rz + 1));
    int maxd = dim[0] > dim[1] ? dim[0] : dim[1];
    if (dim[2] > maxd) maxd = dim[2];
    double* scratch = (double*)malloc(sizeof(double) * (size_t)(maxd + 1) * nthr);
    /* fields: 0 U 1 M 2 G 3 UU 4 MM 5 GG 6 UM 7 UG 8 MG 9 invalid-count */
    double* f[10];
    for (int k = 0; k < 10; ++k) f[k] = (double*)malloc(sizeof(double) * N);
#pragma omp parallel for schedule(static) num_threads(nthr)
    for (long long i = 0; i < (long long)N; ++i) {
        double u = U[i], m = M[i], g = G[i];
        f[0][i] = u; f[1][i] = m; f[2][i] = g;
        f[3][i] = u * u; f[4][i] = m * m; f[5][i] = g * g;
        f[6][i] = u * m; f[7][i] = u * g; f[8][i] = m * g;
        f[9][i] = (u > OR_ZERO_THRESHOLD) ? 0.0 : 1.0;
    }
    for (int k = 0; k < 10; ++k) box_all(f[k], ndim, dim, r, scratch, nthr);

    double sum_m = 0.0, sum_s = 0.0;
#pragma omp parallel for schedule(static) num_threads(nthr) reduction(+ : sum_m, sum_s)
    for (long long i = 0; i < (long long)N; ++i) {
        int x = (int)(i % dim[0]);
        int y = (int)((i / dim[0]) % dim[1]);
        int z = (int)(i / ((long long)dim[0] * dim[1]));
        double sig = 0.0, meas = 0.0;
        if (patch_inside(ndim, dim, x, y, z, r)) {
            if (sigma_in) {
                sig = sigma_in[i];
            } else if (f[9][i] == 0.0) {
                double var = (f[3][i] - f[0][i] * f[0][i] / n) / (n - 1.0);
                if (var > OR_ZERO_THRESHOLD) sig = sqrt(var);
            }
            if (sig > OR_ZERO_THRESHOLD) {
                double cmm = f[4][i] - f[1][i] * f[1][i] / n;
                double cgg = f[5][i] - f[2][i] * f[2][i] / n;
                double cmg = f[8][i] - f[1][i] * f[2][i] / n;
                double cum = f[6][i] - f[0][i] * f[1][i] / n;
                double cug = f[7][i] - f[0][i] * f[2][i] / n;
                meas = clip_measure(sig, explained_ss(n, cmm, cgg, cmg, cum, cug), n);
            }
        }
        if (measure_out) measure_out[i] = meas;
        sum_m += meas;
        sum_s += sig;
    }
    sums[0] = sum_m;
    sums[1] = sum_s;
    for (int k = 0; k < 10; ++k) free(f[k]);
    free(scratch);
}

/* ------------------------------------------------------------------------ */
/* Full evaluation                                                           */
/* ------------------------------------------------------------------------ */

double or_lc2_eval(int resample_ndim, int lc2_ndim, const or_geom* fixed_g, const float* fixed,
                   const or_geom* moving_g, const float* moving, const float* virt_spacing,
                   int r, int hr_moving, const float* mat, int use_boxsum, int nthreads,
                   double* U_out, double* M_out, double* G_out, double* sigma_out,
                   double* measure_out, double* sums_out) {
    or_geom vg;
    or_virtual_geom(resample_ndim, fixed_g, virt_spacing, &vg);
    size_t N = (size_t)vg.dim[0] * vg.dim[1] * vg.dim[2];
    double* vf = (double*)malloc(sizeof(double) * N);
    double* vm = (double*)malloc(sizeof(double) * N);
    double* G = (double*)malloc(sizeof(double) * N);
    double* sig = (double*)malloc(sizeof(double) * N);
    double* meas = (double*)malloc(sizeof(double) * N);
    /* VirtualToFixed is the identity (interpolator.cu:526-528, :1241-1243) */
    float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float ident2[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    or_resample(resample_ndim, &vg, fixed_g, fixed, resample_ndim == 3 ? ident : ident2, vf);
    or_resample(resample_ndim, &vg, moving_g, moving, mat, vm);
    /* roles (interpolator.cu:591-604): the ultrasound is the image that is
     * not the high-resolution modality */
    const double* U = hr_moving ? vf : vm;
    const double* M = hr_moving ? vm : vf;
    or_sobel(lc2_ndim, vg.dim, M, G);
    double sums[2];
    if (use_boxsum) {
        or_lc2_boxsum(lc2_ndim, vg.dim, r, U, M, G, NULL, meas, sums, nthreads);
        if (sigma_out) or_sigma(lc2_ndim, vg.dim, r, U, sigma_out);
    } else {
        or_sigma(lc2_ndim, vg.dim, r, U, sig);
        or_measure_direct(lc2_ndim, vg.dim, r, U, M, G, sig, meas);
        double sm = 0, ss = 0;
        for (size_t i = 0; i < N; ++i) {
            sm += meas[i];
            ss += sig[i];
        }
        sums[0] = sm;
        sums[1] = ss;
        if (sigma_out) memcpy(sigma_out, sig, sizeof(double) * N);
    }
    if (U_out) memcpy(U_out, U, sizeof(double) * N);
    if (M_out) memcpy(M_out, M, sizeof(double) * N);
    if (G_out) memcpy(G_out, G, sizeof(double) * N);
    if (measure_out) memcpy(measure_out, meas, sizeof(double) * N);
    if (sums_out) {
        sums_out[0] = sums[0];
        sums_out[1] = sums[1];
    }
    double lc2 = sums[0] / sums[1];
    if (isnan(lc2) || isinf(lc2)) lc2 = 0.0; /* cu_lc2_3d.cu:1189-1191 */
    free(vf); free(vm); free(G); free(sig); free(meas);
    return lc2;
}

/* ------------------------------------------------------------------------ */
/* Affine builders (spatialMappers.cuh:637-850, :999-1033)                  */
/* ------------------------------------------------------------------------ */

void or_affine3d(const double rot[3], const double trans[3], const double scale[3],
                 const double shear[3], const double center[3], const double shift[3],
                 float out[16]) {
    const double d2r = 3.14159265358979323846 / 180.0;
    double cx = cos(rot[0] * d2r), sx = sin(rot[0] * d2r);
    double cy = cos(rot[1] * d2r), sy = sin(rot[1] * d2r);
    double cz = cos(rot[2] * d2r), sz = sin(rot[2] * d2r);
    double Rx[3][3] = {{1, 0, 0}, {0, cx, -sx}, {0, sx, cx}};
    double Ry[3][3] = {{cy, 0, sy}, {0, 1, 0}, {-sy, 0, cy}};
    double Rz[3][3] = {{cz, -sz, 0}, {sz, cz, 0}, {0, 0, 1}};
    double Sh[3][3] = {{1, shear[0], shear[1]}, {0, 1, shear[2]}, {0, 0, 1}};
    double S[3][3] = {{scale[0], 0, 0}, {0, scale[1], 0}, {0, 0, scale[2]}};
    double A[3][3], B[3][3], L[3][3];
    /* L = Rz Ry Rx Sh S */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            A[i][j] = 0;
            for (int k = 0; k < 3; ++k) A[i][j] += Sh[i][k] * S[k][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            B[i][j] = 0;
            for (int k = 0; k < 3; ++k) B[i][j] += Rx[i][k] * A[k][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            A[i][j] = 0;
            for (int k = 0; k < 3; ++k) A[i][j] += Ry[i][k] * B[k][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            L[i][j] = 0;
            for (int k = 0; k < 3; ++k) L[i][j] += Rz[i][k] * A[k][j];
        }
    for (int i = 0; i < 3; ++i) {
        double t = center[i] + trans[i];
        for (int k = 0; k < 3; ++k) t += L[i][k] * (shift[k] - center[k]);
        for (int j = 0; j < 3; ++j) out[4 * i + j] = (float)L[i][j];
        out[4 * i + 3] = (float)t;
    }
    out[12] = 0.0f; out[13] = 0.0f; out[14] = 0.0f; out[15] = 1.0f;
}

void or_affine2d(double rot, const double trans[2], const double scale[2], double shear,
                 const double center[2], const double shift[2], float out[9]) {
    const double d2r = 3.14159265358979323846 / 180.0;
    double c = cos(rot * d2r), s = sin(rot * d2r);
    /* L = R Sh S, Sh = [[1, sh], [0, 1]] */
    double L[2][2] = {{c * scale[0], scale[1] * (c * shear - s)},
                      {s * scale[0], scale[1] * (s * shear + c)}};
    for (int i = 0; i < 2; ++i) {
        double t = center[i] + trans[i];
        for (int k = 0; k < 2; ++k) t += L[i][k] * (shift[k] - center[k]);
        out[3 * i + 0] = (float)L[i][0];
        out[3 * i + 1] = (float)L[i][1];
        out[3 * i + 2] = (float)t;
    }
    out[6] = 0.0f; out[7] = 0.0f; out[8] = 1.0f;
}

/* ---------------------------------------------------------------- NMI */

static void nmi_bins(const float* v, long long n, int* bins) {
    float lo = v[0], hi = v[0];
    for (long long i = 1; i < n; ++i) {
        if (v[i] < lo) lo = v[i];
        if (v[i] > hi) hi = v[i];
    }
    const float s = hi > lo ? 255.0f / (hi - lo) : 0.0f;
    for (long long i = 0; i < n; ++i) {
        const float t = (v[i] - lo) * s;
        int b = (int)roundf(t);
        bins[i] = b < 0 ? 0 : (b > 255 ? 255 : b);
    }
}

static double entropy_of_counts(const long long* c, int nb, double n) {
    double s = 0.0;
    for (int i = 0; i < nb; ++i)
        if (c[i]) s += (double)c[i] * log((double)c[i]);
    return log(n) - s / n;
}

double or_nmi(const float* U, const float* H, long long n) {
    int* bu = (int*)malloc(sizeof(int) * (size_t)n);
    int* bh = (int*)malloc(sizeof(int) * (size_t)n);
    long long* joint = (long long*)calloc(256 * 256, sizeof(long long));
    long long cu[256] = {0}, ch[256] = {0};
    if (!bu || !bh || !joint) {
        free(bu); free(bh); free(joint);
        return 0.0;
    }
    nmi_bins(U, n, bu);
    nmi_bins(H, n, bh);
    for (long long i = 0; i < n; ++i) {
        ++joint[bu[i] + 256 * bh[i]];
        ++cu[bu[i]];
        ++ch[bh[i]];
    }
    const double hu = entropy_of_counts(cu, 256, (double)n);
    const double hh = entropy_of_counts(ch, 256, (double)n);
    const double hj = entropy_of_counts(joint, 256 * 256, (double)n);
    free(bu); free(bh); free(joint);
    const double v = (hu + hh) / hj;
    return isfinite(v) ? v : 0.0;
}
