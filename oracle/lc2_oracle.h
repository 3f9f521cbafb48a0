/*
 * lc2_oracle.h -- FP64 CPU restatement of the LC2 similarity path of
 * LC2Registration (test infrastructure only).
 *
 * This oracle is the checker for the CUDA path: only tests, the smoke entry
 * point and the CPU-baseline leg of the benchmark may call it. Nothing in the
 * product library links or calls it.
 *
 * Every routine follows one reference routine (paths are relative to the
 * reference project root):
 *   or_resample      src/Interpolator/interpolator.cu:69-179 (3D), :181-232 (2D)
 *   or_sobel         src/cu_LC2/cu_lc2_2d.cu:25-86,548-578 (2D)
 *                    src/cu_LC2/cu_lc2_3d.cu:100-179,977-1005 (3D)
 *   or_sigma         src/cu_LC2/cu_lc2_2d.cu:88-180, cu_lc2_3d.cu:181-287
 *   or_measure_*     src/cu_LC2/cu_lc2_2d.cu:182-480, cu_lc2_3d.cu:289-618,769-827
 *                    (CG replaced by the exact least-squares solution, which is
 *                    the CG fixed point; rank-deficient patches use the
 *                    minimum-norm solution, i.e. the projection onto the span
 *                    of the non-degenerate centred columns)
 *   or_lc2_*         src/cu_LC2/cu_lc2_2d.cu:599-653, cu_lc2_3d.cu:1119-1194
 *   or_nmi           src/cu_LC2/cu_lc2_3d.cu:868-923, 1196-1301 (PatchSize 0)
 *
 * All arithmetic is IEEE double. Inputs are float32 volumes, x fastest
 * (index x + y*X + z*X*Y), exactly as the reference stores them.
 */
#ifndef LC2_ORACLE_H
#define LC2_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry of one image/volume: dims, spacing (mm), origin (mm). 2D images
 * use dim[2] = 1. Spacing/origin are the float32 values the reference keeps. */
typedef struct {
    int dim[3];
    float spacing[3];
    float origin[3];
} or_geom;

/* Reference zero threshold (src/cu_LC2/cu_lc2_helper.cuh:5). */
#define OR_ZERO_THRESHOLD 1e-6

/* Rank rule for the exact LS fit, shared with the GPU kernels: a centred column
 * whose sample variance is <= OR_DEGEN_VAR is dropped; two columns whose
 * squared correlation satisfies 1 - rho^2 <= OR_COLLINEAR are treated as one. */
#define OR_DEGEN_VAR 1e-12
#define OR_COLLINEAR 1e-10

/* Resample `src` (geometry sg, float32) onto the virtual grid vg through the
 * row-major 4x4 mm->mm matrix `mat` (virtual mm -> source mm). ndim = 2 uses
 * the top-left 3x3 block of a 2D homogeneous matrix stored in mat[0..8]
 * (row-major 3x3); ndim = 3 uses mat[0..11] of a row-major 4x4. Samples
 * outside [0, dim-1] are 0. Output is double, N = prod(vg.dim). */
void or_resample(int ndim, const or_geom* vg, const or_geom* sg, const float* src,
                 const float* mat, double* out);

/* Unnormalised Sobel gradient magnitude with zero padding.
 * ndim = 2: on each x-y plane (dim[2] must be 1); ndim = 3: full 3x3x3. */
void or_sobel(int ndim, const int dim[3], const double* in, double* out);

/* Weighting factor sigma per voxel: sqrt(sample variance of the (2r+1)^d
 * patch of U) if every patch value (zero padded) is > 1e-6 and the variance
 * is > 1e-6, else 0. Direct two-pass per voxel (small grids). */
void or_sigma(int ndim, const int dim[3], int r, const double* U, double* sigma);

/* Per-voxel clipped measure sigma - var_res/sigma (computed as
 * explained/((n-1) sigma)) for voxels with sigma > 1e-6, else 0. Direct
 * two-pass over each patch (small grids). */
void or_measure_direct(int ndim, const int dim[3], int r, const double* U, const double* M,
                       const double* G, const double* sigma, double* measure);

/* Same result via separable FP64 box sums (O(1) per voxel per moment);
 * OpenMP parallel over slices; used for large grids and the CPU baseline.
 * Recomputes sigma itself when sigma_in is NULL. Returns sums in sums[0]
 * (sum of measures) and sums[1] (sum of sigma). nthreads <= 0: default. */
void or_lc2_boxsum(int ndim, const int dim[3], int r, const double* U, const double* M,
                   const double* G, const double* sigma_in, double* measure_out,
                   double* sums, int nthreads);

/* Full evaluation on the virtual grid: resample fixed (identity) and moving
 * (mat), pick roles by hr_moving (1: moving is the high-resolution image,
 * fixed is the ultrasound), Sobel of the high-resolution image, sigma,
 * measures, LC2 = sum(measure)/sum(sigma) (0 when NaN/Inf).
 * lc2_ndim = 2 for 2D and 2D-to-3D, 3 for 3D; resample_ndim = 2 for 2D,
 * 3 for 3D and 2D-to-3D. Uses box sums when use_boxsum != 0.
 * Optional outputs (may be NULL): U_out, M_out, G_out, sigma_out, measure_out
 * (each N doubles), sums_out[2]. */
double or_lc2_eval(int resample_ndim, int lc2_ndim, const or_geom* fixed_g, const float* fixed,
                   const or_geom* moving_g, const float* moving, const float* virt_spacing,
                   int r, int hr_moving, const float* mat, int use_boxsum, int nthreads,
                   double* U_out, double* M_out, double* G_out, double* sigma_out,
                   double* measure_out, double* sums_out);

/* Normalised mutual information of two float images of n voxels
 * (src/cu_LC2/cu_lc2_3d.cu:868-923, 1196-1301): 256 bins per image between
 * its own min and max, bin = roundf((v - min) * s) with s = 255 / (max - min)
 * in float arithmetic (s = 0 when max == min), joint histogram
 * U-bin + 256 * H-bin, H(X) = -sum p ln p with p = count / n in double.
 * Returns (H(U) + H(H)) / H(U, H), 0 when not finite. */
double or_nmi(const float* U, const float* H, long long n);

/* Virtual grid per src/Interpolator/interpolator.cu:337-339: origin = fixed
 * origin, dims = ceil(dimF*spF/spV) (float arithmetic as in the reference). */
void or_virtual_geom(int ndim, const or_geom* fixed_g, const float* virt_spacing, or_geom* out);

/* Affine builders, FP64 restatement of Spatial3DMapper::AffineInit
 * (src/Interpolator/spatialMappers.cuh:637-850) and Spatial2DMapper::AffineInit
 * (:999-1033): x_m = L (x_v - C + shift) + C + T, L = Rz Ry Rx Sh S.
 * Output row-major float 4x4 (3D) / 3x3 (2D). Angles in degrees. */
void or_affine3d(const double rot[3], const double trans[3], const double scale[3],
                 const double shear[3], const double center[3], const double shift[3],
                 float out[16]);
void or_affine2d(double rot, const double trans[2], const double scale[2], double shear,
                 const double center[2], const double shift[2], float out[9]);

#ifdef __cplusplus
}
#endif
#endif
