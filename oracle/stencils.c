/* C restatement of NPBench's stencil kernels -- TEST INFRASTRUCTURE ONLY.
 *
 * Built by oracle/Makefile into oracle/_build/liboracle.so with
 * -ffp-contract=off (no fused multiply-add) so that every operation rounds
 * exactly as NumPy's elementwise ufuncs do.  Per grid point the operations and
 * their order are those of the reference NumPy kernels:
 *
 *   jacobi_2d  polybench/jacobi_2d/jacobi_2d_numpy.py:6-10
 *              dst = 0.2 * ((((c + w) + e) + s) + n)
 *   heat_3d    polybench/heat_3d/heat_3d_numpy.py:6-20
 *              dst = ((ti + tj) + tk) + c,  tx = 0.125 * ((nx - 2*c) + px)
 *   hdiff      weather_stencils/hdiff/hdiff_numpy.py:5-29
 *   jacobi_1d  polybench/jacobi_1d/jacobi_1d_numpy.py:4-8
 *   fdtd_2d    polybench/fdtd_2d/fdtd_2d_numpy.py:4-11
 *   vadv       weather_stencils/vadv/vadv_numpy.py:9-78
 *
 * so results are bit-identical to the reference.  Each half-sweep is a
 * parallel loop over the slow axis (OpenMP when built with -fopenmp); the
 * order of points does not matter because every point reads only the source
 * array.
 *
 * Arrays are C-ordered; the last axis is contiguous.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

#define DEF_JACOBI(T, SUFFIX, K02)                                              \
  static void jacobi_half_##SUFFIX(const T* src, T* dst, int64_t ny,            \
                                   int64_t nx) {                                \
    _Pragma("omp parallel for schedule(static)")                               \
    for (int64_t i = 1; i < ny - 1; ++i) {                                      \
      const T* r = src + i * nx;                                               \
      const T* rs = r + nx; /* row i+1 */                                      \
      const T* rn = r - nx; /* row i-1 */                                      \
      T* d = dst + i * nx;                                                     \
      for (int64_t j = 1; j < nx - 1; ++j) {                                    \
        T acc = r[j] + r[j - 1];                                               \
        acc = acc + r[j + 1];                                                  \
        acc = acc + rs[j];                                                     \
        acc = acc + rn[j];                                                     \
        d[j] = K02 * acc;                                                      \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  void oracle_jacobi2d_##SUFFIX(T* a, T* b, int64_t ny, int64_t nx,             \
                                int32_t tsteps) {                              \
    if (ny < 3 || nx < 3) return;                                              \
    for (int32_t t = 1; t < tsteps; ++t) {                                     \
      jacobi_half_##SUFFIX(a, b, ny, nx);                                      \
      jacobi_half_##SUFFIX(b, a, ny, nx);                                      \
    }                                                                          \
  }                                                                            \
  void oracle_jacobi2d_half_##SUFFIX(const T* src, T* dst, int64_t ny,          \
                                     int64_t nx) {                             \
    if (ny < 3 || nx < 3) return;                                              \
    jacobi_half_##SUFFIX(src, dst, ny, nx);                                    \
  }

DEF_JACOBI(double, f64, 0.2)
DEF_JACOBI(float, f32, 0.2f)

#define DEF_HEAT(T, SUFFIX, TWO, EIGHTH)                                        \
  static void heat_half_##SUFFIX(const T* src, T* dst, int64_t n0, int64_t n1,  \
                                 int64_t n2) {                                 \
    const int64_t s0 = n1 * n2, s1 = n2;                                       \
    _Pragma("omp parallel for schedule(static)")                               \
    for (int64_t i = 1; i < n0 - 1; ++i) {                                      \
      for (int64_t j = 1; j < n1 - 1; ++j) {                                    \
        const T* p = src + i * s0 + j * s1;                                    \
        T* d = dst + i * s0 + j * s1;                                          \
        for (int64_t k = 1; k < n2 - 1; ++k) {                                  \
          T c = p[k];                                                          \
          T ti = EIGHTH * ((p[k + s0] - TWO * c) + p[k - s0]);                 \
          T tj = EIGHTH * ((p[k + s1] - TWO * c) + p[k - s1]);                 \
          T tk = EIGHTH * ((p[k + 1] - TWO * c) + p[k - 1]);                   \
          d[k] = ((ti + tj) + tk) + c;                                         \
        }                                                                      \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  void oracle_heat3d_##SUFFIX(T* a, T* b, int64_t n0, int64_t n1, int64_t n2,   \
                              int32_t tsteps) {                                \
    if (n0 < 3 || n1 < 3 || n2 < 3) return;                                    \
    for (int32_t t = 1; t < tsteps; ++t) {                                     \
      heat_half_##SUFFIX(a, b, n0, n1, n2);                                    \
      heat_half_##SUFFIX(b, a, n0, n1, n2);                                    \
    }                                                                          \
  }                                                                            \
  void oracle_heat3d_half_##SUFFIX(const T* src, T* dst, int64_t n0,            \
                                   int64_t n1, int64_t n2) {                   \
    if (n0 < 3 || n1 < 3 || n2 < 3) return;                                    \
    heat_half_##SUFFIX(src, dst, n0, n1, n2);                                  \
  }

DEF_HEAT(double, f64, 2.0, 0.125)
DEF_HEAT(float, f32, 2.0f, 0.125f)

/* Laplacian at in-field point (x, y, k): 4*c - (((x+1) + (x-1)) + (y+1)) + (y-1). */
static inline double hd_lap(const double* f, int64_t s0, int64_t s1, int64_t x,
                            int64_t y, int64_t k) {
  const double* p = f + x * s0 + y * s1 + k;
  double nb = p[s0] + p[-s0];
  nb = nb + p[s1];
  nb = nb + p[-s1];
  return 4.0 * p[0] - nb;
}

/* Limited flux between in-field points lo and hi (one step apart along an
 * axis): res = lap(hi) - lap(lo); zero where res * (in(hi) - in(lo)) > 0. */
static inline double hd_flux(double lap_hi, double lap_lo, double in_hi,
                             double in_lo) {
  double res = lap_hi - lap_lo;
  double prod = res * (in_hi - in_lo);
  return (prod > 0) ? 0.0 : res;
}

void oracle_hdiff_f64(const double* in, double* out, const double* coeff,
                      int64_t I, int64_t J, int64_t K) {
  const int64_t s0 = (J + 4) * K, s1 = K;
  _Pragma("omp parallel for schedule(static)")
  for (int64_t i = 0; i < I; ++i) {
    for (int64_t j = 0; j < J; ++j) {
      const int64_t x = i + 2, y = j + 2;
      for (int64_t k = 0; k < K; ++k) {
        const double* p = in + x * s0 + y * s1 + k;
        double lc = hd_lap(in, s0, s1, x, y, k);
        double lxp = hd_lap(in, s0, s1, x + 1, y, k);
        double lxm = hd_lap(in, s0, s1, x - 1, y, k);
        double lyp = hd_lap(in, s0, s1, x, y + 1, k);
        double lym = hd_lap(in, s0, s1, x, y - 1, k);
        double fxp = hd_flux(lxp, lc, p[s0], p[0]);   /* flx_field[i+1, j] */
        double fxm = hd_flux(lc, lxm, p[0], p[-s0]);  /* flx_field[i, j]   */
        double fyp = hd_flux(lyp, lc, p[s1], p[0]);   /* fly_field[i, j+1] */
        double fym = hd_flux(lc, lym, p[0], p[-s1]);  /* fly_field[i, j]   */
        double div = fxp - fxm;
        div = div + fyp;
        div = div - fym;
        out[(i * J + j) * K + k] = p[0] - coeff[(i * J + j) * K + k] * div;
      }
    }
  }
}

/* jacobi_1d: polybench/jacobi_1d/jacobi_1d_numpy.py:4-8
 *   dst[i] = 0.33333 * ((src[i-1] + src[i]) + src[i+1]),  A -> B then B -> A. */
#define DEF_JACOBI1D(T, SUFFIX, K)                                              \
  void oracle_jacobi1d_##SUFFIX(T* a, T* b, int64_t n, int32_t tsteps) {        \
    if (n < 3) return;                                                         \
    for (int32_t t = 1; t < tsteps; ++t) {                                     \
      for (int64_t i = 1; i < n - 1; ++i) b[i] = K * ((a[i - 1] + a[i]) + a[i + 1]); \
      for (int64_t i = 1; i < n - 1; ++i) a[i] = K * ((b[i - 1] + b[i]) + b[i + 1]); \
    }                                                                          \
  }
DEF_JACOBI1D(double, f64, 0.33333)
DEF_JACOBI1D(float, f32, 0.33333f)

/* fdtd_2d: polybench/fdtd_2d/fdtd_2d_numpy.py:4-11, (nx, ny) arrays, per step:
 *   ey[0,:] = fict[t]; ey[i,j] -= 0.5 * (hz[i,j] - hz[i-1,j])  (i >= 1);
 *   ex[i,j] -= 0.5 * (hz[i,j] - hz[i,j-1])  (j >= 1);
 *   hz[i,j] -= 0.7 * (((ex[i,j+1] - ex[i,j]) + ey[i+1,j]) - ey[i,j])  (i < nx-1, j < ny-1). */
#define DEF_FDTD(T, SUFFIX, HALF, C07)                                          \
  void oracle_fdtd2d_##SUFFIX(T* ex, T* ey, T* hz, const T* fict, int64_t nx,    \
                              int64_t ny, int32_t tmax) {                       \
    for (int32_t t = 0; t < tmax; ++t) {                                       \
      for (int64_t j = 0; j < ny; ++j) ey[j] = fict[t];                        \
      _Pragma("omp parallel for schedule(static)")                             \
      for (int64_t i = 1; i < nx; ++i)                                         \
        for (int64_t j = 0; j < ny; ++j)                                       \
          ey[i * ny + j] = ey[i * ny + j] - HALF * (hz[i * ny + j] - hz[(i - 1) * ny + j]); \
      _Pragma("omp parallel for schedule(static)")                             \
      for (int64_t i = 0; i < nx; ++i)                                         \
        for (int64_t j = 1; j < ny; ++j)                                       \
          ex[i * ny + j] = ex[i * ny + j] - HALF * (hz[i * ny + j] - hz[i * ny + j - 1]); \
      _Pragma("omp parallel for schedule(static)")                             \
      for (int64_t i = 0; i < nx - 1; ++i)                                     \
        for (int64_t j = 0; j < ny - 1; ++j) {                                 \
          T d = ex[i * ny + j + 1] - ex[i * ny + j];                           \
          d = d + ey[(i + 1) * ny + j];                                        \
          d = d - ey[i * ny + j];                                              \
          hz[i * ny + j] = hz[i * ny + j] - C07 * d;                           \
        }                                                                      \
    }                                                                          \
  }
DEF_FDTD(double, f64, 0.5, 0.7)
DEF_FDTD(float, f32, 0.5f, 0.7f)

/* vadv: weather_stencils/vadv/vadv_numpy.py:9-78, float64, arrays (I, J, K) with
 * K contiguous and wcon (I+1, J, K).  One (i, j) column at a time: forward
 * elimination over k = 0..K-1, then back substitution into utens_stage.  The
 * operations and their order per level are those of the reference:
 *   w_k = wcon[i+1,j,k] + wcon[i,j,k];  gcv = 0.25*w_{k+1};  gav = -0.25*w_k
 *   cs = ccol_k = gcv*0.5;  as = acol = gav*0.5
 *   bcol = (dtr - acol) - ccol_k
 *   corr = (-as)*(u[k-1]-u[k]) - cs*(u[k+1]-u[k])
 *   dcol_k = ((dtr*u_pos[k] + utens[k]) + utens_stage[k]) + corr
 *   divided = 1.0 / (bcol - ccol_{k-1}*acol)
 *   ccol_k = ccol_k*divided;  dcol_k = (dcol_k - dcol_{k-1}*acol)*divided
 * with the one-sided forms at k = 0 and k = K-1, and
 *   data = dcol_k - ccol_k*data;  utens_stage[k] = dtr*(data - u_pos[k]).
 * Requires K >= 2 (the Python wrapper raises IndexError otherwise). */
void oracle_vadv_f64(double* us, const double* u, const double* wcon, const double* up,
                     const double* ut, double dtr, int64_t I, int64_t J, int64_t K) {
  if (K < 2) return;
  _Pragma("omp parallel for schedule(static)")
  for (int64_t i = 0; i < I; ++i) {
    double* ccol = (double*)malloc(sizeof(double) * (size_t)K * 2);
    double* dcol = ccol + K;
    for (int64_t j = 0; j < J; ++j) {
      const int64_t c = (i * J + j) * K;
      const double* wl = wcon + c;               /* wcon[i, j, :]   */
      const double* wh = wcon + c + J * K;       /* wcon[i+1, j, :] */
      const double* uu = u + c;
      double* s = us + c;
      for (int64_t k = 0; k < K; ++k) {
        double acol = 0.0, as = 0.0, cs = 0.0, bcol, corr;
        if (k + 1 < K) {
          const double gcv = 0.25 * (wh[k + 1] + wl[k + 1]);
          cs = gcv * 0.5;
          ccol[k] = gcv * 0.5;
        }
        if (k > 0) {
          const double gav = -0.25 * (wh[k] + wl[k]);
          as = gav * 0.5;
          acol = gav * 0.5;
        }
        if (k == 0) {
          bcol = dtr - ccol[k];
          corr = (-cs) * (uu[1] - uu[0]);
        } else if (k < K - 1) {
          bcol = (dtr - acol) - ccol[k];
          corr = (-as) * (uu[k - 1] - uu[k]) - cs * (uu[k + 1] - uu[k]);
        } else {
          bcol = dtr - acol;
          corr = (-as) * (uu[k - 1] - uu[k]);
        }
        double d = dtr * up[c + k] + ut[c + k];
        d = d + s[k];
        d = d + corr;
        if (k == 0) {
          const double divided = 1.0 / bcol;
          ccol[k] = ccol[k] * divided;
          dcol[k] = d * divided;
        } else {
          const double divided = 1.0 / (bcol - ccol[k - 1] * acol);
          if (k < K - 1) ccol[k] = ccol[k] * divided;
          dcol[k] = (d - dcol[k - 1] * acol) * divided;
        }
      }
      double data = dcol[K - 1];
      s[K - 1] = dtr * (data - up[c + K - 1]);
      for (int64_t k = K - 2; k >= 0; --k) {
        data = dcol[k] - ccol[k] * data;
        s[k] = dtr * (data - up[c + k]);
      }
    }
    free(ccol);
  }
}
