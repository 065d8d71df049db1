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
 *   cavity_flow  cavity_flow/cavity_flow_numpy.py:13-82
 *   channel_flow channel_flow/channel_flow_numpy.py:13-152
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

/* cavity_flow: cavity_flow/cavity_flow_numpy.py:13-82, float64, arrays (ny, nx).
 * kc holds the scalars the reference forms in Python (its dx**2 is the C
 * library's pow, not always dx*dx), in this order:
 *   two_dx, two_dy, inv_dt, dx2, dy2, pD = 2*(dx2+dy2), pC = dx2*dy2/pD,
 *   k1u = dt/(2*rho*dx), k1v = dt/(2*rho*dy), k2 = dt/dx2, k3 = dt/dy2.
 * Per time step: b from u, v; nit pressure iterations with the reference's
 * four boundary statements in order; u and v from copies un, vn; walls. */
enum { KC_TWO_DX, KC_TWO_DY, KC_INV_DT, KC_DX2, KC_DY2, KC_PD, KC_PC, KC_K1U, KC_K1V, KC_K2,
       KC_K3 };

static double cfd_comp(const double* f, const double* un, const double* vn, double pdiff,
                       int64_t i, int64_t j, int64_t nx, double dt, double dx, double dy,
                       double nu, double k1, const double* kc) {
  const int64_t o = i * nx + j;
  const double fc = f[o];
  const double a = ((un[o] * dt) / dx) * (fc - f[o - 1]);
  const double b = ((vn[o] * dt) / dy) * (fc - f[o - nx]);
  double out = fc - a;
  out = out - b;
  out = out - k1 * pdiff;
  const double two_f = 2.0 * fc;
  const double d1 = kc[KC_K2] * ((f[o + 1] - two_f) + f[o - 1]);
  const double d2 = kc[KC_K3] * ((f[o + nx] - two_f) + f[o - nx]);
  return out + nu * (d1 + d2);
}

void oracle_cavity_flow_f64(double* u, double* v, double* p, int64_t ny, int64_t nx, int32_t nt,
                            int32_t nit, double dt, double dx, double dy, double rho, double nu,
                            const double* kc) {
  const size_t n = (size_t)(ny * nx);
  double* un = (double*)malloc(sizeof(double) * n * 4 + 1);
  double* vn = un + n;
  double* pn = vn + n;
  double* b = pn + n;
  for (size_t q = 0; q < n; ++q) b[q] = 0.0;
  for (int32_t t = 0; t < nt; ++t) {
    for (size_t q = 0; q < n; ++q) { un[q] = u[q]; vn[q] = v[q]; }
    /* build_up_b */
    for (int64_t i = 1; i < ny - 1; ++i)
      for (int64_t j = 1; j < nx - 1; ++j) {
        const int64_t o = i * nx + j;
        const double x1 = (u[o + 1] - u[o - 1]) / kc[KC_TWO_DX];
        const double x2 = (v[o + nx] - v[o - nx]) / kc[KC_TWO_DY];
        double r = kc[KC_INV_DT] * (x1 + x2);
        r = r - x1 * x1;
        double z = (u[o + nx] - u[o - nx]) / kc[KC_TWO_DY];
        z = z * (v[o + 1] - v[o - 1]);
        z = z / kc[KC_TWO_DX];
        r = r - 2.0 * z;
        r = r - x2 * x2;
        b[o] = rho * r;
      }
    /* pressure_poisson */
    for (int32_t q = 0; q < nit; ++q) {
      for (size_t m = 0; m < n; ++m) pn[m] = p[m];
      for (int64_t i = 1; i < ny - 1; ++i)
        for (int64_t j = 1; j < nx - 1; ++j) {
          const int64_t o = i * nx + j;
          double s = (pn[o + 1] + pn[o - 1]) * kc[KC_DY2];
          s = s + (pn[o + nx] + pn[o - nx]) * kc[KC_DX2];
          s = s / kc[KC_PD];
          p[o] = s - kc[KC_PC] * b[o];
        }
      if (nx >= 2)
        for (int64_t i = 0; i < ny; ++i) p[i * nx + nx - 1] = p[i * nx + nx - 2];
      if (ny >= 2)
        for (int64_t j = 0; j < nx; ++j) p[j] = p[nx + j];
      if (nx >= 2)
        for (int64_t i = 0; i < ny; ++i) p[i * nx] = p[i * nx + 1];
      for (int64_t j = 0; j < nx; ++j) p[(ny - 1) * nx + j] = 0.0;
    }
    /* velocities from un, vn and the new p */
    for (int64_t i = 1; i < ny - 1; ++i)
      for (int64_t j = 1; j < nx - 1; ++j) {
        const int64_t o = i * nx + j;
        u[o] = cfd_comp(un, un, vn, p[o + 1] - p[o - 1], i, j, nx, dt, dx, dy, nu, kc[KC_K1U], kc);
        v[o] = cfd_comp(vn, un, vn, p[o + nx] - p[o - nx], i, j, nx, dt, dx, dy, nu, kc[KC_K1V], kc);
      }
    for (int64_t j = 0; j < nx; ++j) u[j] = 0.0;
    for (int64_t i = 0; i < ny; ++i) u[i * nx] = 0.0;
    for (int64_t i = 0; i < ny; ++i) u[i * nx + nx - 1] = 0.0;
    for (int64_t j = 0; j < nx; ++j) u[(ny - 1) * nx + j] = 1.0;
    for (int64_t j = 0; j < nx; ++j) v[j] = 0.0;
    for (int64_t j = 0; j < nx; ++j) v[(ny - 1) * nx + j] = 0.0;
    for (int64_t i = 0; i < ny; ++i) v[i * nx] = 0.0;
    for (int64_t i = 0; i < ny; ++i) v[i * nx + nx - 1] = 0.0;
  }
  free(un);
}

/* NumPy's sum of a contiguous float64 array (np.sum / np.add.reduce): the
 * output starts at +0.0 and receives the pairwise sum of all n elements.  The
 * pairwise sum (NumPy's pairwise_sum for doubles) adds fewer than 8 elements in
 * order from 0.0; up to 128 with 8 running partial sums r[0..7] over
 * consecutive groups of 8, combined as ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)),
 * then the remainder in order; above 128 it splits at n2 = n/2 rounded down to
 * a multiple of 8 and adds the two halves' sums. */
double oracle_pairwise_sum_f64(const double* a, int64_t n) {
  if (n < 8) {
    double res = 0.0;
    for (int64_t i = 0; i < n; ++i) res = res + a[i];
    return res;
  }
  if (n <= 128) {
    double r[8];
    int64_t i;
    for (int j = 0; j < 8; ++j) r[j] = a[j];
    for (i = 8; i < n - (n % 8); i += 8)
      for (int j = 0; j < 8; ++j) r[j] = r[j] + a[i + j];
    double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; ++i) res = res + a[i];
    return res;
  }
  int64_t n2 = n / 2;
  n2 -= n2 % 8;
  return oracle_pairwise_sum_f64(a, n2) + oracle_pairwise_sum_f64(a + n2, n - n2);
}

double oracle_numpy_sum_f64(const double* a, int64_t n) {
  return 0.0 + oracle_pairwise_sum_f64(a, n);
}

/* channel_flow: the cavity_flow arithmetic with periodic columns (the east
 * neighbour of column nx-1 is column 0, the west neighbour of column 0 is
 * column nx-1), u += F*dt (Fdt), pressure walls p[-1] = p[-2] then p[0] = p[1],
 * velocity walls u = v = 0 on rows 0 and -1, looping while
 * (sum(u) - sum(un)) / sum(u) > .001.  Returns the step count, or -1 if
 * max_steps steps did not converge. */
static inline int64_t wrapc(int64_t j, int64_t nx) { return j < 0 ? j + nx : (j >= nx ? j - nx : j); }

int64_t oracle_channel_flow_f64(double* u, double* v, double* p, int64_t ny, int64_t nx,
                                int32_t nit, double dt, double dx, double dy, double rho,
                                double nu, double Fdt, const double* kc, int64_t max_steps) {
  const size_t n = (size_t)(ny * nx);
  double* un = (double*)malloc(sizeof(double) * n * 4 + 1);
  double* vn = un + n;
  double* pn = vn + n;
  double* b = pn + n;
  int64_t steps = 0;
  double udiff = 1.0;
  while (udiff > .001) {
    if (steps >= max_steps) { steps = -1; break; }
    for (size_t q = 0; q < n; ++q) { un[q] = u[q]; vn[q] = v[q]; b[q] = 0.0; }
    for (int64_t i = 1; i < ny - 1; ++i)
      for (int64_t j = 0; j < nx; ++j) {
        const int64_t o = i * nx, je = wrapc(j + 1, nx), jw = wrapc(j - 1, nx);
        const double x1 = (u[o + je] - u[o + jw]) / kc[KC_TWO_DX];
        const double x2 = (v[o + nx + j] - v[o - nx + j]) / kc[KC_TWO_DY];
        double r = kc[KC_INV_DT] * (x1 + x2);
        r = r - x1 * x1;
        double z = (u[o + nx + j] - u[o - nx + j]) / kc[KC_TWO_DY];
        z = z * (v[o + je] - v[o + jw]);
        z = z / kc[KC_TWO_DX];
        r = r - 2.0 * z;
        r = r - x2 * x2;
        b[o + j] = rho * r;
      }
    for (int32_t q = 0; q < nit; ++q) {
      for (size_t m = 0; m < n; ++m) pn[m] = p[m];
      for (int64_t i = 1; i < ny - 1; ++i)
        for (int64_t j = 0; j < nx; ++j) {
          const int64_t o = i * nx;
          double t = (pn[o + wrapc(j + 1, nx)] + pn[o + wrapc(j - 1, nx)]) * kc[KC_DY2];
          t = t + (pn[o + nx + j] + pn[o - nx + j]) * kc[KC_DX2];
          t = t / kc[KC_PD];
          p[o + j] = t - kc[KC_PC] * b[o + j];
        }
      for (int64_t j = 0; j < nx; ++j) p[(ny - 1) * nx + j] = p[(ny - 2) * nx + j];
      for (int64_t j = 0; j < nx; ++j) p[j] = p[nx + j];
    }
    for (int64_t i = 1; i < ny - 1; ++i)
      for (int64_t j = 0; j < nx; ++j) {
        const int64_t o = i * nx, je = wrapc(j + 1, nx), jw = wrapc(j - 1, nx);
        const double uc = un[o + j], vc = vn[o + j];
        const double cu = (uc * dt) / dx, cv = (vc * dt) / dy;
        double ou = uc - cu * (uc - un[o + jw]);
        ou = ou - cv * (uc - un[o - nx + j]);
        ou = ou - kc[KC_K1U] * (p[o + je] - p[o + jw]);
        double d1 = kc[KC_K2] * ((un[o + je] - 2.0 * uc) + un[o + jw]);
        double d2 = kc[KC_K3] * ((un[o + nx + j] - 2.0 * uc) + un[o - nx + j]);
        ou = ou + nu * (d1 + d2);
        u[o + j] = ou + Fdt;
        double ov = vc - cu * (vc - vn[o + jw]);
        ov = ov - cv * (vc - vn[o - nx + j]);
        ov = ov - kc[KC_K1V] * (p[o + nx + j] - p[o - nx + j]);
        d1 = kc[KC_K2] * ((vn[o + je] - 2.0 * vc) + vn[o + jw]);
        d2 = kc[KC_K3] * ((vn[o + nx + j] - 2.0 * vc) + vn[o - nx + j]);
        v[o + j] = ov + nu * (d1 + d2);
      }
    for (int64_t j = 0; j < nx; ++j) {
      u[j] = 0.0;
      u[(ny - 1) * nx + j] = 0.0;
      v[j] = 0.0;
      v[(ny - 1) * nx + j] = 0.0;
    }
    const double su = oracle_numpy_sum_f64(u, (int64_t)n);
    const double sun = oracle_numpy_sum_f64(un, (int64_t)n);
    udiff = (su - sun) / su;
    ++steps;
  }
  free(un);
  return steps;
}
