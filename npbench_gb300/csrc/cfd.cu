// Lid-driven cavity flow, cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)
// (cavity_flow/cavity_flow_numpy.py:13-82), and channel flow,
// channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)
// (channel_flow/channel_flow_numpy.py:13-152), binary64, arrays (ny, nx).
//
// Per time step the reference runs three kinds of sweeps over the grid, each
// reading its inputs one row and one column around every point:
//   b        build_up_b (:13-21) from u, v;
//   p        nit pressure iterations (:24-38), each from the previous iterate;
//   u, v     the momentum updates (:53-74) from copies un, vn and the new p.
// All of them run here in ONE cooperative persistent launch for the whole
// time loop.  The interior rows are cut into bands, one band per CTA.  A band
// starts sweep s once both neighbouring bands have finished sweep s-1 (their
// counters, published with release semantics after their stores and read
// with acquire semantics), so no grid-wide barrier is needed.  Two buffers
// per field (ping-pong) make that wait enough for write-after-read as well: the
// buffer a sweep overwrites was last read by the neighbours in sweep s-1.
// Grid data that other CTAs wrote is read through L2 (ld.global.cg).  Every
// wait is bounded: after two seconds without the neighbours' progress the CTA
// sets an error word (reported by npbgb_device_status) and returns.
//
// Boundaries.  The reference's pressure boundary statements, in order,
//   p[:, -1] = p[:, -2];  p[0, :] = p[1, :];  p[:, 0] = p[:, 1];  p[-1, :] = 0
// leave every boundary point equal to the new interior value at the clamped
// index (row 0 equal to row 1 including its corners, columns 0 and nx-1 equal
// to columns 1 and nx-2) except row ny-1, which is 0.  So each band computes
// its rows at all nx columns with clamped column indices, and the bands that
// hold rows 1 and ny-2 also write rows 0 and ny-1.  The walls (:75-82) leave u
// = 1 on row ny-1, u = 0 on the other boundary points, and v = 0 on all of them.
//
// Channel flow evaluates the same expressions at every column, the x
// neighbours of columns 0 and nx-1 wrapping around (periodic in x); its
// pressure walls copy row ny-2 to row ny-1 and row 1 to row 0, u gains F*dt,
// and u = v = 0 on rows 0 and ny-1.  It loops while
// (sum(u) - sum(un)) / sum(u) > .001: after each step CTA 0 waits for every
// band, sums u exactly as np.sum does (+0.0 plus NumPy's pairwise sum: blocks
// of at most 128 elements with 8 running sums, halves split at a multiple of 8;
// the blocks are summed in parallel and combined in the tree's order by one
// thread), and publishes a continue/stop word the other bands wait on.  A cap
// on the step count keeps a non-converging input from running forever.
//
// Every operator is one correctly rounded IEEE operation (divisions are
// __ddiv_rn, never multiplication by a reciprocal), in the reference's order,
// with the scalars it forms in Python computed the same way (its dx**2 is the
// C library's pow), so results are bit-identical to NumPy's.  Grids with
// fewer than 3 rows or columns have no interior and take a one-CTA kernel that
// executes the boundary statements literally.
#include "npbgb_common.cuh"

#include <math.h>

#include <vector>

namespace npbgb {

__device__ unsigned int g_cfd_error;  // bit 0: a band waited on its neighbours past the limit

namespace {

constexpr int kCThreads = 256;
constexpr uint64_t kCfdLimitNs = 2000000000ull;

struct CfdConsts {
  double two_dx, two_dy, inv_dt, dx2, dy2, pD, pC, k1u, k1v, k2, k3;
  double dt, dx, dy, rho, nu;
};

struct CfdArgs {
  double* u[2];
  double* v[2];
  double* p[2];
  double* cb;        // pC * b on the interior (b is fixed during the pressure iterations)
  uint32_t* done;    // per band: sweeps completed
  int64_t ny, nx;
  int32_t nt, nit, nbands, rows;
  CfdConsts k;
  // channel_flow only
  double fdt;                  // F * dt
  int64_t max_steps;
  const int64_t* leaf_off;     // np.sum's pairwise blocks of u (offsets, lengths)
  const int32_t* leaf_len;
  int32_t nleaves, nlevels;
  // The pairwise tree's inner nodes, grouped by height: node q (level h holds
  // nodes lvl[h] .. lvl[h+1]-1) sets val[node_out[q]] = val[node_l[q]] +
  // val[node_r[q]].  val[0 .. nleaves) are the blocks' sums; the root is
  // val[root].
  const int32_t* node_l;
  const int32_t* node_r;
  const int32_t* node_out;
  const int32_t* lvl;
  int32_t root;
  double* val;                 // global home of val when it exceeds kSumSmem
  uint32_t* ctl;               // steps allowed to start; kStop bit: finished
  int64_t* steps_out;          // step count (negative: stopped by max_steps)
};

constexpr uint32_t kStop = 0x80000000u;
constexpr int kSumSmem = 4096;   // tree values kept in shared memory up to this many

__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double L(const double* p) { return __ldcg(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until both neighbouring bands have completed `s` sweeps; false on timeout.
__device__ bool wait_neighbours(const uint32_t* done, int b, int nb, uint32_t s) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer();
    int r = 1;
    for (;;) {
      const bool lo = b == 0 || ld_acquire(done + b - 1) >= s;
      const bool hi = b == nb - 1 || ld_acquire(done + b + 1) >= s;
      if (lo && hi) break;
      if (globaltimer() - t0 > kCfdLimitNs) {
        atomicOr(&g_cfd_error, 1u);
        r = 0;
        break;
      }
    }
    ok = r;
  }
  __syncthreads();
  const bool r = ok != 0;
  __syncthreads();
  return r;
}

// bar.sync orders every thread's stores before thread 0's release, and a
// release is cumulative (PTX memory model), so no separate fence is needed.
// The counter counts sweeps, so publishing sweep s is an increment by one; a
// release reduction measured 26% faster per neighbour hand-off on GB300 than a
// release store of s (1.43 against 1.93 us in a chain of 99 bands).
__device__ __forceinline__ void red_release_add(uint32_t* p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void publish(uint32_t* done, int b, uint32_t s) {
  (void)s;  // done[b] == s - 1 here: every band publishes its sweeps in order, once each
  __syncthreads();
  if (threadIdx.x == 0) red_release_add(done + b, 1u);
}

// Points are addressed by their offset o and the offsets oe/ow of their east
// and west neighbours (j+1 and j-1, wrapped around for channel flow).

// build_up_b at interior (i, j), times pC (cavity_flow_numpy.py:15-21, 31-33;
// channel_flow_numpy.py:14-39).
__device__ __forceinline__ double cb_point(const double* u, const double* v, int64_t o, int64_t oe,
                                           int64_t ow, int64_t nx, const CfdConsts& k) {
  const double x1 = ddiv(sub_rn(L(u + oe), L(u + ow)), k.two_dx);
  const double x2 = ddiv(sub_rn(L(v + o + nx), L(v + o - nx)), k.two_dy);
  double r = mul_rn(k.inv_dt, add_rn(x1, x2));
  r = sub_rn(r, mul_rn(x1, x1));
  double z = ddiv(sub_rn(L(u + o + nx), L(u + o - nx)), k.two_dy);
  z = mul_rn(z, sub_rn(L(v + oe), L(v + ow)));
  z = ddiv(z, k.two_dx);
  r = sub_rn(r, mul_rn(2.0, z));
  r = sub_rn(r, mul_rn(x2, x2));
  return mul_rn(k.pC, mul_rn(k.rho, r));
}

// One pressure iterate at interior (i, j) (cavity_flow_numpy.py:30-33;
// channel_flow_numpy.py:47-63).
__device__ __forceinline__ double p_point(const double* x, const double* cb, int64_t o, int64_t oe,
                                          int64_t ow, int64_t nx, const CfdConsts& k) {
  double s = mul_rn(add_rn(L(x + oe), L(x + ow)), k.dy2);
  s = add_rn(s, mul_rn(add_rn(L(x + o + nx), L(x + o - nx)), k.dx2));
  s = ddiv(s, k.pD);
  return sub_rn(s, L(cb + o));
}

// The momentum update of field f (un or vn) at interior (i, j)
// (cavity_flow_numpy.py:53-74; channel_flow_numpy.py:80-143); cu = (un*dt)/dx
// and cv = (vn*dt)/dy at the point.
__device__ __forceinline__ double f_point(const double* f, double fc, double cu, double cv,
                                          double pdiff, double k1, int64_t o, int64_t oe,
                                          int64_t ow, int64_t nx, const CfdConsts& k) {
  const double a = mul_rn(cu, sub_rn(fc, L(f + ow)));
  const double b = mul_rn(cv, sub_rn(fc, L(f + o - nx)));
  double out = sub_rn(sub_rn(sub_rn(fc, a), b), mul_rn(k1, pdiff));
  const double two_f = mul_rn(2.0, fc);
  const double d1 = mul_rn(k.k2, add_rn(sub_rn(L(f + oe), two_f), L(f + ow)));
  const double d2 = mul_rn(k.k3, add_rn(sub_rn(L(f + o + nx), two_f), L(f + o - nx)));
  return add_rn(out, mul_rn(k.nu, add_rn(d1, d2)));
}

// np.sum(u) by the whole CTA; the result is valid in thread 0.  Each block of
// NumPy's pairwise summation (at most 128 elements) goes to a group of 8
// lanes: lane q keeps NumPy's running sum r[q] over elements q, q+8, ... (one
// coalesced 64-byte row of the block per step), the group combines them as
// ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)) with shuffles, and lane 0 adds the
// remainder in order.  The blocks' sums are then combined up the tree, one
// level at a time, each inner node as (left + right), in shared memory when
// the tree fits.  (Below 8 elements in all, NumPy adds them in order from 0.0.)
__device__ double numpy_sum_cta(const CfdArgs& a, const double* u) {
  __shared__ double sval[kSumSmem];
  double* val = 2 * a.nleaves - 1 <= kSumSmem ? sval : a.val;
  const int q = threadIdx.x & 7, grp = threadIdx.x >> 3;
  for (int32_t base = 0; base < a.nleaves; base += kCThreads / 8) {
    const int32_t l = base + grp;
    const bool live = l < a.nleaves;
    const int32_t n = live ? a.leaf_len[l] : 0;
    const double* x = u + (live ? a.leaf_off[l] : 0);
    double r = 0.0;
    if (n >= 8) {
      double v[16];
      const int32_t groups = n / 8;
#pragma unroll
      for (int g = 0; g < 16; ++g) v[g] = g < groups ? L(x + 8 * g + q) : 0.0;
      r = v[0];
#pragma unroll
      for (int g = 1; g < 16; ++g)
        if (g < groups) r = add_rn(r, v[g]);
    }
    const double s2 = add_rn(r, __shfl_down_sync(0xffffffffu, r, 1, 8));
    const double s4 = add_rn(s2, __shfl_down_sync(0xffffffffu, s2, 2, 8));
    const double s8 = add_rn(s4, __shfl_down_sync(0xffffffffu, s4, 4, 8));
    if (live && q == 0) {
      double res = n >= 8 ? s8 : 0.0;
      for (int32_t i = n >= 8 ? n - n % 8 : 0; i < n; ++i) res = add_rn(res, L(x + i));
      val[l] = res;
    }
  }
  __syncthreads();
  for (int32_t h = 0; h < a.nlevels; ++h) {
    for (int32_t k = a.lvl[h] + threadIdx.x; k < a.lvl[h + 1]; k += kCThreads)
      val[a.node_out[k]] = add_rn(val[a.node_l[k]], val[a.node_r[k]]);
    __syncthreads();
  }
  const double total = add_rn(0.0, val[a.root]);
  __syncthreads();
  return total;
}

// Channel flow: CTA 0 waits for every band to finish sweep s, then decides
// whether step n+1 runs.  false on timeout.
__device__ bool channel_decide(const CfdArgs& a, uint32_t s, int32_t n, const double* u,
                               double& s_prev) {
  // One thread per band counter, so the polls overlap.
  int r = 1;
  const uint64_t t0 = globaltimer();
  for (int bb = threadIdx.x; bb < a.nbands && r; bb += kCThreads)
    while (ld_acquire(a.done + bb) < s) {
      if (globaltimer() - t0 > kCfdLimitNs) {
        atomicOr(&g_cfd_error, 1u);
        r = 0;
        break;
      }
    }
  if (!__syncthreads_and(r)) return false;
  const double su = numpy_sum_cta(a, u);
  if (threadIdx.x == 0) {
    const double udiff = ddiv(sub_rn(su, s_prev), su);
    s_prev = su;
    const int64_t steps = int64_t(n) + 1;
    const bool more = udiff > 0.001;
    uint32_t word;
    if (!more) {
      *a.steps_out = steps;
      word = kStop | uint32_t(steps);
    } else if (steps >= a.max_steps) {
      *a.steps_out = -steps;
      word = kStop | uint32_t(steps);
    } else {
      word = uint32_t(steps);
    }
    __threadfence();
    st_release(a.ctl, word);
  }
  __syncthreads();
  return true;
}

// Waits for the decision on step n; 1 = run it, 0 = stop, -1 = timeout.
__device__ int wait_step(const CfdArgs& a, int32_t n) {
  __shared__ int st;
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer();
    int r;
    for (;;) {
      const uint32_t w = ld_acquire(a.ctl);
      if (w & kStop) { r = 0; break; }
      if (w >= uint32_t(n)) { r = 1; break; }
      if (globaltimer() - t0 > kCfdLimitNs) {
        atomicOr(&g_cfd_error, 1u);
        r = -1;
        break;
      }
    }
    st = r;
  }
  __syncthreads();
  const int r = st;
  __syncthreads();
  return r;
}

template <bool CH>
__global__ void __launch_bounds__(kCThreads)
cfd_bands(CfdArgs a) {
  const int b = blockIdx.x;
  const int64_t ny = a.ny, nx = a.nx;
  const int64_t r0 = 1 + int64_t(b) * a.rows;
  const int64_t r1 = r0 + a.rows < ny - 1 ? r0 + a.rows : ny - 1;
  const CfdConsts& k = a.k;
  // Neighbour columns: wrapped (channel) or plain (cavity, interior columns only).
  auto east = [&](int64_t j) { return CH ? (j + 1 == nx ? 0 : j + 1) : j + 1; };
  auto west = [&](int64_t j) { return CH ? (j == 0 ? nx - 1 : j - 1) : j - 1; };
  uint32_t s = 0;  // sweeps completed by this band
  int cu = 0, pc = 0;
  double s_prev = 0.0;  // channel flow, CTA 0: np.sum of the previous u
  if (CH && b == 0) s_prev = numpy_sum_cta(a, a.u[0]);
  const int32_t steps = CH ? 0x7fffffff : a.nt;
  for (int32_t n = 0; n < steps; ++n) {
    if (CH && n > 0) {
      const int w = wait_step(a, n);
      if (w < 0) return;
      if (w == 0) break;
    }
    // b (as pC*b) from u, v.
    if (!wait_neighbours(a.done, b, a.nbands, s)) return;
    {
      const double* u = a.u[cu];
      const double* v = a.v[cu];
      for (int64_t i = r0; i < r1; ++i)
        for (int64_t j = (CH ? 0 : 1) + threadIdx.x; j < (CH ? nx : nx - 1); j += kCThreads)
          a.cb[i * nx + j] = cb_point(u, v, i * nx + j, i * nx + east(j), i * nx + west(j), nx, k);
    }
    publish(a.done, b, ++s);
    // Pressure iterations.
    for (int32_t q = 0; q < a.nit; ++q) {
      if (!wait_neighbours(a.done, b, a.nbands, s)) return;
      const double* x = a.p[pc];
      double* y = a.p[pc ^ 1];
      for (int64_t i = r0; i < r1; ++i)
        for (int64_t j = threadIdx.x; j < nx; j += kCThreads) {
          const int64_t jj = CH ? j : (j < 1 ? 1 : (j > nx - 2 ? nx - 2 : j));
          const double val =
              p_point(x, a.cb, i * nx + jj, i * nx + east(jj), i * nx + west(jj), nx, k);
          y[i * nx + j] = val;
          if (i == 1) y[j] = val;                                     // row 0 = row 1
          if (i == ny - 2) y[(ny - 1) * nx + j] = CH ? val : 0.0;     // row ny-1
        }
      pc ^= 1;
      publish(a.done, b, ++s);
    }
    // u and v from un = u[cu], vn = v[cu] and p[pc].
    if (!wait_neighbours(a.done, b, a.nbands, s)) return;
    {
      const double* un = a.u[cu];
      const double* vn = a.v[cu];
      const double* p = a.p[pc];
      double* uo = a.u[cu ^ 1];
      double* vo = a.v[cu ^ 1];
      for (int64_t i = r0; i < r1; ++i)
        for (int64_t j = threadIdx.x; j < nx; j += kCThreads) {
          const int64_t o = i * nx + j;
          double nu_ = 0.0, nv_ = 0.0;
          if (CH || (j >= 1 && j < nx - 1)) {
            const int64_t oe = i * nx + east(j), ow = i * nx + west(j);
            const double uc = L(un + o), vc = L(vn + o);
            const double cu_ = ddiv(mul_rn(uc, k.dt), k.dx);
            const double cv_ = ddiv(mul_rn(vc, k.dt), k.dy);
            nu_ = f_point(un, uc, cu_, cv_, sub_rn(L(p + oe), L(p + ow)), k.k1u, o, oe, ow, nx, k);
            if (CH) nu_ = add_rn(nu_, a.fdt);
            nv_ = f_point(vn, vc, cu_, cv_, sub_rn(L(p + o + nx), L(p + o - nx)), k.k1v, o, oe,
                          ow, nx, k);
          }
          uo[o] = nu_;
          vo[o] = nv_;
          if (i == 1) {
            uo[j] = 0.0;
            vo[j] = 0.0;
          }
          if (i == ny - 2) {
            uo[(ny - 1) * nx + j] = CH ? 0.0 : 1.0;
            vo[(ny - 1) * nx + j] = 0.0;
          }
        }
    }
    cu ^= 1;
    publish(a.done, b, ++s);
    if (CH && b == 0 && !channel_decide(a, s, n, a.u[cu], s_prev)) return;
  }
  // Results that ended in the second buffers go back to the caller's arrays,
  // once the neighbours no longer read the caller's buffers (channel flow:
  // every band has finished, or CTA 0 would not have stopped the loop).
  if (cu == 0 && pc == 0) return;
  if (!CH && !wait_neighbours(a.done, b, a.nbands, s)) return;
  const int64_t lo = r0 == 1 ? 0 : r0, hi = r1 == ny - 1 ? ny : r1;
  for (int64_t o = lo * nx + threadIdx.x; o < hi * nx; o += kCThreads) {
    if (cu) {
      a.u[0][o] = L(a.u[1] + o);
      a.v[0][o] = L(a.v[1] + o);
    }
    if (pc) a.p[0][o] = L(a.p[1] + o);
  }
}

// Grids with fewer than 3 rows or columns: no interior point exists, so b and
// the interior updates are empty and only the boundary statements act; one CTA
// runs them in the reference's order.
__global__ void __launch_bounds__(kCThreads)
cavity_literal(double* u, double* v, double* p, int64_t ny, int64_t nx, int32_t nt, int32_t nit) {
  const int tid = threadIdx.x;
  for (int32_t n = 0; n < nt; ++n) {
    for (int32_t q = 0; q < nit; ++q) {
      for (int64_t i = tid; i < ny; i += kCThreads) p[i * nx + nx - 1] = p[i * nx + nx - 2];
      __syncthreads();
      for (int64_t j = tid; j < nx; j += kCThreads) p[j] = p[nx + j];
      __syncthreads();
      for (int64_t i = tid; i < ny; i += kCThreads) p[i * nx] = p[i * nx + 1];
      __syncthreads();
      for (int64_t j = tid; j < nx; j += kCThreads) p[(ny - 1) * nx + j] = 0.0;
      __syncthreads();
    }
    for (int64_t o = tid; o < ny * nx; o += kCThreads) {
      u[o] = o / nx == ny - 1 ? 1.0 : 0.0;
      v[o] = 0.0;
    }
    __syncthreads();
  }
}

// Channel flow with fewer than 3 rows: no interior, so every step leaves
// u = v = 0 (all rows are walls) and, with nit >= 1, copies row 0 of p to
// row 1.  The first step's udiff is (0 - sum(u0)) / 0, which continues only
// for sum(u0) < 0; the second is 0/0 = NaN and stops.  One CTA computes
// sum(u0) as np.sum does and applies that.
__global__ void __launch_bounds__(kCThreads)
channel_small(CfdArgs a) {
  const double s0 = numpy_sum_cta(a, a.u[0]);
  const int64_t n = a.ny * a.nx;
  for (int64_t o = threadIdx.x; o < n; o += kCThreads) {
    a.u[0][o] = 0.0;
    a.v[0][o] = 0.0;
  }
  if (a.nit > 0 && a.ny == 2)
    for (int64_t j = threadIdx.x; j < a.nx; j += kCThreads) a.p[0][a.nx + j] = a.p[0][j];
  if (threadIdx.x == 0) *a.steps_out = s0 < 0.0 ? (a.max_steps >= 2 ? 2 : -1) : 1;
}

// The scalars the reference forms with Python floats.  Python's x**2 calls
// the C library's pow (not always the correctly rounded x*x), so pow is called
// through a volatile pointer that the compiler cannot fold into x*x.
CfdConsts make_consts(double dt, double dx, double dy, double rho, double nu) {
  double (*volatile pw)(double, double) = ::pow;
  CfdConsts k;
  const double dx2 = pw(dx, 2.0), dy2 = pw(dy, 2.0);
  volatile double t;  // keeps every product and sum separately rounded
  k.two_dx = 2.0 * dx;
  k.two_dy = 2.0 * dy;
  k.inv_dt = 1.0 / dt;
  k.dx2 = dx2;
  k.dy2 = dy2;
  t = dx2 + dy2;
  k.pD = 2.0 * t;
  t = dx2 * dy2;
  k.pC = t / k.pD;
  t = 2.0 * rho;
  t = t * dx;
  k.k1u = dt / t;
  t = 2.0 * rho;
  t = t * dy;
  k.k1v = dt / t;
  k.k2 = dt / dx2;
  k.k3 = dt / dy2;
  k.dt = dt;
  k.dx = dx;
  k.dy = dy;
  k.rho = rho;
  k.nu = nu;
  return k;
}

}  // namespace

uint32_t take_cfd_device_error() {
  uint32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_cfd_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  if (v) cudaMemcpyToSymbol(g_cfd_error, &zero, sizeof(zero));
  return v;
}

}  // namespace npbgb

namespace {
int64_t cfd_bands(int64_t ny) {
  const int64_t interior = ny - 2;
  if (interior <= 0) return 0;
  const int64_t sms = npbgb::sm_count();
  const int64_t rows = npbgb::cdiv(interior, sms < interior ? sms : interior);
  return npbgb::cdiv(interior, rows);
}
constexpr int64_t kAlign = 256;
int64_t round_up(int64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
}  // namespace

extern "C" int64_t npbgb_cavity_flow_workspace_bytes(int64_t ny, int64_t nx) {
  if (ny <= 0 || nx <= 0) return 0;
  const int64_t field = round_up(ny * nx * int64_t(sizeof(double)));
  return 4 * field + round_up(cfd_bands(ny) * int64_t(sizeof(uint32_t)));
}

extern "C" int32_t npbgb_cavity_flow(void* u, void* v, void* p, int64_t ny, int64_t nx, int32_t nt,
                                     int32_t nit, double dt, double dx, double dy, double rho,
                                     double nu, int32_t dtype, void* workspace,
                                     int64_t workspace_bytes, void* stream) {
  using namespace npbgb;
  if (dtype != NPBGB_F64) return set_error(NPBGB_ERR_DTYPE, "cavity_flow: binary64 only");
  if (ny < 0 || nx < 0 || nt < 0 || nit < 0)
    return set_error(NPBGB_ERR_ARG, "cavity_flow: negative extent or count");
  // The reference indexes row/column 0 in its wall statements and rows/columns
  // 1 and -2 in its pressure boundaries: IndexError below these sizes.
  if (nt > 0 && (ny < 1 || nx < 1 || (nit > 0 && (ny < 2 || nx < 2))))
    return set_error(NPBGB_ERR_ARG, "cavity_flow: ny = %lld, nx = %lld is too small for the "
                     "boundary statements", (long long)ny, (long long)nx);
  if (nt == 0) return NPBGB_OK;
  if (!u || !v || !p) return set_error(NPBGB_ERR_ARG, "cavity_flow: null array");
  if (u == v || u == p || v == p) return set_error(NPBGB_ERR_ARG, "cavity_flow: aliased arrays");
  cudaStream_t st = as_stream(stream);
  if (ny < 3 || nx < 3) {
    cavity_literal<<<1, kCThreads, 0, st>>>(static_cast<double*>(u), static_cast<double*>(v),
                                             static_cast<double*>(p), ny, nx, nt, nit);
    NPBGB_CHECK_LAUNCH("cavity_literal");
    return NPBGB_OK;
  }
  const int64_t need = npbgb_cavity_flow_workspace_bytes(ny, nx);
  void* ws = workspace;
  if (ws != nullptr && workspace_bytes < need)
    return set_error(NPBGB_ERR_ARG, "cavity_flow: workspace of %lld bytes, %lld needed",
                     (long long)workspace_bytes, (long long)need);
  if (ws == nullptr) {
    cudaError_t e = cudaMallocAsync(&ws, size_t(need), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(NPBGB_ERR_NOMEM, "cavity_flow: workspace of %lld bytes: %s",
                       (long long)need, cudaGetErrorString(e));
    }
  }
  const int64_t nb = cfd_bands(ny);
  const int64_t field = round_up(ny * nx * int64_t(sizeof(double)));
  char* w = static_cast<char*>(ws);
  CfdArgs a;
  a.u[0] = static_cast<double*>(u);
  a.v[0] = static_cast<double*>(v);
  a.p[0] = static_cast<double*>(p);
  a.u[1] = reinterpret_cast<double*>(w);
  a.v[1] = reinterpret_cast<double*>(w + field);
  a.p[1] = reinterpret_cast<double*>(w + 2 * field);
  a.cb = reinterpret_cast<double*>(w + 3 * field);
  a.done = reinterpret_cast<uint32_t*>(w + 4 * field);
  a.ny = ny;
  a.nx = nx;
  a.nt = nt;
  a.nit = nit;
  a.nbands = int32_t(nb);
  a.rows = int32_t(cdiv(ny - 2, nb));
  a.k = make_consts(dt, dx, dy, rho, nu);
  int32_t status = NPBGB_OK;
  cudaError_t e = cudaMemsetAsync(a.done, 0, size_t(nb) * sizeof(uint32_t), st);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3{unsigned(nb), 1, 1};
    cfg.blockDim = dim3{unsigned(kCThreads), 1, 1};
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {&a};
    e = counted(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(cfd_bands<false>), args));
  }
  if (e != cudaSuccess) status = cuda_status(e, "cavity_flow: cooperative launch");
  if (workspace == nullptr) cudaFreeAsync(ws, st);
  return status;
}

namespace {
// np.sum's pairwise tree over n elements: blocks of at most 128 in order
// (values 0 .. L-1) and inner nodes, each (left + right), with their heights.
struct SumTree {
  std::vector<int64_t> leaf_off;
  std::vector<int32_t> leaf_len;
  std::vector<int64_t> in_l, in_r;   // children: >= 0 a block, < 0 ~(inner node)
  std::vector<int32_t> in_h;
};

int64_t build_tree(int64_t off, int64_t n, SumTree& t, int32_t& height) {
  if (n <= 128) {
    t.leaf_off.push_back(off);
    t.leaf_len.push_back(int32_t(n));
    height = 0;
    return int64_t(t.leaf_off.size()) - 1;
  }
  int64_t n2 = n / 2;
  n2 -= n2 % 8;
  int32_t hl = 0, hr = 0;
  const int64_t l = build_tree(off, n2, t, hl);
  const int64_t r = build_tree(off + n2, n - n2, t, hr);
  height = (hl > hr ? hl : hr) + 1;
  t.in_l.push_back(l);
  t.in_r.push_back(r);
  t.in_h.push_back(height);
  return ~int64_t(t.in_l.size() - 1);
}

// Device-ready form: value index of block k is k, of inner node m is L + m;
// nodes sorted by height.
struct SumPlan {
  std::vector<int64_t> leaf_off;
  std::vector<int32_t> leaf_len, node_l, node_r, node_out, lvl;
  int32_t root = 0;
};

SumPlan sum_plan(int64_t n) {
  SumTree t;
  int32_t h = 0;
  const int64_t root = build_tree(0, n, t, h);
  SumPlan p;
  const int64_t L = int64_t(t.leaf_off.size());
  auto vidx = [&](int64_t ref) { return int32_t(ref >= 0 ? ref : L + ~ref); };
  p.leaf_off = std::move(t.leaf_off);
  p.leaf_len = std::move(t.leaf_len);
  p.root = vidx(root);
  p.lvl.push_back(0);
  for (int32_t level = 1; level <= h; ++level) {
    for (size_t m = 0; m < t.in_h.size(); ++m)
      if (t.in_h[m] == level) {
        p.node_l.push_back(vidx(t.in_l[m]));
        p.node_r.push_back(vidx(t.in_r[m]));
        p.node_out.push_back(int32_t(L + int64_t(m)));
      }
    p.lvl.push_back(int32_t(p.node_l.size()));
  }
  return p;
}

struct ChannelLayout {
  int64_t field, nb, nleaves, nnodes, nlevels, off_done, off_leaf_off, off_leaf_len, off_node_l,
      off_node_r, off_node_out, off_lvl, off_val, off_ctl, off_steps, total;
};

ChannelLayout channel_layout(int64_t ny, int64_t nx, const SumPlan& p) {
  ChannelLayout l{};
  l.nleaves = int64_t(p.leaf_off.size());
  l.nnodes = int64_t(p.node_l.size());
  l.nlevels = int64_t(p.lvl.size()) - 1;
  l.field = round_up(ny * nx * int64_t(sizeof(double)));
  l.nb = cfd_bands(ny);
  int64_t o = 4 * l.field;
  l.off_done = o;      o += round_up((l.nb > 0 ? l.nb : 1) * 4);
  l.off_leaf_off = o;  o += round_up(l.nleaves * 8);
  l.off_leaf_len = o;  o += round_up(l.nleaves * 4);
  l.off_node_l = o;    o += round_up((l.nnodes > 0 ? l.nnodes : 1) * 4);
  l.off_node_r = o;    o += round_up((l.nnodes > 0 ? l.nnodes : 1) * 4);
  l.off_node_out = o;  o += round_up((l.nnodes > 0 ? l.nnodes : 1) * 4);
  l.off_lvl = o;       o += round_up((l.nlevels + 1) * 4);
  l.off_val = o;       o += round_up((l.nleaves + l.nnodes) * 8);
  l.off_ctl = o;       o += kAlign;
  l.off_steps = o;     o += kAlign;
  l.total = o;
  return l;
}
}  // namespace

extern "C" int64_t npbgb_channel_flow_workspace_bytes(int64_t ny, int64_t nx) {
  if (ny <= 0 || nx <= 0) return 0;
  return channel_layout(ny, nx, sum_plan(ny * nx)).total;
}

extern "C" int32_t npbgb_channel_flow(void* u, void* v, void* p, int64_t ny, int64_t nx,
                                      int32_t nit, double dt, double dx, double dy, double rho,
                                      double nu, double F, int64_t max_steps, int32_t dtype,
                                      void* workspace, int64_t workspace_bytes, int64_t* steps,
                                      void* stream) {
  using namespace npbgb;
  if (dtype != NPBGB_F64) return set_error(NPBGB_ERR_DTYPE, "channel_flow: binary64 only");
  if (nit < 0 || max_steps < 1) return set_error(NPBGB_ERR_ARG, "channel_flow: nit < 0 or max_steps < 1");
  // The reference indexes column -2 (periodic boundaries), row 0 (walls) and,
  // with nit >= 1, row -2 (pressure walls): IndexError below these sizes.
  if (nx < 2 || ny < 1 || (nit > 0 && ny < 2))
    return set_error(NPBGB_ERR_ARG, "channel_flow: ny = %lld, nx = %lld is too small for the "
                     "boundary statements", (long long)ny, (long long)nx);
  if (!u || !v || !p) return set_error(NPBGB_ERR_ARG, "channel_flow: null array");
  if (u == v || u == p || v == p) return set_error(NPBGB_ERR_ARG, "channel_flow: aliased arrays");
  if (max_steps > 0x7fffffff) max_steps = 0x7fffffff;
  cudaStream_t st = as_stream(stream);
  const SumPlan plan = sum_plan(ny * nx);
  const ChannelLayout l = channel_layout(ny, nx, plan);
  void* ws = workspace;
  if (ws != nullptr && workspace_bytes < l.total)
    return set_error(NPBGB_ERR_ARG, "channel_flow: workspace of %lld bytes, %lld needed",
                     (long long)workspace_bytes, (long long)l.total);
  if (ws == nullptr) {
    cudaError_t e = cudaMallocAsync(&ws, size_t(l.total), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(NPBGB_ERR_NOMEM, "channel_flow: workspace of %lld bytes: %s",
                       (long long)l.total, cudaGetErrorString(e));
    }
  }
  char* w = static_cast<char*>(ws);
  CfdArgs a{};
  a.u[0] = static_cast<double*>(u);
  a.v[0] = static_cast<double*>(v);
  a.p[0] = static_cast<double*>(p);
  a.u[1] = reinterpret_cast<double*>(w);
  a.v[1] = reinterpret_cast<double*>(w + l.field);
  a.p[1] = reinterpret_cast<double*>(w + 2 * l.field);
  a.cb = reinterpret_cast<double*>(w + 3 * l.field);
  a.done = reinterpret_cast<uint32_t*>(w + l.off_done);
  a.ny = ny;
  a.nx = nx;
  a.nt = 0;
  a.nit = nit;
  a.nbands = int32_t(l.nb);
  a.rows = l.nb > 0 ? int32_t(cdiv(ny - 2, l.nb)) : 0;
  a.k = make_consts(dt, dx, dy, rho, nu);
  volatile double fdt = F * dt;
  a.fdt = fdt;
  a.max_steps = max_steps;
  a.leaf_off = reinterpret_cast<const int64_t*>(w + l.off_leaf_off);
  a.leaf_len = reinterpret_cast<const int32_t*>(w + l.off_leaf_len);
  a.nleaves = int32_t(l.nleaves);
  a.nlevels = int32_t(l.nlevels);
  a.node_l = reinterpret_cast<const int32_t*>(w + l.off_node_l);
  a.node_r = reinterpret_cast<const int32_t*>(w + l.off_node_r);
  a.node_out = reinterpret_cast<const int32_t*>(w + l.off_node_out);
  a.lvl = reinterpret_cast<const int32_t*>(w + l.off_lvl);
  a.root = plan.root;
  a.val = reinterpret_cast<double*>(w + l.off_val);
  a.ctl = reinterpret_cast<uint32_t*>(w + l.off_ctl);
  a.steps_out = reinterpret_cast<int64_t*>(w + l.off_steps);
  int32_t status = NPBGB_OK;
  cudaError_t e = cudaSuccess;
  // Pageable sources: these copies have read the vectors when they return.
  auto put = [&](int64_t off, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes > 0)
      e = cudaMemcpyAsync(w + off, src, bytes, cudaMemcpyHostToDevice, st);
  };
  put(l.off_leaf_off, plan.leaf_off.data(), plan.leaf_off.size() * 8);
  put(l.off_leaf_len, plan.leaf_len.data(), plan.leaf_len.size() * 4);
  put(l.off_node_l, plan.node_l.data(), plan.node_l.size() * 4);
  put(l.off_node_r, plan.node_r.data(), plan.node_r.size() * 4);
  put(l.off_node_out, plan.node_out.data(), plan.node_out.size() * 4);
  put(l.off_lvl, plan.lvl.data(), plan.lvl.size() * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(w + l.off_done, 0, size_t(l.off_leaf_off - l.off_done), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w + l.off_ctl, 0, size_t(2 * kAlign), st);
  if (e == cudaSuccess) {
    if (ny < 3) {
      channel_small<<<1, kCThreads, 0, st>>>(a);
      e = counted(cudaGetLastError());
    } else {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3{unsigned(l.nb), 1, 1};
      cfg.blockDim = dim3{unsigned(kCThreads), 1, 1};
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      void* args[] = {&a};
      e = counted(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(cfd_bands<true>), args));
    }
  }
  if (e == cudaSuccess && steps != nullptr) {
    e = cudaMemcpyAsync(steps, a.steps_out, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e != cudaSuccess) status = cuda_status(e, "channel_flow");
  if (workspace == nullptr) cudaFreeAsync(ws, st);
  return status;
}
