// eval_kernels.cuh — FP64 reductions for termination checks and restart scoring.
//
// The reference computes each statistic with its own broadcast kernel and a host
// round trip per norm, and allocates temporaries for concatenated norms
// (src/iteration_stats_utils_gpu.jl:23-372, src/saddle_point_gpu.jl:250-278). Here every
// statistic of one evaluation is accumulated in FP64 in a single pass per side (n columns,
// m rows) over fixed segments (batch_kernels.cuh), into per-segment partials that one
// finalize CTA per instance reduces in a fixed order; the host reads back one small array.
// Comparisons, maxima and sign tests run on the integer pipe (bit patterns), so the FP64
// pipe only does the arithmetic itself.
#pragma once

#include "common.cuh"

namespace gpdhg {

// The evaluation's max-quantities are all magnitudes (|v|, or a positive part): their
// NaN-propagating maximum is the integer maximum of the bit patterns with the sign cleared
// (+0 < ... < +inf < NaN), done on the integer pipe instead of GB300's narrow FP64 pipe.
__device__ __forceinline__ double nan_max(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffULL;
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b) & 0x7fffffffffffffffULL;
  return __longlong_as_double((long long)(ua > ub ? ua : ub));
}

__device__ __forceinline__ bool bits_nan(long long b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }

// Julia's max(v, 0) and min(v, 0) (NaN-propagating), by sign and NaN tests on the bits.
__device__ __forceinline__ double pos_part(double v) {
  const long long b = __double_as_longlong(v);
  return (b > 0 || bits_nan(b)) ? v : 0.0;  // +x (x != 0) and NaN kept; -x, -0, +0 -> +0
}
__device__ __forceinline__ double neg_part(double v) {
  const long long b = __double_as_longlong(v);
  return ((b < 0 && (b & 0x7fffffffffffffffLL) != 0) || bits_nan(b)) ? v : 0.0;
}
__device__ __forceinline__ bool bits_finite(double v) {
  return (__double_as_longlong(v) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

__device__ __forceinline__ double warp_nan_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double block_nan_max(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_nan_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_nan_max(r);
  }
  return r;
}

// Q per-thread accumulators reduced over the CTA in a fixed order. The values go through
// shared memory (sh: kRedChunk x kBlock doubles, kRedChunk quantities at a time); warp w
// reduces quantities w, w + 8, ... of a chunk: lane l combines entry l of every warp in warp
// order, then a shuffle tree finishes (12 warp-wide FP64 adds per summed quantity, where a
// shuffle tree in every warp takes 40; maxima run on the integer pipe). Bit q of MAXMASK
// selects max (else sum). A quantity's order does not depend on Q. The result for q is
// valid in thread q (res: Q doubles).
constexpr int kRedChunk = 16;
template <int Q, unsigned MAXMASK>
__device__ __forceinline__ double block_reduce_q(const double* acc, double* sh, double* res) {
  static_assert(Q <= 32, "MAXMASK holds 32 quantities");
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
#pragma unroll
  for (int q0 = 0; q0 < Q; q0 += kRedChunk) {
    if (q0 > 0) __syncthreads();  // the previous chunk's readers are done with sh
#pragma unroll
    for (int q = q0; q < Q && q < q0 + kRedChunk; ++q) sh[(q - q0) * kBlock + t] = acc[q];
    __syncthreads();
    for (int q = q0 + wid; q < Q && q < q0 + kRedChunk; q += kBlock / 32) {
      const bool is_max = (MAXMASK >> q) & 1u;
      const double* c = sh + (q - q0) * kBlock + lane;
      double v = c[0];
#pragma unroll
      for (int w = 1; w < kBlock / 32; ++w) v = is_max ? nan_max(v, c[w * 32]) : v + c[w * 32];
      v = is_max ? warp_nan_max(v) : warp_sum(v);
      if (lane == 0) res[q] = v;
    }
  }
  __syncthreads();
  return t < Q ? res[t] : 0.0;
}

// a / b from r = 1 / b (correctly rounded, computed once per divisor): the product a r
// corrected once with the exact residual a - q b (Markstein's correction step, P. Markstein,
// "IA-64 and Elementary Functions", 2000), three FP64 operations instead of a division. It
// returns the correctly rounded quotient for normal operands (a CPU check of 5e7 random
// pairs over a 2^200 range found no difference from a / b); zero and non-finite products
// are returned as they are, which keeps the quotient's sign and infinities.
__device__ __forceinline__ double div_rcp(double a, double b, double r) {
  const double q = a * r;
  const long long bq = __double_as_longlong(q) & 0x7fffffffffffffffLL;
  if (bq == 0 || bq >= 0x7ff0000000000000LL) return q;
  const double e = fma(-q, b, a);
  return fma(e, r, q);
}

__device__ __forceinline__ double reduced_cost(double g, bool fl, bool fu) {
  // src/iteration_stats_utils_gpu.jl:168: max(g,0)*isfinite(l) + min(g,0)*isfinite(u). At
  // most one term is nonzero unless g is NaN (then the sum is NaN), so the sum is a select.
  const double p = fl ? pos_part(g) : 0.0;
  const double q = fu ? neg_part(g) : 0.0;
  const long long bp = __double_as_longlong(p);
  return (bp != 0) ? p : q;  // p is +0 or a positive value / NaN
}
__device__ __forceinline__ double rc_contribution(double rc, double l, double u) {
  // src/iteration_stats_utils_gpu.jl:120-126 (rc > 0, rc < 0 tested on the bits)
  const long long b = __double_as_longlong(rc);
  if (bits_nan(b) || (b & 0x7fffffffffffffffLL) == 0) return 0.0;  // neither rc > 0 nor rc < 0
  return b > 0 ? l * rc : u * rc;
}

// Unscaled primal-side statistics of the averaged iterate (original problem).
enum EvalNQ {
  kN_LuSq = 0, kN_LuMax, kN_Cx, kN_XMax, kN_XSq, kN_RcvSq, kN_RcvMax, kN_Contrib,
  kN_RayLuMax, kN_RayRcvMax, kN_RayContrib, kN_RayRcMax, kEvalNQ
};
constexpr unsigned kEvalNMax = (1u << kN_LuMax) | (1u << kN_XMax) | (1u << kN_RcvMax) | (1u << kN_RayLuMax) |
                               (1u << kN_RayRcvMax) | (1u << kN_RayRcMax);

template <class T>
struct EvalN {
  const T* ax;
  const T* agrad;
  const double* var;   // variable_rescaling (D)
  const double* rvar;  // 1 / D
  const double* ol;
  const double* ou;
  const double* oc;
  __device__ __forceinline__ void operator()(long long j, double* a) const { stats(j, ax[j], agrad[j], a); }
  // the statistics of element j of the scaled point (axv, agv)
  __device__ __forceinline__ void stats(long long j, T axv, T agv, double* a) const {
    const double x = div_rcp((double)axv, var[j], rvar[j]);   // :470-471
    const double g = (double)agv * var[j];         // :472-473
    const double l = ol[j], u = ou[j], c = oc[j];
    const bool fl = bits_finite(l), fu = bits_finite(u);
    const double lv = pos_part(l - x), uv = pos_part(x - u);
    a[kN_LuSq] += lv * lv + uv * uv;
    a[kN_LuMax] = nan_max(a[kN_LuMax], nan_max(fabs(lv), fabs(uv)));
    a[kN_Cx] += c * x;
    a[kN_XMax] = nan_max(a[kN_XMax], fabs(x));
    a[kN_XSq] += x * x;
    const double rc = reduced_cost(g, fl, fu);
    const double rcv = g - rc;
    a[kN_RcvSq] += rcv * rcv;
    a[kN_RcvMax] = nan_max(a[kN_RcvMax], fabs(rcv));
    a[kN_Contrib] += rc_contribution(rc, l, u);
    // primal ray, before division by ||x||_inf: bounds 0 where finite (:335-336)
    const double lr = fl ? pos_part(-x) : 0.0, ur = fu ? pos_part(x) : 0.0;
    a[kN_RayLuMax] = nan_max(a[kN_RayLuMax], nan_max(lr, ur));
    // dual ray: objective set to zero, gradient - c (:346-354)
    const double gr = g - c;
    const double rcr = reduced_cost(gr, fl, fu);
    a[kN_RayRcvMax] = nan_max(a[kN_RayRcvMax], fabs(gr - rcr));
    a[kN_RayContrib] += rc_contribution(rcr, l, u);
    a[kN_RayRcMax] = nan_max(a[kN_RayRcMax], fabs(rcr));
  }
};

enum EvalMQ { kM_CvSq = 0, kM_CvMax, kM_DrSq, kM_DrMax, kM_By, kM_YMax, kM_YSq, kM_RayCvMax, kEvalMQ };
constexpr unsigned kEvalMMax = (1u << kM_CvMax) | (1u << kM_DrMax) | (1u << kM_YMax) | (1u << kM_RayCvMax);

template <class T>
struct EvalM {
  const T* ay;
  const T* akx;
  const double* con;   // constraint_rescaling (E)
  const double* rcon;  // 1 / E
  const double* ob;
  int neq;
  const uint8_t* ineq_flag;  // per-row '>=' flag (packed batches); NULL: rows >= neq
  __device__ __forceinline__ void operator()(long long i, double* a) const { stats(i, ay[i], akx[i], a); }
  __device__ __forceinline__ void stats(long long i, T ayv, T akv, double* a) const {
    const double y = div_rcp((double)ayv, con[i], rcon[i]);   // :474-475
    const double kx = (double)akv * con[i];        // :476-477
    const double b = ob[i];
    const bool ineq = ineq_flag ? ineq_flag[i] != 0 : i >= neq;
    double cv = b - kx;                            // :26-45
    if (ineq) cv = pos_part(cv);
    a[kM_CvSq] += cv * cv;
    a[kM_CvMax] = nan_max(a[kM_CvMax], fabs(cv));
    if (ineq) {
      const double dr = pos_part(-y);             // :198-211
      a[kM_DrSq] += dr * dr;
      a[kM_DrMax] = nan_max(a[kM_DrMax], dr);
    }
    a[kM_By] += b * y;
    a[kM_YMax] = nan_max(a[kM_YMax], fabs(y));
    a[kM_YSq] += y * y;
    double cvr = -kx;                              // ray: right-hand side 0 (:338)
    if (ineq) cvr = pos_part(cvr);
    a[kM_RayCvMax] = nan_max(a[kM_RayCvMax], fabs(cvr));
  }
};

// Scaled weighted-KKT ingredients (src/saddle_point_gpu.jl:250-278) of three points:
// 0 = current, 1 = average, 2 = last restart; plus ||avg - last restart||^2.
constexpr int kKktNQ = 13;
constexpr int kKktMQ = 10;

template <class T>
struct KktN {
  const T* l;
  const T* u;
  const T* c;
  const T* x0; const T* x1; const T* x2;
  const T* g0; const T* g1; const T* g2;
  __device__ __forceinline__ void operator()(long long j, double* a) const {
    at(j, x0[j], g0[j], x1[j], g1[j], true, a);
  }
  // the three points' ingredients from the values of the current (xc, gc) and average
  // (xa, ga) points; the last restart point's (quantities 8-11) only when with_restart
  __device__ __forceinline__ void at(long long j, T xc, T gc, T xa, T ga, bool with_restart, double* a) const {
    const double l = (double)this->l[j], u = (double)this->u[j], c = (double)this->c[j];
    const bool fl = bits_finite(l), fu = bits_finite(u);
    value_point(0, xc, gc, l, u, c, fl, fu, a);
    value_point(1, xa, ga, l, u, c, fl, fu, a);
    const T xr = x2[j];
    if (with_restart) value_point(2, xr, g2[j], l, u, c, fl, fu, a);
    const double d = (double)xa - (double)xr;
    a[12] += d * d;
  }
  __device__ __forceinline__ void value_point(int p, T xv, T gv, double l, double u, double c, bool fl, bool fu,
                                              double* a) const {
    const double x = (double)xv, g = (double)gv;
    const double lv = pos_part(l - x), uv = pos_part(x - u);
    a[4 * p + 0] += lv * lv + uv * uv;
    a[4 * p + 1] += c * x;
    const double rc = reduced_cost(g, fl, fu);
    const double rcv = g - rc;
    a[4 * p + 2] += rcv * rcv;
    a[4 * p + 3] += rc_contribution(rc, l, u);
  }
};

template <class T>
struct KktM {
  const T* b;
  const T* y0; const T* y1; const T* y2;
  const T* k0; const T* k1; const T* k2;
  int neq;
  const uint8_t* ineq_flag;  // as in EvalM
  __device__ __forceinline__ void value_point(int p, T yv, T kv, double b, bool ineq, double* a) const {
    const double y = (double)yv, kx = (double)kv;
    double cv = b - kx;
    if (ineq) cv = pos_part(cv);
    a[3 * p + 0] += cv * cv;
    if (ineq) {
      const double dr = pos_part(-y);
      a[3 * p + 1] += dr * dr;
    }
    a[3 * p + 2] += b * y;
  }
  __device__ __forceinline__ void operator()(long long i, double* a) const { at(i, y0[i], k0[i], y1[i], k1[i], true, a); }
  __device__ __forceinline__ void at(long long i, T yc, T kc, T ya, T ka, bool with_restart, double* a) const {
    const double b = (double)this->b[i];
    const bool ineq = ineq_flag ? ineq_flag[i] != 0 : i >= neq;
    value_point(0, yc, kc, b, ineq, a);
    value_point(1, ya, ka, b, ineq, a);
    const T yr = y2[i];
    if (with_restart) value_point(2, yr, k2[i], b, ineq, a);
    const double d = (double)ya - (double)yr;
    a[9] += d * d;
  }
};

// One evaluation's column pass (optimize(), src/primal_dual_hybrid_gradient_gpu.jl:633-760):
// the average (compute_average!, src/saddle_point_gpu.jl:226-240, with the average's K'y
// given as aty = A' y-bar, computed after the row pass formed y-bar; or the current point when
// there is none, which takes the gradient buffer as it stood), its unscaled statistics
// (EvalN), buffer_primal_gradient = c - K'y (:742), and the KKT ingredients of the current,
// average and last-restart points (KktN). The last restart point's ingredients depend on
// that point alone, so the caller recomputes them (with_restart) only after it changed.
// Per element the arithmetic is that of the separate kernels, so the sums are the same.
template <class T>
struct EvalPassN {
  EvalN<T> en;   // its ax / agrad are not read: the average comes from sx and aty here
  KktN<T> kn;    // kn.x0 = x, kn.x2 = rx, kn.g2 = rgrad
  const T* sx;
  const T* aty;  // A' y-bar
  const T* kty;
  T* ax;         // the average, written
  T* agrad;
  T* grad;
  double wx, wy, rwx, rwy;
  int use_current;
  int with_restart;
  __device__ __forceinline__ void operator()(long long j, double* a) const {
    const T c = kn.c[j];
    const T gold = grad[j];
    const T xc = kn.x0[j];
    T xa, ga;
    if (use_current) {
      xa = xc;
      ga = gold;
    } else {
      xa = (T)div_rcp((double)sx[j], wx, rwx);
      ga = c - aty[j];
    }
    ax[j] = xa;
    agrad[j] = ga;
    const T gc = c - kty[j];
    grad[j] = gc;
    en.stats(j, xa, ga, a);
    kn.at(j, xc, gc, xa, ga, with_restart != 0, a + kEvalNQ);
  }
};

// The row pass of the same evaluation: average (or current) y and K x, EvalM, KktM.
template <class T>
struct EvalPassM {
  EvalM<T> em;   // its ay / akx are not read
  KktM<T> km;    // km.y0 / km.k0 = current y / K x, km.y2 / km.k2 = restart point
  const T* sy;
  const T* skx;
  T* ay;         // the average, written
  T* akx;
  double wx, wy, rwx, rwy;
  int use_current;
  int with_restart;
  __device__ __forceinline__ void operator()(long long i, double* a) const {
    const T yc = km.y0[i], kc = km.k0[i];
    T ya, ka;
    if (use_current) {
      ya = yc;
      ka = kc;
    } else {
      ya = (T)div_rcp((double)sy[i], wy, rwy);
      ka = (T)div_rcp((double)skx[i], wx, rwx);
    }
    ay[i] = ya;
    akx[i] = ka;
    em.stats(i, ya, ka, a);
    km.at(i, yc, kc, ya, ka, with_restart != 0, a + kEvalMQ);
  }
};

// ---- small vector kernels --------------------------------------------------------

template <class T>
__global__ void grad_kernel(int n, const T* c, const T* kty, T* grad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) grad[j] = c[j] - kty[j];
}

// restart to average, src/saddle_point_gpu.jl:579-583
template <class T>
__global__ void restart_n_kernel(int n, const T* ax, const T* agrad, const T* c, T* x, T* kty, T* grad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    x[j] = ax[j];
    kty[j] = c[j] - agrad[j];
    grad[j] = agrad[j];
  }
}

template <class S, class D>
__global__ void convert_kernel(long long len, const S* src, D* dst) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (D)src[i];
}

}  // namespace gpdhg
