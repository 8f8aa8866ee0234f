// qt_wsd.cu -- weighted simultaneous diagonalisation of the CDVR grids
// (LayerGrid with several matrices, src/DVR/TDDVR.cpp:72-88, around
// WeightedSimultaneousDiagonalization::calculate,
// src/Util/WeightedSimultaneousDiagonalization.cpp:5-378, and the Jacobi
// rotation helpers of src/Core/JacobiRotationFramework.cpp:4-164).
//
// One block of four warps per problem (one warp per FP64 unit of the SM).  The
// iteration accepts or rejects optimiser steps on
// comparisons of nearly equal numbers, so its result is a discontinuous
// function of the inputs; this file therefore fixes one operation order,
// which the CPU restatement follows bit for bit:
//  * compiled with -fmad=false: no multiply-add is fused; a complex product
//    is (ac - bd) + i(ad + bc), sums run left to right; a sum over the
//    matrices of a problem is the pairwise tree of the values padded with
//    zeros to a power of two, and the measure adds its per-matrix traces in
//    index order;
//  * |z| is sqrt(re^2 + im^2); real(x / w) is (xr wr + xi wi) / (wr^2 + wi^2);
//    the rotated diagonals of a candidate rotation use the Hermitian form
//    c^2 A_pp + 2c Re(s A_pq) + |s|^2 A_qq (c is real);
//  * the optimiser's 3x3 eigenvector (Matrix::rDiag) comes from the largest
//    root of the characteristic polynomial (Newton from the Gershgorin bound)
//    and the largest cross product of two rows of H - lambda.
// Work is spread over the threads item by item -- the rotated 2x2 diagonal
// blocks of every matrix at every candidate rotation (nine at once for the
// finite-difference derivatives), the levels of the tree sums, the elements
// of the matrix products of the off-diagonality measure, the rows and
// columns of every Givens rotation.  The scalar control flow is uniform
// (every thread holds the same values and runs it redundantly).  All
// loops are bounded (at most 25 sweeps, 30 optimiser iterations, 64 step
// halvings per search, 100 Newton steps).
#include <cuda_runtime.h>

#include "qt_internal.h"

namespace qt {
namespace {

__device__ __forceinline__ double2 cm(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 ca(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cs(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cc(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cabs_(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ double cdiv_re(double2 x, double2 w) {
  return (x.x * w.x + x.y * w.y) / (w.x * w.x + w.y * w.y);
}

struct Prob {
  int d, n;
  double2* xw;   // n weighted matrices (global)
  double2* xp;   // n plain (shifted) matrices (global)
  double2* w;    // weight (global)
  double2* T;    // transformation (global)
  double2* tmp;  // 3 d^2: X T, Y and Y Y of the off-diagonality measure (global)
  // shared memory
  double2* blk;  // (n + 1) x 4: (pp, pq, qp, qq) of every matrix and of w at the current pair
  double* sq;    // 2 x (2 x 10 x P): squared rotated diagonals per candidate, two tree buffers
  int P2;        // n padded to a power of two
  double* wd;    // 2 x 10: rotated diagonals of w per candidate
  double2* cand; // 2 x 10: candidate (c, s)
  double* red;   // 32 + d: xold (0, 1), measure (2), xold / w (4, 5), losses (8..17), traces (32..)
  __device__ double2* X(int k) const { return xw + (int64_t)k * d * d; }
  __device__ double2* Xp(int k) const { return xp + (int64_t)k * d * d; }
};

constexpr int kWsdThreads = 128;
__device__ __forceinline__ int lane_id() { return threadIdx.x; }
__device__ __forceinline__ void wsync() { __syncthreads(); }

// Matrix::rDiag of the optimiser's symmetric 3x3 matrix: eigenvector of the
// largest eigenvalue as u0 = v0/v2, u1 = v1/v2 and v0^2 + v1^2 for |v| = 1
__device__ void eig3_top(const double H[9], double* u0, double* u1, double* top2) {
  const double h00 = H[0], h01 = H[3], h02 = H[6], h11 = H[4], h12 = H[7], h22 = H[8];
  const double tr = h00 + h11 + h22;
  const double m = (h00 * h11 - h01 * h01) + (h00 * h22 - h02 * h02) + (h11 * h22 - h12 * h12);
  const double det = h00 * (h11 * h22 - h12 * h12) - h01 * (h01 * h22 - h12 * h02) + h02 * (h01 * h12 - h11 * h02);
  double lam = h00 + fabs(h01) + fabs(h02);
  const double r1 = h11 + fabs(h01) + fabs(h12);
  const double r2 = h22 + fabs(h02) + fabs(h12);
  if (r1 > lam) lam = r1;
  if (r2 > lam) lam = r2;
  for (int it = 0; it < 100; ++it) {
    const double p = ((-lam + tr) * lam - m) * lam + det;
    const double dp = (-3.0 * lam + 2.0 * tr) * lam - m;
    if (!(dp < 0.0)) break;
    const double nxt = lam - p / dp;
    if (!(nxt < lam)) break;
    lam = nxt;
  }
  const double m00 = h00 - lam, m11 = h11 - lam, m22 = h22 - lam;
  const double c01[3] = {h01 * h12 - h02 * m11, h02 * h01 - m00 * h12, m00 * m11 - h01 * h01};
  const double c02[3] = {h01 * m22 - h02 * h12, h02 * h02 - m00 * m22, m00 * h12 - h01 * h02};
  const double c12[3] = {m11 * m22 - h12 * h12, h12 * h02 - h01 * m22, h01 * h12 - m11 * h02};
  const double n01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
  const double n02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
  const double n12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
  double v0 = c01[0], v1 = c01[1], v2 = c01[2], nv = n01;
  if (n02 > nv) {
    v0 = c02[0];
    v1 = c02[1];
    v2 = c02[2];
    nv = n02;
  }
  if (n12 > nv) {
    v0 = c12[0];
    v1 = c12[1];
    v2 = c12[2];
  }
  *u0 = v0 / v2;
  *u1 = v1 / v2;
  const double q = v0 * v0 + v1 * v1;
  *top2 = q / (q + v2 * v2);
}

// rotatedDiagonals of a cached 2x2 block (pp, pq, qp, qq) of a Hermitian
// matrix for a real c: a0 = c^2 A_pp + 2c Re(s A_pq) + |s|^2 A_qq and
// a1 = c^2 A_qq - 2c Re(s A_pq) + |s|^2 A_pp
__device__ __forceinline__ void rotated_diagonals(const double2* b, double2 c, double2 s, double& a0, double& a1) {
  const double cc2 = c.x * c.x;
  const double ss2 = s.x * s.x + s.y * s.y;
  const double c2 = 2.0 * c.x;
  const double2 apq = b[1];
  const double t = s.x * apq.x - s.y * apq.y;
  const double ct = c2 * t;
  a0 = (cc2 * b[0].x + ct) + ss2 * b[3].x;
  a1 = (cc2 * b[3].x - ct) + ss2 * b[0].x;
}

// weightedJacobiLoc for `count` candidates at once (cand[0 .. 2 count)):
// red[8 + j] = diff of candidate j; red[4], red[5] hold xold / w of the pair
__device__ void loc_many(const Prob& P, int count) {
  const int n = P.n, tid = lane_id(), P2 = P.P2;
  double* buf = P.sq;                     // [comp][cand][P2], level 0
  double* alt = P.sq + 2 * 10 * (int64_t)P2;
  const int items = count * P2;
  for (int it = tid; it < count * (n + 1); it += kWsdThreads) {
    const int j = it / (n + 1), k = it % (n + 1);
    double r0, r1;
    rotated_diagonals(P.blk + 4 * k, P.cand[2 * j], P.cand[2 * j + 1], r0, r1);
    if (k < n) {
      buf[j * P2 + k] = r0 * r0;
      buf[10 * P2 + j * P2 + k] = r1 * r1;
    } else {
      P.wd[2 * j] = r0;
      P.wd[2 * j + 1] = r1;
    }
  }
  for (int it = tid; it < items; it += kWsdThreads) {  // zero padding
    const int j = it / P2, k = it % P2;
    if (k >= n) {
      buf[j * P2 + k] = 0.0;
      buf[10 * P2 + j * P2 + k] = 0.0;
    }
  }
  wsync();
  for (int size = P2; size > 1; size >>= 1) {  // pairwise tree, both components
    const int half = size >> 1;
    for (int it = tid; it < 2 * count * half; it += kWsdThreads) {
      const int comp = it / (count * half), rem = it % (count * half);
      const int j = rem / half, i = rem % half;
      const double* src = buf + comp * 10 * P2 + j * P2;
      alt[comp * 10 * P2 + j * P2 + i] = src[2 * i] + src[2 * i + 1];
    }
    wsync();
    double* t = buf;
    buf = alt;
    alt = t;
  }
  if (tid < count) {
    const int j = tid;
    const double xnew0 = buf[j * P2], xnew1 = buf[10 * P2 + j * P2];
    double diff = 0;
    diff += xnew0 / P.wd[2 * j] - P.red[4];
    diff += xnew1 / P.wd[2 * j + 1] - P.red[5];
    P.red[8 + j] = diff;
  }
  wsync();
}

// weightedJacobiDerivatives: the loss at the nine points of the central
// differences around s_in (as candidates 1..9, after `first` candidates the
// caller placed at 0 .. first-1); y[q] of point q = i + 3 j gets
// red[8 + first + q]
__device__ void set_samples(const Prob& P, double2 s_in, double delta, int first) {
  const int t = lane_id();
  if (t >= first && t < first + 9) {
    const int q = t - first;
    const int i = q % 3, j = q / 3;
    const double x0 = s_in.x + (double)(i - 1) * delta;
    const double x1 = s_in.y + (double)(j - 1) * delta;
    const double z = x0 * x0 + x1 * x1;
    P.cand[2 * t] = make_double2(sqrt(fabs(1 - z)), 0.0);
    P.cand[2 * t + 1] = make_double2(x0, x1);
  }
}
__device__ void grad_pre(const double y[9], double grad[2], double pre[4], double delta) {
  grad[0] = (y[2 + 3 * 1] - y[0 + 3 * 1]) / (2 * delta);
  grad[1] = (y[1 + 3 * 2] - y[1 + 3 * 0]) / (2 * delta);
  pre[0] = (y[2 + 3 * 1] + y[0 + 3 * 1] - 2 * y[1 + 3 * 1]) / (delta * delta);
  pre[3] = (y[1 + 3 * 2] + y[1 + 3 * 0] - 2 * y[1 + 3 * 1]) / (delta * delta);
  pre[2] = (y[2 + 3 * 2] + y[0 + 3 * 0] - y[2 + 3 * 0] - y[0 + 3 * 2]) / (4 * delta * delta);
  pre[1] = pre[2];
}

// calculateWeightedAngles: rational function optimisation of (c, s).  The
// loss of every new candidate is evaluated together with the nine samples of
// the central differences around it: if the candidate is accepted they are
// the next iteration's derivatives, if not the derivatives at the unchanged
// point are still valid -- the same numbers the reference recomputes.
__device__ void angles(const Prob& P, double2& c, double2& s) {
  int iter = 0;
  const int maxiter = 30;
  const double eps = 1E-3;
  double diff_rel = 2 * eps * eps;
  const double amin = 1E-12, amax = 1;
  double a = amax;
  const double delta = 1E-5;
  double snew[2] = {0, 0}, cnew[2] = {0, 0};
  c = make_double2(sqrt(1 - 2 * eps * eps), 0);
  s = make_double2(eps, -eps);
  // loss at the start point and the samples around it
  if (lane_id() == 0) {
    P.cand[0] = c;
    P.cand[1] = s;
  }
  set_samples(P, s, delta, 1);
  wsync();
  loc_many(P, 10);
  double loc_alt = P.red[8];
  double ycur[9], ynew[9];
  for (int q = 0; q < 9; ++q) ycur[q] = P.red[9 + q];
  wsync();
  double loc_new = 0;
  while (iter < maxiter && diff_rel > eps * eps && a > amin) {
    double pre[4], grad[2];
    grad_pre(ycur, grad, pre, delta);
    double diff = -1;
    int guard = 0;
    while (a > amin && diff < 0 && diff_rel > eps * eps && guard++ < 64) {
      double z = 1;
      double top2 = 0;
      int guard2 = 0;
      while (a > amin && z > 0.5 && guard2++ < 64) {
        double H[9];
        H[0] = pre[0] * a * a;
        H[1] = pre[1] * a * a;
        H[3] = pre[2] * a * a;
        H[4] = pre[3] * a * a;
        H[2] = grad[0] * a;
        H[6] = grad[0] * a;
        H[5] = grad[1] * a;
        H[7] = grad[1] * a;
        H[8] = 0;
        double u0, u1;
        eig3_top(H, &u0, &u1, &top2);
        const double ds0 = a * u0;
        const double ds1 = a * u1;
        snew[0] = s.x + ds0;
        snew[1] = s.y + ds1;
        const double zab = cabs_(make_double2(snew[0], snew[1]));
        z = zab * zab;
        if (z > 0.5) a /= 2;
      }
      cnew[0] = sqrt(fabs(1 - z));
      cnew[1] = 0;
      if (lane_id() == 0) {
        P.cand[0] = make_double2(cnew[0], cnew[1]);
        P.cand[1] = make_double2(snew[0], snew[1]);
      }
      set_samples(P, make_double2(snew[0], snew[1]), delta, 1);
      wsync();
      loc_many(P, 10);
      loc_new = P.red[8];
      for (int q = 0; q < 9; ++q) ynew[q] = P.red[9 + q];
      wsync();
      const double trafoabs = top2;
      const double sab = cabs_(s);
      const double sabs = sab * sab + eps * eps;
      diff_rel = trafoabs / sabs;
      diff = loc_new - loc_alt;
      if (diff < 0) {
        a /= 2;
      } else {
        if (a < amax) a *= 2;
      }
    }
    if (a > amin && diff > 0) {
      c = make_double2(cnew[0], cnew[1]);
      s = make_double2(snew[0], snew[1]);
      loc_alt = loc_new;
      for (int q = 0; q < 9; ++q) ycur[q] = ynew[q];
    }
    iter++;
  }
}

// givensRotation on m_count matrices at once (lanes over matrix x row)
__device__ void givens_all(const Prob& P, double2* base, int m_count, int64_t stride, double2 c, double2 s,
                           int i, int j) {
  const int d = P.d;
  const int lane = lane_id();
  const int64_t tot = (int64_t)m_count * d;
  for (int64_t e = lane; e < tot; e += kWsdThreads) {  // columns i, j
    double2* B = base + (e / d) * stride;
    const int r = (int)(e % d);
    const double2 bri = B[r + (int64_t)d * i], brj = B[r + (int64_t)d * j];
    B[r + (int64_t)d * i] = ca(cm(c, bri), cm(s, brj));
    B[r + (int64_t)d * j] = cs(cm(c, brj), cm(cc(s), bri));
  }
  wsync();
  for (int64_t e = lane; e < tot; e += kWsdThreads) {  // rows i, j
    double2* B = base + (e / d) * stride;
    const int r = (int)(e % d);
    const double2 c0 = B[i + (int64_t)d * r], c1 = B[j + (int64_t)d * r];
    B[i + (int64_t)d * r] = ca(cm(c, c0), cm(cc(s), c1));
    B[j + (int64_t)d * r] = cs(cm(c, c1), cm(s, c0));
  }
  wsync();
}

__device__ void rotations(const Prob& P) {
  const int d = P.d, n = P.n;
  const int lane = lane_id();
  for (int i = 0; i < d - 1; ++i)
    for (int j = i + 1; j < d; ++j) {
      for (int k = lane; k <= n; k += kWsdThreads) {  // cache the (i, j) blocks
        const double2* A = k < n ? P.X(k) : P.w;
        P.blk[4 * k + 0] = A[i + (int64_t)d * i];
        P.blk[4 * k + 1] = A[i + (int64_t)d * j];
        P.blk[4 * k + 2] = A[j + (int64_t)d * i];
        P.blk[4 * k + 3] = A[j + (int64_t)d * j];
      }
      wsync();
      // sums of the current squared diagonals (tree order) and xold / w
      for (int k = lane; k < P.P2; k += kWsdThreads) {
        const double x0 = k < n ? P.blk[4 * k].x : 0.0, x1 = k < n ? P.blk[4 * k + 3].x : 0.0;
        P.sq[k] = k < n ? x0 * x0 : 0.0;
        P.sq[10 * P.P2 + k] = k < n ? x1 * x1 : 0.0;
      }
      wsync();
      {
        double* buf = P.sq;
        double* alt = P.sq + 2 * 10 * (int64_t)P.P2;
        for (int size = P.P2; size > 1; size >>= 1) {
          const int half = size >> 1;
          for (int it = lane; it < 2 * half; it += kWsdThreads) {
            const int comp = it / half, q = it % half;
            alt[comp * 10 * P.P2 + q] = buf[comp * 10 * P.P2 + 2 * q] + buf[comp * 10 * P.P2 + 2 * q + 1];
          }
          wsync();
          double* t = buf;
          buf = alt;
          alt = t;
        }
        if (lane == 0) {
          P.red[0] = buf[0];
          P.red[1] = buf[10 * P.P2];
          P.red[4] = buf[0] / P.blk[4 * n + 0].x;
          P.red[5] = buf[10 * P.P2] / P.blk[4 * n + 3].x;
        }
        wsync();
      }
      double2 c, s;
      angles(P, c, s);
      givens_all(P, P.xw, n, (int64_t)d * d, c, s, i, j);
      givens_all(P, P.w, 1, 0, c, s, i, j);
      for (int r = lane; r < d; r += kWsdThreads) {  // givensTrafoRotation
        const double2 ti = P.T[r + (int64_t)d * i], tj = P.T[r + (int64_t)d * j];
        P.T[r + (int64_t)d * i] = ca(cm(c, ti), cm(s, tj));
        P.T[r + (int64_t)d * j] = cs(cm(c, tj), cm(cc(s), ti));
      }
      wsync();
    }
}

// measureWeightedOffDiagonality: sum_k Re tr(W (D_k - T^H X_k T)^2), matrix by
// matrix; the elements of each product in parallel, each an ordered sum
__device__ double offdiag(const Prob& P) {
  const int d = P.d, lane = lane_id();
  const int64_t dd = (int64_t)d * d;
  double2* M = P.tmp;
  double2* Y = M + dd;
  double2* Z = Y + dd;
  double total = 0;
  for (int k = 0; k < P.n; ++k) {
    const double2* X = P.Xp(k);
    const double2* Xw = P.X(k);
    for (int64_t e = lane; e < dd; e += kWsdThreads) {
      const int i = (int)(e % d), j = (int)(e / d);
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(X[i + (int64_t)d * l], P.T[l + (int64_t)d * j]));
      M[e] = acc;
    }
    wsync();
    for (int64_t e = lane; e < dd; e += kWsdThreads) {
      const int i = (int)(e % d), j = (int)(e / d);
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(cc(P.T[l + (int64_t)d * i]), M[l + (int64_t)d * j]));
      double2 dg = make_double2(0, 0);
      if (i == j) dg = make_double2(cdiv_re(Xw[i + (int64_t)d * i], P.w[i + (int64_t)d * i]), 0);
      Y[e] = cs(dg, acc);
    }
    wsync();
    for (int64_t e = lane; e < dd; e += kWsdThreads) {
      const int i = (int)(e % d), j = (int)(e / d);
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(Y[i + (int64_t)d * l], Y[l + (int64_t)d * j]));
      Z[e] = acc;
    }
    wsync();
    for (int i = lane; i < d; i += kWsdThreads) {
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(P.w[i + (int64_t)d * l], Z[l + (int64_t)d * i]));
      P.red[32 + i] = acc.x;
    }
    wsync();
    if (lane == 0) {
      double tr = 0;
      for (int i = 0; i < d; ++i) tr += P.red[32 + i];
      total += tr;
    }
    wsync();
  }
  if (lane == 0) P.red[2] = total;
  wsync();
  const double v = P.red[2];
  wsync();
  return v;
}

__global__ void __launch_bounds__(kWsdThreads) k_wsd(const WSDTask* __restrict__ tasks, const WSDTerm* __restrict__ terms,
                                            int64_t first) {
  const WSDTask t = tasks[first + blockIdx.x];
  const int d = t.d, n = t.n;
  const int lane = threadIdx.x;
  const int64_t dd = (int64_t)d * d;
  extern __shared__ double2 wsd_smem[];
  Prob P;
  P.d = d;
  P.n = n;
  P.xw = t.scratch;
  P.xp = t.scratch + n * dd;
  P.w = t.scratch + 2 * n * dd;
  P.T = P.w + dd;
  P.tmp = P.T + dd;
  P.blk = wsd_smem;
  P.P2 = 1;
  while (P.P2 < n) P.P2 <<= 1;
  P.cand = P.blk + 4 * (n + 1);
  P.sq = reinterpret_cast<double*>(P.cand + 20);
  P.wd = P.sq + 4 * 10 * (int64_t)P.P2;
  P.red = P.wd + 20;
  // w = regularize(W, 1e-9), T = 1
  for (int64_t e = lane; e < dd; e += kWsdThreads) {
    double2 v = t.W[e];
    const int i = (int)(e % d), j = (int)(e / d);
    if (i == j) v.x += 1e-9 * exp(-cabs_(v) / 1e-9);
    P.w[e] = v;
    P.T[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  // plain matrices shifted by |tr X| (calculateShift / shift)
  for (int k = lane; k < n; k += kWsdThreads) {
    const double2* X = terms[t.first + k].X;
    double2* Xp = P.Xp(k);
    double2 tr = make_double2(0, 0);
    for (int i = 0; i < d; ++i) tr = ca(tr, X[i + (int64_t)d * i]);
    const double sh = cabs_(tr);
    for (int64_t e = 0; e < dd; ++e) Xp[e] = X[e];
    for (int i = 0; i < d; ++i) Xp[i + (int64_t)d * i].x -= sh;
    t.grid[(int64_t)k * d].y = sh;  // kept until the end (the grid's imaginary parts are zero)
  }
  wsync();
  // weightMatrices: (X w + w X) / 2
  for (int64_t e = lane; e < (int64_t)n * dd; e += kWsdThreads) {
    const int k = (int)(e / dd);
    const int i = (int)(e % dd % d), j = (int)(e % dd / d);
    const double2* x = P.Xp(k);
    double2 xw = make_double2(0, 0), wx = make_double2(0, 0);
    for (int l = 0; l < d; ++l) {
      xw = ca(xw, cm(x[i + (int64_t)d * l], P.w[l + (int64_t)d * j]));
      wx = ca(wx, cm(P.w[i + (int64_t)d * l], x[l + (int64_t)d * j]));
    }
    const double2 sum = ca(xw, wx);
    P.X(k)[i + (int64_t)d * j] = make_double2(0.5 * sum.x, 0.5 * sum.y);
  }
  wsync();
  double delta = offdiag(P);
  wsync();
  int iter = 0;
  bool converged = false;
  const double eps = 1e-5;
  while (!converged && iter < 25) {
    rotations(P);
    const double delta_last = delta;
    delta = offdiag(P);
    wsync();
    const double change = fabs(delta_last - delta);
    if (delta < eps || change < eps) converged = true;
    iter++;
  }
  // grid = Re(Xw(i,i) / w(i,i)) + shift; trafo = T^dagger
  for (int k = lane; k < n; k += kWsdThreads) {
    const double sh = t.grid[(int64_t)k * d].y;
    for (int i = 0; i < d; ++i)
      t.grid[(int64_t)k * d + i] = make_double2(cdiv_re(P.X(k)[i + (int64_t)d * i], P.w[i + (int64_t)d * i]) + sh, 0.0);
  }
  for (int64_t e = lane; e < dd; e += kWsdThreads) {
    const int i = (int)(e % d), j = (int)(e / d);
    t.trafo[e] = cc(P.T[j + (int64_t)d * i]);
  }
}

}  // namespace

// shared memory of a problem with n matrices of order d (see Prob)
int64_t wsd_smem_bytes(int n, int d) {
  int64_t p2 = 1;
  while (p2 < n) p2 <<= 1;
  return 16 * (4 * (int64_t)(n + 1) + 20) + 8 * (40 * p2 + 20 + 32 + d) + 64;
}

cudaError_t launch_wsd(const WSDTask* tasks, const WSDTerm* terms, int64_t first, int64_t n, int max_n,
                       int max_d, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t sm = wsd_smem_bytes(max_n, max_d);
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_wsd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_wsd<<<(unsigned)n, kWsdThreads, sm, s>>>(tasks, terms, first);
  return cudaGetLastError();
}

}  // namespace qt
