// qt_wsd.cu -- weighted simultaneous diagonalisation of the CDVR grids
// (LayerGrid with several matrices, src/DVR/TDDVR.cpp:72-88, around
// WeightedSimultaneousDiagonalization::calculate,
// src/Util/WeightedSimultaneousDiagonalization.cpp:5-378, and the Jacobi
// rotation helpers of src/Core/JacobiRotationFramework.cpp:4-164).
//
// One warp per problem.  The iteration accepts or rejects optimiser steps on
// comparisons of nearly equal numbers, so its result is a discontinuous
// function of the inputs; this file therefore fixes one operation order,
// which the CPU restatement follows bit for bit:
//  * compiled with -fmad=false: no multiply-add is fused; a complex product
//    is (ac - bd) + i(ad + bc), sums run left to right;
//  * a sum over the matrices of a problem: lane t adds matrices t, t + 32,
//    ... in order, then the lanes are combined by the xor butterfly
//    (offsets 16, 8, 4, 2, 1), which leaves every lane with the same value;
//  * |z| is sqrt(re^2 + im^2); real(x / w) is (xr wr + xi wi) / (wr^2 + wi^2);
//  * the 3x3 symmetric eigenproblem of the optimiser (Matrix::rDiag) is
//    cyclic Jacobi; only ratios and squares of the eigenvector of the largest
//    eigenvalue enter, which do not depend on the solver's sign choice.
// The optimiser's control flow is uniform: every lane holds the same values
// and runs it redundantly.  All loops are bounded (at most 25 sweeps, 30
// optimiser iterations, 64 step halvings per search, 50 Jacobi sweeps).
#include <cuda_runtime.h>

#include "qt_internal.h"

namespace qt {
namespace {

constexpr unsigned kFull = 0xffffffffu;

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
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v = v + __shfl_xor_sync(kFull, v, o);
  return v;
}

struct Prob {
  int d, n;
  double2* xw;   // n weighted matrices
  double2* xp;   // n plain (shifted) matrices
  double2* w;    // weight
  double2* T;    // transformation
  double2* tmp;  // 2 d^2 per lane: X T and Y of the off-diagonality measure
  __device__ double2& at(double2* m, int i, int j) const { return m[i + (int64_t)d * j]; }
  __device__ double2* X(int k) const { return xw + (int64_t)k * d * d; }
  __device__ double2* Xp(int k) const { return xp + (int64_t)k * d * d; }
};

// Matrix::rDiag of a symmetric 3x3 matrix: eigenvector of the largest eigenvalue
__device__ void eig3_top(const double H[9], double v[3]) {
  double A[9], V[9];
  for (int i = 0; i < 9; ++i) {
    A[i] = H[i];
    V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  }
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = A[3] * A[3] + A[6] * A[6] + A[7] * A[7];
    if (off == 0.0) break;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const double apq = A[p + 3 * q];
      if (apq == 0.0) continue;
      const double theta = (A[q + 3 * q] - A[p + 3 * p]) / (2.0 * apq);
      double t;
      if (fabs(theta) > 1e150)
        t = 0.5 / theta;
      else
        t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
      for (int k = 0; k < 3; ++k) {
        const double akp = A[k + 3 * p], akq = A[k + 3 * q];
        A[k + 3 * p] = c * akp - s * akq;
        A[k + 3 * q] = s * akp + c * akq;
        const double vkp = V[k + 3 * p], vkq = V[k + 3 * q];
        V[k + 3 * p] = c * vkp - s * vkq;
        V[k + 3 * q] = s * vkp + c * vkq;
      }
      for (int k = 0; k < 3; ++k) {
        const double apk = A[p + 3 * k], aqk = A[q + 3 * k];
        A[p + 3 * k] = c * apk - s * aqk;
        A[q + 3 * k] = s * apk + c * aqk;
      }
      A[p + 3 * q] = 0.0;
      A[q + 3 * p] = 0.0;
    }
  }
  int top = 0;
  for (int k = 1; k < 3; ++k)
    if (A[k + 3 * k] > A[top + 3 * top]) top = k;
  for (int k = 0; k < 3; ++k) v[k] = V[k + 3 * top];
}

__device__ __forceinline__ void rotated_diagonals(const Prob& P, const double2* A, int p, int q, double2 c,
                                                  double2 s, double& a0, double& a1) {
  const int d = P.d;
  const double2 App = A[p + (int64_t)d * p], Apq = A[p + (int64_t)d * q];
  const double2 Aqp = A[q + (int64_t)d * p], Aqq = A[q + (int64_t)d * q];
  const double2 c00 = ca(cm(c, App), cm(s, Apq));
  const double2 c01 = cs(cm(c, Apq), cm(cc(s), App));
  const double2 c10 = ca(cm(c, Aqp), cm(s, Aqq));
  const double2 c11 = cs(cm(c, Aqq), cm(cc(s), Aqp));
  a0 = ca(cm(c, c00), cm(cc(s), c10)).x;
  a1 = cs(cm(c, c11), cm(s, c01)).x;
}

// weightedJacobiLoc
__device__ double loc(const Prob& P, int p, int q, double2 c, double2 s) {
  const int lane = threadIdx.x & 31;
  double w0, w1;
  rotated_diagonals(P, P.w, p, q, c, s, w0, w1);
  double o0 = 0, o1 = 0, n0 = 0, n1 = 0;
  for (int k = lane; k < P.n; k += 32) {
    const double2* X = P.X(k);
    const double x0 = X[p + (int64_t)P.d * p].x, x1 = X[q + (int64_t)P.d * q].x;
    o0 += x0 * x0;
    o1 += x1 * x1;
  }
  for (int k = lane; k < P.n; k += 32) {
    double r0, r1;
    rotated_diagonals(P, P.X(k), p, q, c, s, r0, r1);
    n0 += r0 * r0;
    n1 += r1 * r1;
  }
  const double xold0 = warp_sum(o0), xold1 = warp_sum(o1);
  const double xnew0 = warp_sum(n0), xnew1 = warp_sum(n1);
  double diff = 0;
  diff += xnew0 / w0 - xold0 / P.w[p + (int64_t)P.d * p].x;
  diff += xnew1 / w1 - xold1 / P.w[q + (int64_t)P.d * q].x;
  return diff;
}

// weightedJacobiDerivatives
__device__ void derivatives(const Prob& P, double grad[2], double pre[4], double2 s_in, int p, int q,
                            double delta) {
  const double s0 = s_in.x, s1 = s_in.y;
  double y[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double x0 = s0 + (double)(i - 1) * delta;
      const double x1 = s1 + (double)(j - 1) * delta;
      const double z = x0 * x0 + x1 * x1;
      const double2 cnow = make_double2(sqrt(fabs(1 - z)), 0.0);
      y[i + 3 * j] = loc(P, p, q, cnow, make_double2(x0, x1));
    }
  grad[0] = (y[2 + 3 * 1] - y[0 + 3 * 1]) / (2 * delta);
  grad[1] = (y[1 + 3 * 2] - y[1 + 3 * 0]) / (2 * delta);
  pre[0] = (y[2 + 3 * 1] + y[0 + 3 * 1] - 2 * y[1 + 3 * 1]) / (delta * delta);
  pre[3] = (y[1 + 3 * 2] + y[1 + 3 * 0] - 2 * y[1 + 3 * 1]) / (delta * delta);
  pre[2] = (y[2 + 3 * 2] + y[0 + 3 * 0] - y[2 + 3 * 0] - y[0 + 3 * 2]) / (4 * delta * delta);
  pre[1] = pre[2];
}

// calculateWeightedAngles: rational function optimisation of (c, s)
__device__ void angles(const Prob& P, double2& c, double2& s, int p, int q) {
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
  double loc_alt = loc(P, p, q, c, s);
  double loc_new = 0;
  while (iter < maxiter && diff_rel > eps * eps && a > amin) {
    double pre[4], grad[2];
    derivatives(P, grad, pre, s, p, q, delta);
    double diff = -1;
    int guard = 0;
    while (a > amin && diff < 0 && diff_rel > eps * eps && guard++ < 64) {
      double z = 1;
      double v[3] = {0, 0, 0};
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
        eig3_top(H, v);
        const double ds0 = a * v[0] / v[2];
        const double ds1 = a * v[1] / v[2];
        snew[0] = s.x + ds0;
        snew[1] = s.y + ds1;
        const double zab = cabs_(make_double2(snew[0], snew[1]));
        z = zab * zab;
        if (z > 0.5) a /= 2;
      }
      cnew[0] = sqrt(fabs(1 - z));
      cnew[1] = 0;
      loc_new = loc(P, p, q, make_double2(cnew[0], cnew[1]), make_double2(snew[0], snew[1]));
      const double trafoabs = v[0] * v[0] + v[1] * v[1];
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
    }
    iter++;
  }
}

// givensRotation on m_count matrices at once (lanes over matrix x row)
__device__ void givens_all(const Prob& P, double2* base, int m_count, int64_t stride, double2 c, double2 s,
                           int i, int j) {
  const int d = P.d;
  const int lane = threadIdx.x & 31;
  const int64_t tot = (int64_t)m_count * d;
  for (int64_t e = lane; e < tot; e += 32) {  // columns i, j
    double2* B = base + (e / d) * stride;
    const int r = (int)(e % d);
    const double2 bri = B[r + (int64_t)d * i], brj = B[r + (int64_t)d * j];
    B[r + (int64_t)d * i] = ca(cm(c, bri), cm(s, brj));
    B[r + (int64_t)d * j] = cs(cm(c, brj), cm(cc(s), bri));
  }
  __syncwarp();
  for (int64_t e = lane; e < tot; e += 32) {  // rows i, j
    double2* B = base + (e / d) * stride;
    const int r = (int)(e % d);
    const double2 c0 = B[i + (int64_t)d * r], c1 = B[j + (int64_t)d * r];
    B[i + (int64_t)d * r] = ca(cm(c, c0), cm(cc(s), c1));
    B[j + (int64_t)d * r] = cs(cm(c, c1), cm(s, c0));
  }
  __syncwarp();
}

__device__ void rotations(const Prob& P) {
  const int d = P.d;
  const int lane = threadIdx.x & 31;
  for (int i = 0; i < d - 1; ++i)
    for (int j = i + 1; j < d; ++j) {
      double2 c, s;
      angles(P, c, s, i, j);
      givens_all(P, P.xw, P.n, (int64_t)d * d, c, s, i, j);
      givens_all(P, P.w, 1, 0, c, s, i, j);
      for (int r = lane; r < d; r += 32) {  // givensTrafoRotation
        const double2 ti = P.T[r + (int64_t)d * i], tj = P.T[r + (int64_t)d * j];
        P.T[r + (int64_t)d * i] = ca(cm(c, ti), cm(s, tj));
        P.T[r + (int64_t)d * j] = cs(cm(c, tj), cm(cc(s), ti));
      }
      __syncwarp();
    }
}

// measureWeightedOffDiagonality: sum_k Re tr(W (D_k - T^H X_k T)^2)
__device__ double offdiag(const Prob& P) {
  const int d = P.d;
  const int lane = threadIdx.x & 31;
  double2* M = P.tmp + (int64_t)lane * 2 * d * d;
  double2* Y = M + (int64_t)d * d;
  double part = 0;
  for (int k = lane; k < P.n; k += 32) {
    const double2* X = P.Xp(k);
    const double2* Xw = P.X(k);
    for (int j = 0; j < d; ++j)
      for (int i = 0; i < d; ++i) {
        double2 acc = make_double2(0, 0);
        for (int l = 0; l < d; ++l) acc = ca(acc, cm(X[i + (int64_t)d * l], P.T[l + (int64_t)d * j]));
        M[i + (int64_t)d * j] = acc;
      }
    for (int j = 0; j < d; ++j)
      for (int i = 0; i < d; ++i) {
        double2 acc = make_double2(0, 0);
        for (int l = 0; l < d; ++l) acc = ca(acc, cm(cc(P.T[l + (int64_t)d * i]), M[l + (int64_t)d * j]));
        double2 dg = make_double2(0, 0);
        if (i == j) dg = make_double2(cdiv_re(Xw[i + (int64_t)d * i], P.w[i + (int64_t)d * i]), 0);
        Y[i + (int64_t)d * j] = cs(dg, acc);
      }
    double tr = 0;
    for (int i = 0; i < d; ++i) {
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) {
        double2 z = make_double2(0, 0);  // (Y Y)(l, i)
        for (int q = 0; q < d; ++q) z = ca(z, cm(Y[l + (int64_t)d * q], Y[q + (int64_t)d * i]));
        acc = ca(acc, cm(P.w[i + (int64_t)d * l], z));
      }
      tr += acc.x;
    }
    part += tr;
  }
  return warp_sum(part);
}

__global__ void __launch_bounds__(32) k_wsd(const WSDTask* __restrict__ tasks, const WSDTerm* __restrict__ terms,
                                            int64_t first) {
  const WSDTask t = tasks[first + blockIdx.x];
  const int d = t.d, n = t.n;
  const int lane = threadIdx.x;
  const int64_t dd = (int64_t)d * d;
  Prob P;
  P.d = d;
  P.n = n;
  P.xw = t.scratch;
  P.xp = t.scratch + n * dd;
  P.w = t.scratch + 2 * n * dd;
  P.T = P.w + dd;
  P.tmp = P.T + dd;
  // w = regularize(W, 1e-9), T = 1
  for (int64_t e = lane; e < dd; e += 32) {
    double2 v = t.W[e];
    const int i = (int)(e % d), j = (int)(e / d);
    if (i == j) v.x += 1e-9 * exp(-cabs_(v) / 1e-9);
    P.w[e] = v;
    P.T[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  // plain matrices shifted by |tr X| (calculateShift / shift)
  for (int k = lane; k < n; k += 32) {
    const double2* X = terms[t.first + k].X;
    double2* Xp = P.Xp(k);
    double2 tr = make_double2(0, 0);
    for (int i = 0; i < d; ++i) tr = ca(tr, X[i + (int64_t)d * i]);
    const double sh = cabs_(tr);
    for (int64_t e = 0; e < dd; ++e) Xp[e] = X[e];
    for (int i = 0; i < d; ++i) Xp[i + (int64_t)d * i].x -= sh;
    t.grid[(int64_t)k * d].y = sh;  // kept until the end (the grid's imaginary parts are zero)
  }
  __syncwarp();
  // weightMatrices: (X w + w X) / 2
  for (int64_t e = lane; e < (int64_t)n * dd; e += 32) {
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
  __syncwarp();
  double delta = offdiag(P);
  __syncwarp();
  int iter = 0;
  bool converged = false;
  const double eps = 1e-5;
  while (!converged && iter < 25) {
    rotations(P);
    const double delta_last = delta;
    delta = offdiag(P);
    __syncwarp();
    const double change = fabs(delta_last - delta);
    if (delta < eps || change < eps) converged = true;
    iter++;
  }
  // grid = Re(Xw(i,i) / w(i,i)) + shift; trafo = T^dagger
  for (int k = lane; k < n; k += 32) {
    const double sh = t.grid[(int64_t)k * d].y;
    for (int i = 0; i < d; ++i)
      t.grid[(int64_t)k * d + i] = make_double2(cdiv_re(P.X(k)[i + (int64_t)d * i], P.w[i + (int64_t)d * i]) + sh, 0.0);
  }
  for (int64_t e = lane; e < dd; e += 32) {
    const int i = (int)(e % d), j = (int)(e / d);
    t.trafo[e] = cc(P.T[j + (int64_t)d * i]);
  }
}

}  // namespace

cudaError_t launch_wsd(const WSDTask* tasks, const WSDTerm* terms, int64_t first, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_wsd<<<(unsigned)n, 32, 0, s>>>(tasks, terms, first);
  return cudaGetLastError();
}

}  // namespace qt
